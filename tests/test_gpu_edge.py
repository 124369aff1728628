"""Edge cases of the step through the C ABI: an empty batch, act=None (the
reference accepts it, brax/generalized/pipeline_test.py:75), batch sizes that
do not fill the last CTA, one non-finite env among finite ones, invalid
arguments, and the widest matrix tile (nv 48: 64-wide tiles)."""

import numpy as np
import pytest

from tests.parity_util import actions, load, rel_err, seeded_inputs

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _P():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import _native as N
  from brax_gb300 import pipeline
  return pipeline, N


def _t(x):
  return torch.as_tensor(np.asarray(x, np.float32), device='cuda')


def test_empty_batch_launches_nothing():
  P, N = _P()
  sys_ = load('quadruped')
  s = P.init(sys_, _t(np.zeros((0, sys_.q_size()))), _t(np.zeros((0, sys_.qd_size()))))
  assert N.lib().braxg_last_launch_count() == 0
  out = P.step(sys_, s, _t(np.zeros((0, sys_.act_size()))), n_frames=5)
  torch.cuda.synchronize()
  assert out.q.shape == (0, sys_.q_size()) and N.lib().braxg_last_launch_count() == 0


def test_act_none_is_no_actuation():
  P, _ = _P()
  sys_ = load('quadruped')  # motors only: zero actions give zero actuator force
  q, qd = seeded_inputs(sys_, 64, 51)
  s = P.init(sys_, _t(q), _t(qd))
  a = P.step(sys_, s, None, n_frames=5, inverse_mode=P.CHOLESKY)
  b = P.step(sys_, s, _t(np.zeros((64, sys_.act_size()))), n_frames=5, inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  torch.testing.assert_close(a.q, b.q, rtol=0, atol=0)
  torch.testing.assert_close(a.qd, b.qd, rtol=0, atol=0)


@pytest.mark.parametrize('n', [1, 17, 37])
def test_ragged_batch_sizes(n):
  P, _ = _P()
  from oracle.pipeline import Oracle
  sys_ = load('quadruped')
  q, qd = seeded_inputs(sys_, n, 52)
  rng = np.random.default_rng(53)
  act = actions(sys_, n, rng)
  o32 = Oracle(sys_, np.float32, exact_inverse=True)
  ref = o32.step(o32.init(q.astype(np.float32), qd.astype(np.float32)), act.astype(np.float32))
  s = P.init(sys_, _t(q), _t(qd))
  got = P.step(sys_, s, _t(act), inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  assert (got.status.cpu().numpy() == 0).all()
  for f in ('q', 'qd'):
    e = rel_err(getattr(got, f).cpu().numpy(), getattr(ref, f))
    assert e.max() <= 1e-4, (n, f, e.max())


def test_nonfinite_env_is_flagged_and_isolated():
  P, N = _P()
  sys_ = load('quadruped')
  n = 40
  q, qd = seeded_inputs(sys_, n, 54)
  s = P.init(sys_, _t(q), _t(qd))
  bad_qd = s.qd.clone()
  bad_qd[5, 3] = float('nan')
  s_bad = s.replace(qd=bad_qd)
  act = _t(actions(sys_, n, np.random.default_rng(55)))
  got = P.step(sys_, s_bad, act, n_frames=5, inverse_mode=P.CHOLESKY)
  ref = P.step(sys_, s, act, n_frames=5, inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  st = got.status.cpu().numpy()
  assert st[5] & N.ENV_NONFINITE
  others = np.arange(n) != 5
  assert (st[others] == 0).all()
  torch.testing.assert_close(got.q[others], ref.q[others], rtol=0, atol=0)


def test_invalid_arguments_raise():
  P, _ = _P()
  sys_ = load('quadruped')
  q, qd = seeded_inputs(sys_, 8, 56)
  s = P.init(sys_, _t(q), _t(qd))
  act = _t(np.zeros((8, sys_.act_size())))
  with pytest.raises(ValueError):
    P.step(sys_, s, act, n_frames=0)
  with pytest.raises(ValueError):
    P.step(sys_, s, act, threads_per_env=8)
  with pytest.raises(ValueError):
    P.step(sys_, s, act, inverse_mode=7)
  with pytest.raises(ValueError):
    P.step(sys_, s, act, envs_per_cta=100)
  with pytest.raises(ValueError):
    P.step(sys_, s, _t(np.zeros((8, sys_.act_size() + 1))))


def test_widest_tile_chain48():
  P, _ = _P()
  from brax_gb300 import workloads as W
  from oracle.pipeline import Oracle
  sys_ = W.chain(48)
  n = 16
  rng = np.random.default_rng(57)
  q, qd = W.reset(sys_, n, rng)
  q, qd = q.astype(np.float32), qd.astype(np.float32)
  o32 = Oracle(sys_, np.float32, exact_inverse=True)
  o64 = Oracle(sys_, np.float64, exact_inverse=True)
  r32 = o32.step(o32.init(q, qd), np.zeros((n, sys_.act_size()), np.float32))
  r64 = o64.step(o64.init(q.astype(np.float64), qd.astype(np.float64)), np.zeros((n, sys_.act_size())))
  s = P.init(sys_, _t(q), _t(qd))
  got = P.step(sys_, s, None, inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  assert P.model_for(sys_).launch_shape(P.CHOLESKY)[0] == 32
  assert (got.status.cpu().numpy() == 0).all()
  for f in ('q', 'qd'):
    g = getattr(got, f).cpu().numpy()
    e64 = rel_err(g, getattr(r64, f))
    eo = rel_err(getattr(r32, f), getattr(r64, f))
    print(f'chain48 {f}: vs fp64 p99 {np.quantile(e64, 0.99):.2e} | fp32 oracle vs fp64 p99 {np.quantile(eo, 0.99):.2e}')
    assert np.quantile(e64, 0.99) <= max(1e-5, 3 * np.quantile(eo, 0.99)), f


@pytest.mark.parametrize('relax', [1, 2, 3])
def test_relaxed_barriers_change_no_result(relax):
  P, _ = _P()
  sys_ = load('quadruped')
  n = 64
  q, qd = seeded_inputs(sys_, n, 58)
  act = _t(actions(sys_, n, np.random.default_rng(59)))
  s = P.init(sys_, _t(q), _t(qd))
  a = P.step(sys_, s, act, n_frames=5, inverse_mode=P.CHOLESKY)
  b = P.step(sys_, s, act, n_frames=5, inverse_mode=P.CHOLESKY, relax_barriers=relax)
  torch.cuda.synchronize()
  for f in ('q', 'qd', 'mass_mx_inv', 'x_pos'):
    torch.testing.assert_close(getattr(a, f), getattr(b, f), rtol=0, atol=0)


def test_default_shape_balances_waves():
  """The default envs per CTA: the fewest waves of one full CTA per SM, the
  envs spread evenly over every SM of each wave."""
  P, _ = _P()
  sys_ = load('quadruped')
  m = P.model_for(sys_)
  sms = torch.cuda.get_device_properties(0).multi_processor_count
  full = m.launch_shape(P.CHOLESKY)[1]  # the largest CTA
  for n in (1, sms, sms * full, sms * full + 1, 4096, 3 * sms * full - 5):
    waves = -(-n // (sms * full))
    expect = -(-n // (sms * waves))
    t, e, _ = m.launch_shape(P.CHOLESKY, n_env=n)
    assert (t, e) == (32, expect), (n, e, expect)
    assert -(-n // e) <= waves * sms
