"""The position-term cache a state carries (braxg_state.cache): a step that
reuses it gives the same result, bit for bit, as one that recomputes the
terms, and it is not reused where it no longer applies (changed q / qd, other
per-env parameters, another inverse mode or team width, a non-finite env)."""

import numpy as np
import pytest

from tests.parity_util import actions, load, seeded_inputs

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

FIELDS = ('q', 'qd', 'x_pos', 'x_rot', 'xd_ang', 'xd_vel', 'mass_mx_inv', 'qf_smooth', 'qf_constraint', 'qdd',
          'status')


def _P():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline
  return pipeline


def _t(x):
  return torch.as_tensor(np.asarray(x, np.float32), device='cuda')


def _same(a, b, fields=FIELDS):
  for f in fields:
    torch.testing.assert_close(getattr(a, f), getattr(b, f), rtol=0, atol=0, equal_nan=True, msg=f)


@pytest.mark.parametrize('mode', ['cholesky', 'newton_schulz'])
@pytest.mark.parametrize('name', ['quadruped', 'humanoid_like'])
def test_cached_steps_equal_uncached(name, mode):
  P = _P()
  sys_ = load(name)
  inv = P.CHOLESKY if mode == 'cholesky' else P.NEWTON_SCHULZ
  n = 48
  q, qd = seeded_inputs(sys_, n, 91)
  rng = np.random.default_rng(92)
  c = P.init(sys_, _t(q), _t(qd))
  u = P.init(sys_, _t(q), _t(qd), cache=False)
  assert c.cache is not None and u.cache is None
  _same(c, u)
  for _ in range(4):
    act = _t(actions(sys_, n, rng))
    c = P.step(sys_, c, act, n_frames=5, inverse_mode=inv)
    u = P.step(sys_, u, act, n_frames=5, inverse_mode=inv)
    assert c.cache is not None and u.cache is None
    torch.cuda.synchronize()
    _same(c, u)


def test_full_outputs_from_cache():
  P = _P()
  sys_ = load('quadruped')
  n = 32
  q, qd = seeded_inputs(sys_, n, 93)
  act = _t(actions(sys_, n, np.random.default_rng(94)))
  c = P.step(sys_, P.init(sys_, _t(q), _t(qd)), act, n_frames=5, inverse_mode=P.CHOLESKY)
  u = P.step(sys_, P.init(sys_, _t(q), _t(qd), cache=False), act, n_frames=5, inverse_mode=P.CHOLESKY)
  c2 = P.step(sys_, c, act, n_frames=2, inverse_mode=P.CHOLESKY, full=True)
  u2 = P.step(sys_, u, act, n_frames=2, inverse_mode=P.CHOLESKY, full=True)
  torch.cuda.synchronize()
  _same(c2, u2, FIELDS + ('root_com', 'cinr_pos', 'cinr_i', 'cd_packed', 'cdof_packed', 'cdofd_packed', 'mass_mx', 'con_jac',
                          'con_diag', 'con_aref'))


def test_changed_state_is_recomputed():
  """Envs whose q or qd was edited after the cache was written recompute."""
  P = _P()
  sys_ = load('quadruped')
  n = 40
  q, qd = seeded_inputs(sys_, n, 95)
  act = _t(actions(sys_, n, np.random.default_rng(96)))
  s = P.step(sys_, P.init(sys_, _t(q), _t(qd)), act, n_frames=5, inverse_mode=P.CHOLESKY)
  q2, qd2 = s.q.clone(), s.qd.clone()
  q2[3, 2] += 0.05
  qd2[7, 0] = -0.25
  q2[11, 4] = torch.nextafter(q2[11, 4], torch.tensor(2.0, device='cuda'))  # one ulp
  edited = s.replace(q=q2, qd=qd2)
  got = P.step(sys_, edited, act, n_frames=5, inverse_mode=P.CHOLESKY)
  ref = P.step(sys_, edited.replace(cache=None), act, n_frames=5, inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  _same(got, ref)


def test_changed_parameters_are_recomputed():
  P = _P()
  sys_ = load('quadruped')
  n = 32
  q, qd = seeded_inputs(sys_, n, 97)
  act = _t(actions(sys_, n, np.random.default_rng(98)))
  s = P.step(sys_, P.init(sys_, _t(q), _t(qd)), act, n_frames=5, inverse_mode=P.CHOLESKY)
  gen = torch.Generator(device='cuda').manual_seed(99)
  dr = P.randomize(sys_, n, gen, friction_range=(0.5, 1.5), gain_scale_range=(0.7, 1.3))
  got = P.step(sys_, s, act, n_frames=5, inverse_mode=P.CHOLESKY, randomization=dr)
  ref = P.step(sys_, s.replace(cache=None), act, n_frames=5, inverse_mode=P.CHOLESKY, randomization=dr)
  torch.cuda.synchronize()
  _same(got, ref)


def test_other_mode_or_width_is_recomputed():
  """A cache from a Newton-Schulz step is not an exact inverse; one from a
  16-lane team is not what a 32-lane team computes."""
  P = _P()
  sys_ = load('quadruped')
  n = 32
  q, qd = seeded_inputs(sys_, n, 100)
  act = _t(actions(sys_, n, np.random.default_rng(101)))
  s0 = P.init(sys_, _t(q), _t(qd))
  ns = P.step(sys_, s0, act, n_frames=5, inverse_mode=P.NEWTON_SCHULZ)
  got = P.step(sys_, ns, act, n_frames=5, inverse_mode=P.CHOLESKY)
  ref = P.step(sys_, ns.replace(cache=None), act, n_frames=5, inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  _same(got, ref)
  t16 = P.step(sys_, s0, act, n_frames=5, inverse_mode=P.CHOLESKY, threads_per_env=16)
  got = P.step(sys_, t16, act, n_frames=5, inverse_mode=P.CHOLESKY, threads_per_env=32)
  ref = P.step(sys_, t16.replace(cache=None), act, n_frames=5, inverse_mode=P.CHOLESKY, threads_per_env=32)
  torch.cuda.synchronize()
  _same(got, ref)


def test_nonfinite_env_does_not_cache():
  P = _P()
  from brax_gb300 import _native as N
  sys_ = load('quadruped')
  n = 24
  q, qd = seeded_inputs(sys_, n, 102)
  act = _t(actions(sys_, n, np.random.default_rng(103)))
  s = P.init(sys_, _t(q), _t(qd))
  bad = s.qd.clone()
  bad[2, 1] = float('nan')
  a = P.step(sys_, s.replace(qd=bad), act, n_frames=5, inverse_mode=P.CHOLESKY)
  b = P.step(sys_, a, act, n_frames=5, inverse_mode=P.CHOLESKY)
  b_ref = P.step(sys_, a.replace(cache=None), act, n_frames=5, inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  assert a.status[2].item() & N.ENV_NONFINITE
  _same(b, b_ref)


def test_env_rollout_with_cache():
  P = _P()
  from brax_gb300 import envs
  sys_ = load('quadruped')
  n = 64
  env = envs.Locomotion(sys_, episode_length=6)
  gen = torch.Generator(device='cuda').manual_seed(104)
  st = env.reset(n, generator=gen)
  st_u = envs.State(st.pipeline_state.replace(cache=None), st.obs, st.reward, st.done, st.metrics, st.info)
  for k in range(4):
    a = torch.rand(3, n, sys_.act_size(), device='cuda', generator=gen) * 2 - 1
    st, r, d = env.rollout(st, a)
    st_u, r_u, d_u = env.rollout(st_u, a)
    torch.cuda.synchronize()
    assert st.pipeline_state.cache is not None and st_u.pipeline_state.cache is None
    torch.testing.assert_close(r, r_u, rtol=0, atol=0)
    torch.testing.assert_close(d, d_u, rtol=0, atol=0)
    torch.testing.assert_close(st.obs, st_u.obs, rtol=0, atol=0)
    _same(st.pipeline_state, st_u.pipeline_state)


def test_misaligned_cache_raises():
  P = _P()
  sys_ = load('quadruped')
  m = P.model_for(sys_)
  n = 4
  q, qd = seeded_inputs(sys_, n, 105)
  s = P.init(sys_, _t(q), _t(qd))
  buf = torch.empty(n * m.cache_words + 4, dtype=torch.float32, device='cuda')
  with pytest.raises(ValueError):
    P.step(sys_, s.replace(cache=buf[1:1 + n * m.cache_words].view(n, m.cache_words)), None)


def test_cache_skips_the_launch_start_position_stage():
  """With every env's cache valid, the per-stage cycle counters show the
  launch-start position stage gone: n_frames position stages per launch
  instead of n_frames + 1."""
  P = _P()
  sys_ = load('quadruped')
  n = 256
  q, qd = seeded_inputs(sys_, n, 106)
  act = _t(actions(sys_, n, np.random.default_rng(107)))
  s = P.step(sys_, P.init(sys_, _t(q), _t(qd)), act, n_frames=2, inverse_mode=P.CHOLESKY)
  fk = []
  for st in (s, s.replace(cache=None)):
    buf = P.profile_buffer()
    P.step(sys_, st, act, n_frames=2, inverse_mode=P.CHOLESKY, profile=buf)
    torch.cuda.synchronize()
    fk.append(P.profile_report(buf)['fk'])
  # 2 forward-kinematics passes with the cache, 3 without
  assert fk[0] < 0.85 * fk[1], fk


def test_cache_with_overflow_rows_and_implicit_solve():
  """Lying humanoid-like models (most envs with more than 32 active rows:
  the Jacobian rows beyond 32 live at the end of scratch and the cache copies
  them): cached steps equal uncached ones bit for bit."""
  P = _P()
  sys_ = load('humanoid_like')
  n = 48
  rng = np.random.default_rng(108)
  q = sys_.init_q[None] + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))
  qd = 0.1 * rng.normal(size=(n, sys_.qd_size()))
  q[:, 3:7] = [np.cos(np.pi / 4), np.sin(np.pi / 4), 0.0, 0.0]
  q[:, 2] = rng.uniform(0.05, 0.2, n)
  act = _t(np.clip(rng.normal(0.0, 0.3, (n, sys_.act_size())), -1, 1))
  full = P.init(sys_, _t(q), _t(qd), full=True)
  torch.cuda.synchronize()
  assert ((full.con_diag.abs() > 0).sum(-1) > 32).float().mean().item() >= 0.5
  c = P.init(sys_, _t(q), _t(qd))
  u = P.init(sys_, _t(q), _t(qd), cache=False)
  for _ in range(3):
    c = P.step(sys_, c, act, n_frames=2, inverse_mode=P.CHOLESKY)
    u = P.step(sys_, u, act, n_frames=2, inverse_mode=P.CHOLESKY)
    torch.cuda.synchronize()
    _same(c, u)


@pytest.mark.parametrize('tpe', [16, 32])
def test_cache_chain_both_team_widths(tpe):
  P = _P()
  sys_ = load('chain3')
  n = 40
  q, qd = seeded_inputs(sys_, n, 109)
  rng = np.random.default_rng(110)
  c = P.init(sys_, _t(q), _t(qd), threads_per_env=tpe)
  u = P.init(sys_, _t(q), _t(qd), cache=False, threads_per_env=tpe)
  for _ in range(3):
    act = _t(actions(sys_, n, rng))
    for mode in (P.CHOLESKY, P.NEWTON_SCHULZ):
      c = P.step(sys_, c, act, n_frames=2, inverse_mode=mode, threads_per_env=tpe)
      u = P.step(sys_, u, act, n_frames=2, inverse_mode=mode, threads_per_env=tpe)
      torch.cuda.synchronize()
      _same(c, u)
