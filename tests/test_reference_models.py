"""The reference's environment models (brax/envs/assets/*.xml) through the
GPU step, against the oracle.

The models are compiled by brax_gb300.mjcf and carried as JSON
(tests/golden/reference_models.json, written by make_reference_models.py),
so the GPU tests need no reference checkout.  Each model takes one pipeline
step (the unit of the single-step error bar) from seeded states near its
init_q with U(-1, 1) actions; every field of the step must match the FP64
oracle within max(floor, 3x the FP32 oracle's own FP64 error) for 99 % of
envs, with floor 1e-5 for q and qd (the single-step bar) and 1e-4 for the
intermediate fields.  The FP32 error of a contact step is set by the projected-gradient
solve's tolerance-based stopping and varies several-fold with the operation
order, so the FP32 scale is the largest over three FP32 oracle runs: the
inputs as given and two copies with every input moved by one ulp.
"""

import dataclasses
import json
import os

import numpy as np
import pytest

from brax_gb300 import mjcf
from brax_gb300 import system as S
from oracle.pipeline import Oracle
from tests.parity_util import rel_err

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'reference_models.json')
MODELS = json.load(open(GOLDEN))


def _sys(name):
  return S.from_json(json.dumps(MODELS[name]))


def _inputs(sys_, n, seed):
  rng = np.random.default_rng(seed)
  q = np.tile(sys_.init_q, (n, 1)) + rng.uniform(-0.05, 0.05, (n, sys_.q_size()))
  qa = 0
  for t in sys_.link_types:
    if t == 'f':
      r = q[:, qa + 3:qa + 7]
      q[:, qa + 3:qa + 7] = r / np.linalg.norm(r, axis=1, keepdims=True)
    qa += S.Q_WIDTHS[t]
  qd = 0.05 * rng.normal(size=(n, sys_.qd_size()))
  act = rng.uniform(-1, 1, (n, sys_.act_size()))
  return q.astype(np.float32), qd.astype(np.float32), act.astype(np.float32)


def _eq(a, b):
  if dataclasses.is_dataclass(a):
    return type(a) is type(b) and all(_eq(getattr(a, f.name), getattr(b, f.name))
                                      for f in dataclasses.fields(a))
  if isinstance(a, np.ndarray):
    return (isinstance(b, np.ndarray) and a.dtype == b.dtype and a.shape == b.shape
            and np.array_equal(a, b, equal_nan=True))
  if isinstance(a, (list, tuple)):
    return type(a) is type(b) and len(a) == len(b) and all(_eq(x, y) for x, y in zip(a, b))
  return a == b


@pytest.mark.parametrize('asset', ['quadruped', 'humanoid_like', 'chain3'])
def test_json_round_trip_is_exact(asset):
  s = mjcf.load_asset(asset)
  assert _eq(S.from_json(S.to_json(s)), s)


def test_fixture_matches_the_compiler(ref_path):
  """The committed models are what the compiler makes of the reference's XML."""
  for name in MODELS:
    s = mjcf.load(os.path.join(ref_path, 'brax/envs/assets', name + '.xml'))
    assert _eq(_sys(name), s), name


@pytest.mark.gpu
@pytest.mark.parametrize('name,inverse', [(n, 'cholesky') for n in sorted(MODELS)] +
                         [('ant', 'newton_schulz'), ('humanoid', 'newton_schulz'),
                          ('walker2d', 'newton_schulz')])
def test_gpu_step_matches_oracle(name, inverse):
  torch = pytest.importorskip('torch')
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline as P
  sys_ = _sys(name)
  n = 48
  q, qd, act = _inputs(sys_, n, 11)
  exact = inverse == 'cholesky'
  o32 = Oracle(sys_, np.float32, exact_inverse=exact)
  o64 = Oracle(sys_, np.float64, exact_inverse=exact)
  r64 = o64.step(o64.init(q.astype(np.float64), qd.astype(np.float64)), act.astype(np.float64))
  rng = np.random.default_rng(12)
  ulp = lambda x: np.nextafter(x, np.where(rng.random(x.shape) < 0.5, -np.inf, np.inf).astype(np.float32))
  r32s = [o32.step(o32.init(qq, qqd), act) for qq, qqd in ((q, qd), (ulp(q), ulp(qd)), (ulp(q), ulp(qd)))]
  t = lambda x: torch.as_tensor(x, device='cuda')
  s = P.init(sys_, t(q), t(qd), full=True)
  s = P.step(sys_, s, t(act), n_frames=1, inverse_mode=P.CHOLESKY if exact else P.NEWTON_SCHULZ,
             full=True)
  torch.cuda.synchronize()
  assert (s.status.cpu().numpy() == 0).all(), name
  for f in ('q', 'qd', 'qf_smooth', 'qf_constraint', 'qdd', 'x_pos', 'x_rot', 'mass_mx', 'mass_mx_inv',
            'con_jac', 'con_diag', 'con_aref'):
    g = getattr(s, f).cpu().numpy()
    e64 = rel_err(g, getattr(r64, f))
    eos = [rel_err(getattr(r, f), getattr(r64, f)) for r in r32s]
    eo99 = max(np.quantile(e, 0.99) for e in eos)
    eomax = max(e.max() for e in eos)
    print(f'{name} {inverse} {f}: vs fp64 p99 {np.quantile(e64, 0.99):.2e} max {e64.max():.2e} | '
          f'fp32 oracle vs fp64 p99 {eo99:.2e} max {eomax:.2e}')
    floor = 1e-5 if f in ('q', 'qd') else 1e-4  # the metric's bar on q / qd
    assert np.quantile(e64, 0.99) <= max(floor, 3 * eo99), (name, f)
    assert e64.max() <= max(10 * floor, 3 * eomax), (name, f)


@pytest.mark.gpu
@pytest.mark.parametrize('name', sorted(MODELS))
def test_gpu_rollout_gradient(name):
  """APG's gradient on each of the reference's env models (the swimmer's
  through its fluid forces): 4 envs, 2 env steps, the
  gradient kernel's forward equal to the plain rollout bit for bit, no env
  flagged, and d loss / d qd0 against FP64 central differences of the FP64
  rollout (the median of steps 1e-5, 1e-6, 1e-7 per env; median env within
  1e-4, every env within 1e-3; measured <= 2.4e-6)."""
  torch = pytest.importorskip('torch')
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline as P
  sys_ = _sys(name)
  n, H = 4, 2
  q, qd, _ = _inputs(sys_, n, 21)
  rng = np.random.default_rng(22)
  u = rng.uniform(-1, 1, (H, n, sys_.act_size())).astype(np.float32)
  q_bar = rng.normal(size=(H, n, sys_.q_size())) * 0.1
  qd_bar = rng.normal(size=(H, n, sys_.qd_size())) * 0.1
  t = lambda x: torch.as_tensor(np.asarray(x, np.float32), device='cuda')
  r = P.rollout_grad(sys_, t(q), t(qd), t(u), t(q_bar), t(qd_bar), n_frames=1, ckpt_every=1, trajectory=True)
  _, (rq, rqd) = P.rollout(sys_, P.bare_state(t(q), t(qd)), t(u), n_frames=1, inverse_mode=P.CHOLESKY,
                           trajectory=True)
  torch.cuda.synchronize()
  assert (r[3].cpu().numpy() == 0).all(), (name, r[3])
  torch.testing.assert_close(r[4][0], rq, rtol=0, atol=0)
  torch.testing.assert_close(r[4][1], rqd, rtol=0, atol=0)
  o = Oracle(sys_, np.float64, exact_inverse=True)
  q64, qd64, u64 = q.astype(np.float64), qd.astype(np.float64), u.astype(np.float64)

  def loss(qd0):
    s = o.init(q64, qd0)
    tot = np.zeros(n)
    for k in range(H):
      s = o.env_step(s, u64[k], 1)
      tot += np.sum(q_bar[k] * s.q, -1) + np.sum(qd_bar[k] * s.qd, -1)
    return tot

  fd = np.zeros((n, sys_.qd_size()))
  for j in range(sys_.qd_size()):
    est = []
    for eps in (1e-5, 1e-6, 1e-7):
      a, b = qd64.copy(), qd64.copy()
      a[:, j] += eps
      b[:, j] -= eps
      est.append((loss(a) - loss(b)) / (2 * eps))
    fd[:, j] = np.median(np.stack(est), 0)
  got = r[2].cpu().numpy().astype(np.float64)
  e = np.abs(got - fd).max(-1) / np.maximum(np.abs(fd).max(-1), 1e-6)
  print(f'{name} rollout gradient d/dqd0 vs FP64 FD: per env {" ".join(f"{v:.2e}" for v in e)}')
  assert np.median(e) <= 1e-4 and e.max() <= 1e-3, name
