"""Fluid forces (brax/fluid.py:53-82, added to the passive forces at
brax/generalized/dynamics.py:198-211).

The reference's own fluid tests compare against MuJoCo, which is not
available; the oracle's restatement is pinned instead by closed-form
behaviour of a free sphere (mass m, radius r, principal moments 0.4 m r^2, so
an inertia box of edge sqrt(2.4) r): under viscosity mu alone it falls at
the Stokes terminal velocity m g / (3 pi d mu) with d the box's mean edge, under
density rho alone at sqrt(2 m g / (rho b^2)), and its spin decays by the
factor 1 - dt pi d^3 mu / I per Euler step.  The GPU step is then held to the
oracle on a free-floating three-link swimmer-like chain.
"""

import dataclasses

import numpy as np
import pytest

from brax_gb300 import mjcf
from oracle.pipeline import Oracle
from tests.parity_util import rel_err

_BALL = """<mujoco model="ball">
  <option timestep="0.01" viscosity="%g" density="%g"/>
  <worldbody>
    <body name="ball" pos="0 0 1">
      <freejoint/>
      <geom type="sphere" size="0.1" mass="1" contype="0" conaffinity="0"/>
    </body>
  </worldbody>
</mujoco>"""

# three capsules in a plane, free root, two hinges, in a viscous dense fluid
_SWIMMER = """<mujoco model="swimmer3">
  <option timestep="0.01" viscosity="0.1" density="4000" gravity="0 0 0"/>
  <default>
    <joint damping="0.1" armature="0.1" limited="true" range="-100 100"/>
    <geom type="capsule" size="0.1" density="1000" contype="0" conaffinity="0"/>
  </default>
  <worldbody>
    <body name="head" pos="0 0 0">
      <freejoint/>
      <geom fromto="0 0 0 -1 0 0"/>
      <body name="mid" pos="-1 0 0">
        <joint name="j1" type="hinge" axis="0 0 1"/>
        <geom fromto="0 0 0 -1 0 0"/>
        <body name="tail" pos="-1 0 0">
          <joint name="j2" type="hinge" axis="0 0 1"/>
          <geom fromto="0 0 0 -1 0 0"/>
        </body>
      </body>
    </body>
  </worldbody>
  <actuator>
    <motor joint="j1" gear="150" ctrlrange="-1 1" ctrllimited="true"/>
    <motor joint="j2" gear="150" ctrlrange="-1 1" ctrllimited="true"/>
  </actuator>
</mujoco>"""


def _ball(mu, rho):
  return mjcf.loads(_BALL % (mu, rho))


@pytest.mark.parametrize('mu,rho', [(1.0, 0.0), (0.0, 100.0)])
def test_terminal_velocity(mu, rho):
  sys = _ball(mu, rho)
  assert sys.enable_fluid
  o = Oracle(sys, np.float64, exact_inverse=True)
  s = o.init(sys.init_q[None].copy(), np.zeros((1, 6)))
  for _ in range(1500):
    s = o.step(s, np.zeros((1, 0)))
  b = np.sqrt(2.4) * 0.1
  vt = 9.81 / (3 * np.pi * b * mu) if mu else np.sqrt(2 * 9.81 / (rho * b * b))
  np.testing.assert_allclose(s.qd[0, 2], -vt, rtol=1e-9)
  np.testing.assert_allclose(s.qd[0, [0, 1, 3, 4, 5]], 0, atol=1e-12)


def test_viscous_spin_decay():
  mu = 1.0
  sys = dataclasses.replace(_ball(mu, 0.0), gravity=np.zeros(3))
  o = Oracle(sys, np.float64, exact_inverse=True)
  qd = np.zeros((1, 6))
  qd[0, 3] = 2.0
  s = o.init(sys.init_q[None].copy(), qd)
  n = 50
  for _ in range(n):
    s = o.step(s, np.zeros((1, 0)))
  b = np.sqrt(2.4) * 0.1
  inertia = 0.4 * 1.0 * 0.1 ** 2
  expect = 2.0 * (1 - sys.dt * np.pi * b ** 3 * mu / inertia) ** n
  np.testing.assert_allclose(s.qd[0, 3], expect, rtol=1e-9)


def test_fluid_off_changes_nothing():
  """viscosity = density = 0 leaves the passive forces as they were."""
  sys = _ball(0.0, 0.0)
  assert not sys.enable_fluid


def _seeded(sys, n, seed):
  rng = np.random.default_rng(seed)
  q = np.tile(sys.init_q, (n, 1))
  q[:, 7:] += rng.uniform(-0.5, 0.5, (n, sys.q_size() - 7))
  qd = rng.normal(0, 0.5, (n, sys.qd_size()))
  return q.astype(np.float32), qd.astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize('inverse', ['cholesky', 'newton_schulz'])
def test_gpu_swimmer_matches_oracle(inverse):
  torch = pytest.importorskip('torch')
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline as P
  sys = mjcf.loads(_SWIMMER)
  assert sys.enable_fluid
  n = 64
  q, qd = _seeded(sys, n, 3)
  act = np.random.default_rng(4).uniform(-1, 1, (n, sys.act_size())).astype(np.float32)
  exact = inverse == 'cholesky'
  mode = P.CHOLESKY if exact else P.NEWTON_SCHULZ
  o32 = Oracle(sys, np.float32, exact_inverse=exact)
  o64 = Oracle(sys, np.float64, exact_inverse=exact)
  r32 = o32.init(q, qd)
  r64 = o64.init(q.astype(np.float64), qd.astype(np.float64))
  t = lambda x: torch.as_tensor(x, device='cuda')
  s = P.init(sys, t(q), t(qd))
  for _ in range(3):
    s = P.step(sys, s, t(act), n_frames=5, inverse_mode=mode)
    for _ in range(5):
      r32 = o32.step(r32, act)
      r64 = o64.step(r64, act.astype(np.float64))
  torch.cuda.synchronize()
  assert (s.status.cpu().numpy() == 0).all()
  for f in ('q', 'qd'):
    g = getattr(s, f).cpu().numpy()
    e64 = rel_err(g, getattr(r64, f))
    eo = rel_err(getattr(r32, f), getattr(r64, f))
    print(f'swimmer {inverse} {f}: vs fp64 p99 {np.quantile(e64, 0.99):.2e} max {e64.max():.2e} | '
          f'fp32 oracle vs fp64 p99 {np.quantile(eo, 0.99):.2e}')
    assert np.quantile(e64, 0.99) <= max(1e-5, 3 * np.quantile(eo, 0.99)), f
    assert e64.max() <= max(1e-4, 3 * eo.max()), f


@pytest.mark.gpu
def test_gpu_ball_terminal_velocity():
  torch = pytest.importorskip('torch')
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline as P
  sys = _ball(1.0, 0.0)
  n = 8
  q = np.tile(sys.init_q, (n, 1)).astype(np.float32)
  s = P.init(sys, torch.as_tensor(q, device='cuda'), torch.zeros(n, 6, device='cuda'))
  s, _ = P.rollout(sys, s, torch.zeros(1500, n, 0, device='cuda'), inverse_mode=P.CHOLESKY)
  torch.cuda.synchronize()
  vt = 9.81 / (3 * np.pi * np.sqrt(2.4) * 0.1)
  np.testing.assert_allclose(s.qd[:, 2].cpu().numpy(), -vt, rtol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize('inverse', ['cholesky', 'newton_schulz'])
def test_gpu_swimmer_gradient(inverse):
  """The gradient through the fluid forces (the inertia-box drag of
  fluid.py:53-82 added to the passive forces, dynamics.py:198-211): the
  swimmer, 8 envs, 3 env steps of 5 frames, d loss / d (qd0, actions)
  against FP64 central differences of the FP64 rollout (the median of steps
  1e-5, 1e-6, 1e-7 per env)."""
  torch = pytest.importorskip('torch')
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline as P
  sys = mjcf.loads(_SWIMMER)
  n, H, F = 8, 3, 5
  q, qd = _seeded(sys, n, 5)
  rng = np.random.default_rng(6)
  u = rng.uniform(-1, 1, (H, n, sys.act_size())).astype(np.float32)
  q_bar = rng.normal(size=(H, n, sys.q_size()))
  qd_bar = rng.normal(size=(H, n, sys.qd_size()))
  exact = inverse == 'cholesky'
  mode = P.CHOLESKY if exact else P.NEWTON_SCHULZ
  t = lambda x: torch.as_tensor(np.asarray(x, np.float32), device='cuda')
  r = P.rollout_grad(sys, t(q), t(qd), t(u), t(q_bar), t(qd_bar), n_frames=F, ckpt_every=1, trajectory=True,
                     inverse_mode=mode)
  s0 = P.bare_state(t(q), t(qd)) if exact else P.init(sys, t(q), t(qd))
  _, (rq, rqd) = P.rollout(sys, s0, t(u), n_frames=F, inverse_mode=mode, trajectory=True)
  torch.cuda.synchronize()
  assert (r[3].cpu().numpy() == 0).all()
  torch.testing.assert_close(r[4][0], rq, rtol=0, atol=0)
  torch.testing.assert_close(r[4][1], rqd, rtol=0, atol=0)
  o = Oracle(sys, np.float64, exact_inverse=exact)
  q64, qd64, u64 = q.astype(np.float64), qd.astype(np.float64), u.astype(np.float64)

  def loss(qd0, uu):
    st = o.init(q64, qd0)
    tot = np.zeros(n)
    for k in range(H):
      st = o.env_step(st, uu[k], F)
      tot += np.sum(q_bar[k] * st.q, -1) + np.sum(qd_bar[k] * st.qd, -1)
    return tot

  def fd(f, x, idx):
    est = []
    for eps in (1e-5, 1e-6, 1e-7):
      a, b = x.copy(), x.copy()
      a[idx] += eps
      b[idx] -= eps
      est.append((f(a) - f(b)) / (2 * eps))
    return np.median(np.stack(est), 0)

  g_qd = np.stack([fd(lambda x: loss(x, u64), qd64, (slice(None), j)) for j in range(sys.qd_size())], 1)
  g_u = np.stack([np.stack([fd(lambda x: loss(qd64, x), u64, (k, slice(None), j)) for j in range(sys.act_size())], 1)
                  for k in range(H)], 0)
  rel = lambda a, b: np.abs(a - b).reshape(n, -1).max(-1) / np.maximum(np.abs(b).reshape(n, -1).max(-1), 1e-6)
  eq = rel(r[2].cpu().numpy(), g_qd)
  eu = rel(np.swapaxes(r[0].cpu().numpy(), 0, 1), np.swapaxes(g_u, 0, 1))
  print(f'swimmer {inverse} gradient vs FP64 FD: qd0 per env {" ".join(f"{v:.2e}" for v in eq)}; '
        f'act per env {" ".join(f"{v:.2e}" for v in eu)}')
  for e in (eq, eu):
    assert np.median(e) <= 1e-4 and e.max() <= 1e-3
