"""The numpy restatement of the step's reverse-mode derivative (the checker
for the CUDA adjoint) against FP64 central finite differences."""

import numpy as np
import pytest

from oracle.adjoint import StepAdjoint
from oracle.pipeline import Oracle
from tests.parity_util import actions, load, seeded_inputs


def _fd_check(name, steps, B=4, seed=5):
  sys_ = load(name)
  o = Oracle(sys_, np.float64, exact_inverse=True)
  q, qd = seeded_inputs(sys_, B, seed)
  s = o.init(q, qd)
  rng = np.random.default_rng(seed + 1)
  for _ in range(steps):
    s = o.step(s, actions(sys_, B, rng))
  q, qd = s.q.copy(), s.qd.copy()
  act = actions(sys_, B, rng)
  adj = StepAdjoint(sys_)
  qn, qdn, T = adj.forward(q, qd, act)
  qbo, qdbo = rng.normal(size=qn.shape), rng.normal(size=qdn.shape)
  adj._xr = T['s'].x_rot
  grads = adj.vjp(T, qbo, qdbo)

  def f(q_, qd_, a_):
    r = o.step(o.restore(q_, qd_, None), a_)  # exact inverse of M(q_)
    return np.sum(qbo * r.q, -1) + np.sum(qdbo * r.qd, -1)

  eps = 1e-6
  for which, got in enumerate(grads):
    base = [q, qd, act]
    fd = np.zeros_like(got)
    for j in range(got.shape[1]):
      a = [x.copy() for x in base]
      a[which][:, j] += eps
      fp = f(*a)
      a[which][:, j] -= 2 * eps
      fd[:, j] = (fp - f(*a)) / (2 * eps)
    err = np.abs(got - fd).max(-1) / np.maximum(np.abs(fd).max(-1), 1e-9)
    assert err.max() < 1e-5, (name, which, err)
  return T


@pytest.mark.parametrize('name,steps', [('chain3', 3), ('quadruped', 6), ('quadruped', 40)])
def test_step_vjp_matches_finite_differences(name, steps):
  T = _fd_check(name, steps)
  if steps == 40:  # the landed quadruped exercises contact and limit rows
    assert (np.abs(T['s'].con_jac).max(-1) > 0).sum() > 0


def test_tail_fd_forced_onto_its_own_branch():
  """tests/grad_util.tail_fd with every projected-gradient solve forced onto
  the decisions the FP64 rollout takes by itself reproduces the free tail and
  its differences (the forcing the APG-workload check uses with the GPU's
  decisions)."""
  from oracle.adjoint import StepAdjoint
  from oracle.pipeline import Oracle
  from brax_gb300 import mjcf
  from tests import grad_util
  sys_ = mjcf.load_asset('quadruped')
  rng = np.random.default_rng(5)
  o = Oracle(sys_, np.float64, exact_inverse=True)
  s = o.init((sys_.init_q + rng.uniform(-0.1, 0.1, sys_.q_size()))[None], np.zeros((1, sys_.qd_size())))
  for _ in range(6):  # land
    s = o.env_step(s, rng.uniform(-1, 1, (1, sys_.act_size())), 5)
  L, F = 2, 2
  act = rng.uniform(-1, 1, (L, sys_.act_size()))
  adj = StepAdjoint(sys_)
  q, qd, forced = s.q.copy(), s.qd.copy(), []
  for j in range(L):
    row = []
    for _ in range(F):
      q, qd, T = adj.forward(q, qd, act[j][None])
      pg = T.get('pg', [])
      row.append((len(pg), int(np.count_nonzero(T['s'].con_diag[0])), [float(r['step'][0]) for r in pg]))
    forced.append(row)
  assert sum(r[1] for rr in forced for r in rr) > 0  # in contact
  args = ('quadruped', s.q[0], s.qd[0], act, F, (1e-4, 1e-5), [0, 3, 6], L)
  free = grad_util.tail_fd(args)
  pinned = grad_util.tail_fd(args + (forced,))
  assert pinned[3] and pinned[4] > 0
  np.testing.assert_allclose(pinned[1], free[1], rtol=0, atol=1e-10)
  np.testing.assert_allclose(pinned[2], free[2], rtol=0, atol=1e-10)
  for eps in (1e-4, 1e-5):
    np.testing.assert_allclose(pinned[0][eps], free[0][eps], rtol=1e-4, atol=1e-8)


@pytest.mark.parametrize('name,steps', [('chain3', 4), ('quadruped', 8), ('chain16', 3)])
def test_newton_schulz_rollout_vjp_matches_finite_differences(name, steps):
  """The reverse through the Newton-Schulz update of the carried inverse
  (brax/math.py:278-305, reset and best-iterate acceptance piecewise
  constant): three pipeline steps from an init state (exact inverse, as
  pipeline.init), the later two carrying Newton-Schulz inverses, against FP64
  central differences of the same Newton-Schulz rollout.  A hanging chain of
  16 links (mass-matrix condition 2e5), whose inverse resets every step,
  exercises the reset's derivative."""
  if name.startswith('chain') and name != 'chain3':
    from brax_gb300 import workloads
    sys_ = workloads.chain(int(name[5:]))
  else:
    sys_ = load(name)
  if sys_.matrix_inv_iterations == 0:
    pytest.skip('model uses the exact inverse')
  B, F = 4, 3
  o = Oracle(sys_, np.float64, exact_inverse=False)
  if name == 'chain16':
    from brax_gb300 import workloads
    q, qd = workloads.reset(sys_, B, np.random.default_rng(11))
  else:
    q, qd = seeded_inputs(sys_, B, 11)
  s = o.init(q, qd)
  rng = np.random.default_rng(12)
  for _ in range(steps):
    s = o.step(s, actions(sys_, B, rng))
  q0, qd0 = s.q.copy(), s.qd.copy()
  act = actions(sys_, B, rng)
  adj = StepAdjoint(sys_, newton_schulz=True)
  tapes, qq, qqd, minv = [], q0, qd0, None
  for _ in range(F):
    qn, qdn, T = adj.forward(qq, qqd, act, minv)
    tapes.append((T, T['s'].x_rot))
    qq, qqd, minv = qn, qdn, T['s'].mass_mx_inv
  qbo, qdbo = rng.normal(size=qq.shape), rng.normal(size=qqd.shape)
  qb, qdb, ab_tot, mb = qbo, qdbo, np.zeros_like(act), None
  for T, xr in reversed(tapes):
    adj._xr = xr
    qb, qdb, ab = adj.vjp(T, qb, qdb, mb)
    mb = adj.minvb_prev
    ab_tot += ab
  assert mb is None  # the first step's inverse is the exact one of pipeline.init
  if name == 'chain16':
    assert any(bool(T['ns']['reset'].any()) for T, _ in tapes[1:])

  def f(q_, qd_, a_):
    r = o.env_step(o.init(q_, qd_), a_, F)
    return np.sum(qbo * r.q, -1) + np.sum(qdbo * r.qd, -1)

  eps = 1e-6
  for which, got in enumerate((qb, qdb, ab_tot)):
    base = [q0, qd0, act]
    fd = np.zeros_like(got)
    for j in range(got.shape[1]):
      a = [x.copy() for x in base]
      a[which][:, j] += eps
      fp = f(*a)
      a[which][:, j] -= 2 * eps
      fd[:, j] = (fp - f(*a)) / (2 * eps)
    err = np.abs(got - fd).max(-1) / np.maximum(np.abs(fd).max(-1), 1e-9)
    assert err.max() < 1e-5, (name, which, err)
