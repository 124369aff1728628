"""GPU adjoint: braxg_rollout_vjp against (1) the numpy reverse of one
pipeline step (oracle/adjoint.py, itself pinned to FP64 finite differences)
and (2) FP64 central finite differences of an APG-style rollout loss.

Tolerances: relative error (max-abs difference / max-abs reference, per env)
<= 2e-3 for the single step against the FP64 reverse (95 % of envs), and
median <= 1e-3 with 7 of 8 envs <= 1e-2 for the 6-env-step rollout against FP64
central differences.  The differences use eps = 1e-5: at eps = 1e-4 the
perturbed rollouts of some envs cross a discrete switch (a contact activating,
a line-search or projection decision flipping), and the difference quotient
jumps by 100x (e.g. 39.8 against a true slope of -0.336, which eps 1e-5 and
1e-6 both reproduce); the adjoint, like jax.grad, differentiates the branch
taken.
"""

import numpy as np
import pytest

from tests.parity_util import actions, load, seeded_inputs

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _P():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline
  return pipeline


def _t(x):
  return torch.as_tensor(np.asarray(x, np.float32), device='cuda')


def _rel(a, b):
  a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
  b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
  return np.abs(a - b).max(-1) / np.maximum(np.abs(b).max(-1), 1e-6)


def _fd_median(loss, x, index, eps_list=(1e-5, 1e-6, 1e-7)):
  """Central differences of loss (per env) in x[index], at three step sizes,
  the median of the three per env: a perturbation that moves a discrete
  decision of the solve (a line-search test, an iteration count) spoils one
  of the three, not the median."""
  out = []
  for eps in eps_list:
    a_, b_ = x.copy(), x.copy()
    a_[index] += eps
    b_[index] -= eps
    out.append((loss(a_) - loss(b_)) / (2 * eps))
  return np.median(np.stack(out), 0)


@pytest.mark.parametrize('name,steps', [('chain3', 3), ('quadruped', 3), ('quadruped', 40)])
def test_single_step_vjp_matches_numpy_reverse(name, steps):
  P = _P()
  from oracle.adjoint import StepAdjoint
  from oracle.pipeline import Oracle
  sys_ = load(name)
  n = 32
  o = Oracle(sys_, np.float64, exact_inverse=True)
  q, qd = seeded_inputs(sys_, n, 7)
  s = o.init(q, qd)
  rng = np.random.default_rng(8)
  for _ in range(steps):
    s = o.step(s, actions(sys_, n, rng))
  q, qd = s.q.astype(np.float32).astype(np.float64), s.qd.astype(np.float32).astype(np.float64)
  act = actions(sys_, n, rng).astype(np.float32).astype(np.float64)
  qbo, qdbo = rng.normal(size=q.shape), rng.normal(size=qd.shape)
  adj = StepAdjoint(sys_)
  _, _, T = adj.forward(q, qd, act)
  adj._xr = T['s'].x_rot
  rq, rqd, ract = adj.vjp(T, qbo, qdbo)
  act_bar, q0b, qd0b, status, _ = P.rollout_grad(
      sys_, _t(q), _t(qd), _t(act[None]), _t(qbo[None]), _t(qdbo[None]), n_frames=1, ckpt_every=1)
  torch.cuda.synchronize()
  st = status.cpu().numpy()
  assert (st == 0).all(), st
  for nm, g, r in (('q', q0b, rq), ('qd', qd0b, rqd), ('act', act_bar[0], ract)):
    e = _rel(g.cpu().numpy(), r)
    print(f'{name} steps={steps} {nm}: p50 {np.median(e):.2e} max {e.max():.2e}')
    assert np.quantile(e, 0.95) <= 2e-3, (nm, np.sort(e)[-4:])


def test_rollout_gradient_matches_finite_differences():
  P = _P()
  from oracle.pipeline import Oracle
  sys_ = load('quadruped')
  n, H, F = 8, 6, 5
  q0, qd0 = seeded_inputs(sys_, n, 21)
  rng = np.random.default_rng(22)
  u = rng.uniform(-1, 1, (H, n, sys_.act_size()))
  o = Oracle(sys_, np.float64, exact_inverse=True)

  def loss(qd0_, u_):  # -mean_t torso x-velocity + 1e-3 sum |u|^2, per env
    s = o.init(q0, qd0_)
    tot = np.zeros(n)
    for t in range(H):
      s = o.env_step(s, u_[t], F)
      tot += -s.qd[:, 0] / H
    return tot + 1e-3 * np.sum(u_ ** 2, axis=(0, 2))

  qd_bar = np.zeros((H, n, sys_.qd_size()))
  qd_bar[:, :, 0] = -1.0 / H
  act_bar, _, qd0b, status, _ = P.rollout_grad(
      sys_, _t(q0), _t(qd0), _t(u), None, _t(qd_bar), n_frames=F, ckpt_every=2)
  torch.cuda.synchronize()
  assert (status.cpu().numpy() == 0).all()
  g_u = act_bar.cpu().numpy() + 2e-3 * u
  eps = 1e-5
  fd_u = np.zeros_like(u)
  for t in range(H):
    for k in range(sys_.act_size()):
      up, um = u.copy(), u.copy()
      up[t, :, k] += eps
      um[t, :, k] -= eps
      fd_u[t, :, k] = (loss(qd0, up) - loss(qd0, um)) / (2 * eps)
  fd_qd = np.zeros((n, sys_.qd_size()))
  for k in range(sys_.qd_size()):
    a, b = qd0.copy(), qd0.copy()
    a[:, k] += eps
    b[:, k] -= eps
    fd_qd[:, k] = (loss(a, u) - loss(b, u)) / (2 * eps)
  eu = _rel(np.swapaxes(g_u, 0, 1), np.swapaxes(fd_u, 0, 1))
  eq = _rel(qd0b.cpu().numpy(), fd_qd)
  print(f'rollout grad vs FP64 FD: act p50 {np.median(eu):.2e} max {eu.max():.2e}; '
        f'qd0 p50 {np.median(eq):.2e} max {eq.max():.2e}')
  assert np.median(eu) <= 1e-3 and (eu <= 1e-2).mean() >= 7 / 8
  assert np.median(eq) <= 1e-3 and (eq <= 1e-2).mean() >= 7 / 8


@pytest.mark.parametrize('name', ['chain3', 'quadruped'])
def test_newton_schulz_gradient(name):
  """Gradients in the reference's inverse mode (the carried Newton-Schulz
  inverse, exact at the first frame as pipeline.init computes it): the
  gradient kernel's forward is the Newton-Schulz rollout bit for bit, the
  split halves and every residency give the fused launch's bits, and the
  gradient matches FP64 central differences of the FP64 Newton-Schulz
  rollout (brax/math.py:278-305 under jax.grad)."""
  P = _P()
  from oracle.pipeline import Oracle
  sys_ = load(name)
  n, H, F, k = 8, 4, (1 if name == 'chain3' else 5), 2
  q0, qd0 = seeded_inputs(sys_, n, 23)
  rng = np.random.default_rng(24)
  u = actions(sys_, n * H, rng).reshape(H, n, -1) if sys_.act_size() else np.zeros((H, n, 0))
  qd_bar = np.zeros((H, n, sys_.qd_size()))
  qd_bar[:, :, 0] = -1.0 / H
  q_bar = rng.normal(size=(H, n, sys_.q_size())) * 1e-2
  NS = P.NEWTON_SCHULZ
  fused = P.rollout_grad(sys_, _t(q0), _t(qd0), _t(u), _t(q_bar), _t(qd_bar), n_frames=F, ckpt_every=k,
                         trajectory=True, inverse_mode=NS)
  small = P.rollout_grad(sys_, _t(q0), _t(qd0), _t(u), _t(q_bar), _t(qd_bar), n_frames=F, ckpt_every=k,
                         resident_segments=1, inverse_mode=NS)
  (tq, tqd), tape = P.rollout_vjp_fwd(sys_, _t(q0), _t(qd0), _t(u), n_frames=F, ckpt_every=k, inverse_mode=NS)
  split = P.rollout_vjp_bwd(tape, _t(q_bar), _t(qd_bar))
  roll, (rq, rqd) = P.rollout(sys_, P.init(sys_, _t(q0), _t(qd0)), _t(u), n_frames=F, inverse_mode=NS,
                              trajectory=True)
  torch.cuda.synchronize()
  assert (fused[3] == 0).all()
  torch.testing.assert_close(fused[4][0], rq, rtol=0, atol=0)  # the Newton-Schulz rollout's trajectory
  torch.testing.assert_close(fused[4][1], rqd, rtol=0, atol=0)
  for other in (small, split):
    for a_, b_ in zip(other[:3], fused[:3]):
      torch.testing.assert_close(a_, b_, rtol=0, atol=0)
  # torch.autograd through differentiable_rollout: the same bits, and without
  # a gradient to take the plain Newton-Schulz rollout
  ut = _t(u).requires_grad_(True)
  dq, dqd = P.differentiable_rollout(sys_, _t(q0), _t(qd0), ut, n_frames=F, ckpt_every=k, inverse_mode=NS)
  ((dq * _t(q_bar)).sum() + (dqd * _t(qd_bar)).sum()).backward()
  with torch.no_grad():
    pq, pqd = P.differentiable_rollout(sys_, _t(q0), _t(qd0), _t(u), n_frames=F, inverse_mode=NS)
  torch.cuda.synchronize()
  for a_, b_ in ((dq, rq), (dqd, rqd), (pq, rq), (pqd, rqd)):
    torch.testing.assert_close(a_.detach(), b_, rtol=0, atol=0)
  torch.testing.assert_close(ut.grad, fused[0], rtol=0, atol=0)
  # against FP64 central differences of the Newton-Schulz rollout
  o = Oracle(sys_, np.float64, exact_inverse=False)

  def loss(q0_, qd0_, u_):
    s = o.init(q0_, qd0_)
    tot = np.zeros(n)
    for t in range(H):
      s = o.env_step(s, u_[t], F)
      tot += np.sum(q_bar[t] * s.q, -1) + np.sum(qd_bar[t] * s.qd, -1)
    return tot

  eps = 1e-5
  errs = []
  for which, got in ((2, fused[2].cpu().numpy()), (0, fused[0].cpu().numpy())):
    if which == 0 and sys_.act_size() == 0:
      continue
    base = [q0, qd0, u]
    fd = np.zeros(got.shape)
    if which == 2:
      for j in range(sys_.qd_size()):
        a_, b_ = qd0.copy(), qd0.copy()
        a_[:, j] += eps
        b_[:, j] -= eps
        fd[:, j] = (loss(q0, a_, u) - loss(q0, b_, u)) / (2 * eps)
      e = _rel(got, fd)
    else:
      for t in range(H):
        for j in range(sys_.act_size()):
          a_, b_ = u.copy(), u.copy()
          a_[t, :, j] += eps
          b_[t, :, j] -= eps
          fd[t, :, j] = (loss(q0, qd0, a_) - loss(q0, qd0, b_)) / (2 * eps)
      e = _rel(np.swapaxes(got, 0, 1), np.swapaxes(fd, 0, 1))
    errs.append(e)
    print(f'{name} Newton-Schulz gradient vs FP64 FD ({["act", "", "qd0"][which]}): p50 {np.median(e):.2e} '
          f'max {e.max():.2e}')
  for e in errs:
    assert np.median(e) <= 1e-3 and (e <= 1e-2).mean() >= 7 / 8


def test_newton_schulz_gradient_reset():
  """The reset branch of the Newton-Schulz update on the GPU: a hanging chain
  of 16 links (mass-matrix condition 2e5) whose carried inverse resets to
  0.5 M^T / tr(M M^T) (brax/math.py:292-295) on the frames after the first;
  one env step of 3 frames, gradient against FP64 central differences of the
  FP64 Newton-Schulz rollout.  The oracle's tape of the same step shows the
  resets.  Bar: every env within 5e-3; FP32 rounding in this model's
  inverse is of order cond(M) x 6e-8 ~ 1e-2 relative in the worst
  direction (measured: 5e-5 .. 2.4e-3)."""
  P = _P()
  from brax_gb300 import workloads
  from oracle.adjoint import StepAdjoint
  from oracle.pipeline import Oracle
  sys_ = workloads.chain(16)
  n, F = 4, 3
  o = Oracle(sys_, np.float64, exact_inverse=False)
  q, qd = workloads.reset(sys_, n, np.random.default_rng(11))
  s = o.init(q, qd)
  rng = np.random.default_rng(12)
  for _ in range(3):
    s = o.step(s, actions(sys_, n, rng))
  q0, qd0 = s.q.astype(np.float32).astype(np.float64), s.qd.astype(np.float32).astype(np.float64)
  act = actions(sys_, n, rng).astype(np.float32).astype(np.float64)
  # the resets happen on this step (FP64 tape of the same frames)
  adj = StepAdjoint(sys_, newton_schulz=True)
  qq, qqd, minv, resets = q0, qd0, None, 0
  for f in range(F):
    qq, qqd, T = adj.forward(qq, qqd, act, minv)
    minv = T['s'].mass_mx_inv
    if f > 0:
      resets += int(T['ns']['reset'].sum())
  assert resets > 0
  qbo, qdbo = rng.normal(size=(n, sys_.q_size())), rng.normal(size=(n, sys_.qd_size()))
  act_bar, q0_bar, qd0_bar, status, _ = P.rollout_grad(
      sys_, _t(q0), _t(qd0), _t(act[None]), _t(qbo[None]), _t(qdbo[None]), n_frames=F, ckpt_every=1,
      inverse_mode=P.NEWTON_SCHULZ)
  torch.cuda.synchronize()
  assert (status.cpu().numpy() == 0).all()

  def f(q_, qd_, a_):
    r = o.env_step(o.init(q_, qd_), a_, F)
    return np.sum(qbo * r.q, -1) + np.sum(qdbo * r.qd, -1)

  eps = 1e-6
  for which, got in enumerate((q0_bar.cpu().numpy(), qd0_bar.cpu().numpy(), act_bar[0].cpu().numpy())):
    base = [q0, qd0, act]
    fd = np.zeros_like(got, dtype=np.float64)
    for j in range(got.shape[1]):
      a_ = [x.copy() for x in base]
      a_[which][:, j] += eps
      fp = f(*a_)
      a_[which][:, j] -= 2 * eps
      fd[:, j] = (fp - f(*a_)) / (2 * eps)
    e = _rel(got, fd)
    print(f'chain16 Newton-Schulz (resets {resets}) gradient vs FP64 FD ({["q0", "qd0", "act"][which]}): '
          f'per env {" ".join(f"{v:.2e}" for v in e)}')
    assert e.max() <= 5e-3


def test_torch_autograd_function():
  P = _P()
  sys_ = load('quadruped')
  n, H = 16, 4
  q0, qd0 = seeded_inputs(sys_, n, 31)
  q0t, qd0t = _t(q0), _t(qd0).requires_grad_(True)
  u = _t(np.random.default_rng(32).uniform(-1, 1, (H, n, sys_.act_size()))).requires_grad_(True)
  tq, tqd = P.differentiable_rollout(sys_, q0t, qd0t, u, n_frames=5, ckpt_every=2)
  loss = -tqd[:, :, 0].mean() + 1e-3 * (u ** 2).sum()
  loss.backward()
  assert u.grad is not None and torch.isfinite(u.grad).all()
  assert qd0t.grad is not None and torch.isfinite(qd0t.grad).all()
  assert u.grad.abs().sum() > 0


def test_gradient_independent_of_resident_segments():
  """Checkpoint segments either stay resident from the checkpoint pass or are
  recomputed; both give the same frame snapshots, so the same gradient bits."""
  P = _P()
  sys_ = load('quadruped')
  n, H, k = 24, 8, 2  # four checkpoint segments
  q0, qd0 = seeded_inputs(sys_, n, 33)
  rng = np.random.default_rng(34)
  u = _t(rng.uniform(-1, 1, (H, n, sys_.act_size())))
  qdb = _t(rng.normal(size=(H, n, sys_.qd_size())))
  res = [P.rollout_grad(sys_, _t(q0), _t(qd0), u, None, qdb, n_frames=5, ckpt_every=k,
                        resident_segments=r) for r in (1, 2, 4, None)]
  torch.cuda.synchronize()
  for r in res[1:]:
    for a, b in zip(r[:4], res[0][:4]):
      torch.testing.assert_close(a, b, rtol=0, atol=0)


@pytest.mark.parametrize('resident', [1, None])
def test_split_forward_and_reverse_equal_the_fused_launch(resident):
  """braxg_rollout_vjp_fwd then braxg_rollout_vjp_bwd on its workspace give
  bitwise the trajectory and gradient of one braxg_rollout_vjp launch, with
  every segment resident and with the smallest workspace (the reverse then
  recomputes the non-resident segments from the forward's checkpoints)."""
  P = _P()
  sys_ = load('quadruped')
  n, H, k = 24, 8, 2
  q0, qd0 = seeded_inputs(sys_, n, 35)
  rng = np.random.default_rng(36)
  u = _t(rng.uniform(-1, 1, (H, n, sys_.act_size())))
  qb = _t(rng.normal(size=(H, n, sys_.q_size())))
  qdb = _t(rng.normal(size=(H, n, sys_.qd_size())))
  fused = P.rollout_grad(sys_, _t(q0), _t(qd0), u, qb, qdb, n_frames=5, ckpt_every=k, trajectory=True,
                         resident_segments=resident)
  (tq, tqd), tape = P.rollout_vjp_fwd(sys_, _t(q0), _t(qd0), u, n_frames=5, ckpt_every=k,
                                      resident_segments=resident)
  act_bar, q0_bar, qd0_bar, status = P.rollout_vjp_bwd(tape, qb, qdb)
  torch.cuda.synchronize()
  assert (status == 0).all()
  for a, b in ((act_bar, fused[0]), (q0_bar, fused[1]), (qd0_bar, fused[2]), (status, fused[3]),
               (tq, fused[4][0]), (tqd, fused[4][1])):
    torch.testing.assert_close(a, b, rtol=0, atol=0)
  # the torch Function on the split halves: the same gradient as the fused launch
  u2 = u.clone().requires_grad_(True)
  qd2 = _t(qd0).requires_grad_(True)
  tq2, tqd2 = P.differentiable_rollout(sys_, _t(q0), qd2, u2, n_frames=5, ckpt_every=k)
  ((tq2 * qb).sum() + (tqd2 * qdb).sum()).backward()
  torch.testing.assert_close(u2.grad, fused[0], rtol=0, atol=0)
  torch.testing.assert_close(qd2.grad, fused[2], rtol=0, atol=0)


def _lying_quadrupeds(sys_, n, seed):
  """Quadrupeds pressed into the ground (torso 0.05-0.1 m high, legs as at
  init): most envs have more than 32 active constraint rows, so every frame's
  solve takes the implicit projected-gradient path."""
  rng = np.random.default_rng(seed)
  q = sys_.init_q[None] + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))
  q[:, 2] = 0.05 + rng.uniform(0.0, 0.05, n)
  qd = 0.1 * rng.normal(size=(n, sys_.qd_size()))
  return q.astype(np.float32).astype(np.float64), qd.astype(np.float32).astype(np.float64), rng


def test_single_step_vjp_implicit_solve():
  """The reverse of a step whose constraint solve ran the implicit path (more
  than 32 active rows, A applied as J (Minv (J^T x)) + diag x) against the
  numpy reverse of the same step (oracle/adjoint.py), which differentiates the
  dense A; no env may be flagged BRAXG_ENV_NO_GRADIENT."""
  P = _P()
  from oracle.adjoint import StepAdjoint
  sys_ = load('quadruped')
  n = 32
  q, qd, rng = _lying_quadrupeds(sys_, n, 71)
  full = P.init(sys_, _t(q), _t(qd), full=True)
  torch.cuda.synchronize()
  rows = (full.con_diag.cpu().numpy() != 0).sum(-1)
  assert (rows > 32).mean() >= 0.5, rows
  act = actions(sys_, n, rng).astype(np.float32).astype(np.float64)
  qbo, qdbo = rng.normal(size=q.shape), rng.normal(size=qd.shape)
  adj = StepAdjoint(sys_)
  _, _, T = adj.forward(q, qd, act)
  adj._xr = T['s'].x_rot
  rq, rqd, ract = adj.vjp(T, qbo, qdbo)
  act_bar, q0b, qd0b, status, _ = P.rollout_grad(
      sys_, _t(q), _t(qd), _t(act[None]), _t(qbo[None]), _t(qdbo[None]), n_frames=1, ckpt_every=1)
  torch.cuda.synchronize()
  st = status.cpu().numpy()
  assert (st == 0).all(), st
  for nm, g, r in (('q', q0b, rq), ('qd', qd0b, rqd), ('act', act_bar[0], ract)):
    e = _rel(g.cpu().numpy(), r)
    big, small = e[rows > 32], e[rows <= 32]
    print(f'lying quadruped (rows > 32 in {(rows > 32).sum()} of {n}) {nm}: implicit p50 {np.median(big):.2e} '
          f'max {big.max():.2e}; explicit max {small.max() if small.size else 0:.2e}')
    assert np.quantile(e, 0.95) <= 2e-3, (nm, np.sort(e)[-4:])


def test_rollout_gradient_implicit_solve_finite_differences():
  """Gradient of a 2-env-step x 2-frame rollout of the lying quadrupeds (every
  solve on the implicit path) against FP64 central differences (eps 1e-5)."""
  P = _P()
  from oracle.pipeline import Oracle
  sys_ = load('quadruped')
  n, H, F = 8, 2, 2
  q0, qd0, rng = _lying_quadrupeds(sys_, n, 72)
  u = rng.uniform(-1, 1, (H, n, sys_.act_size()))
  o = Oracle(sys_, np.float64, exact_inverse=True)

  def loss(qd0_, u_):  # -mean_t torso x-velocity + 1e-3 sum |u|^2, per env
    s = o.init(q0, qd0_)
    tot = np.zeros(n)
    for t in range(H):
      s = o.env_step(s, u_[t], F)
      tot += -s.qd[:, 0] / H
    return tot + 1e-3 * np.sum(u_ ** 2, axis=(0, 2))

  qd_bar = np.zeros((H, n, sys_.qd_size()))
  qd_bar[:, :, 0] = -1.0 / H
  act_bar, _, qd0b, status, _ = P.rollout_grad(
      sys_, _t(q0), _t(qd0), _t(u), None, _t(qd_bar), n_frames=F, ckpt_every=1)
  torch.cuda.synchronize()
  assert (status.cpu().numpy() == 0).all()
  g_u = act_bar.cpu().numpy() + 2e-3 * u
  eps = 1e-5
  fd_u = np.zeros_like(u)
  for t in range(H):
    for k in range(sys_.act_size()):
      up, um = u.copy(), u.copy()
      up[t, :, k] += eps
      um[t, :, k] -= eps
      fd_u[t, :, k] = (loss(qd0, up) - loss(qd0, um)) / (2 * eps)
  fd_qd = np.zeros((n, sys_.qd_size()))
  for k in range(sys_.qd_size()):
    a, b = qd0.copy(), qd0.copy()
    a[:, k] += eps
    b[:, k] -= eps
    fd_qd[:, k] = (loss(a, u) - loss(b, u)) / (2 * eps)
  eu = _rel(np.swapaxes(g_u, 0, 1), np.swapaxes(fd_u, 0, 1))
  eq = _rel(qd0b.cpu().numpy(), fd_qd)
  print(f'lying quadruped rollout grad vs FP64 FD: act p50 {np.median(eu):.2e} max {eu.max():.2e}; '
        f'qd0 p50 {np.median(eq):.2e} max {eq.max():.2e}')
  assert np.median(eu) <= 1e-3 and (eu <= 1e-2).mean() >= 7 / 8
  assert np.median(eq) <= 1e-3 and (eq <= 1e-2).mean() >= 7 / 8


def _humanoid_inputs(sys_, n, pose, seed):
  """Humanoid-like envs standing (the reset of the workload) or lying on the
  ground (torso turned 90 degrees about x, 0.05-0.2 m high: most envs above
  32 active rows, the implicit solve path)."""
  from brax_gb300 import workloads
  rng = np.random.default_rng(seed)
  if pose == 'standing':
    q, qd = workloads.reset(sys_, n, rng)
    q, qd = np.asarray(q, np.float64), np.asarray(qd, np.float64)
  else:
    q = sys_.init_q[None] + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))
    qd = 0.1 * rng.normal(size=(n, sys_.qd_size()))
    q[:, 3:7] = [np.cos(np.pi / 4), np.sin(np.pi / 4), 0.0, 0.0]
    q[:, 2] = rng.uniform(0.05, 0.2, n)
  return q.astype(np.float32).astype(np.float64), qd.astype(np.float32).astype(np.float64), rng


@pytest.mark.parametrize('mode', ['exact', 'newton_schulz'])
@pytest.mark.parametrize('pose', ['standing', 'lying'])
def test_humanoid_gradient(mode, pose):
  """The gradient kernel on 27 dofs (vjp_kernel<32, 32>): 4 humanoid-like
  envs, 2 env steps of 2 frames (dt 0.003), in both inverse modes (the
  reference's K = 20 Newton-Schulz inverse resets every step on this model),
  standing and lying (the implicit solve path); the model's contacts include
  the feet's capsule-capsule pair.  The gradient kernel's
  forward is the plain rollout bit for bit, the split halves give the fused
  launch's bits, and the gradient matches FP64 central differences of the
  FP64 rollout in the same mode."""
  P = _P()
  from oracle.pipeline import Oracle
  sys_ = load('humanoid_like')
  n, H, F = 4, 2, 2
  q0, qd0, rng = _humanoid_inputs(sys_, n, pose, 81)
  u = np.clip(rng.normal(0.0, 0.3, (H, n, sys_.act_size())), -1, 1).astype(np.float32).astype(np.float64)
  q_bar = rng.normal(size=(H, n, sys_.q_size())) * 1e-2
  qd_bar = rng.normal(size=(H, n, sys_.qd_size())) * 1e-2
  inv = P.CHOLESKY if mode == 'exact' else P.NEWTON_SCHULZ
  fused = P.rollout_grad(sys_, _t(q0), _t(qd0), _t(u), _t(q_bar), _t(qd_bar), n_frames=F, ckpt_every=1,
                         trajectory=True, inverse_mode=inv)
  (tq, tqd), tape = P.rollout_vjp_fwd(sys_, _t(q0), _t(qd0), _t(u), n_frames=F, ckpt_every=1, inverse_mode=inv)
  split = P.rollout_vjp_bwd(tape, _t(q_bar), _t(qd_bar))
  s0 = P.bare_state(_t(q0), _t(qd0)) if mode == 'exact' else P.init(sys_, _t(q0), _t(qd0))
  _, (rq, rqd) = P.rollout(sys_, s0, _t(u), n_frames=F, inverse_mode=inv, trajectory=True)
  full = P.init(sys_, _t(q0), _t(qd0), full=True)
  torch.cuda.synchronize()
  rows = (full.con_diag.cpu().numpy() != 0).sum(-1)
  assert (fused[3] == 0).all(), fused[3]
  if pose == 'lying':
    assert (rows > 32).any(), rows
  torch.testing.assert_close(fused[4][0], rq, rtol=0, atol=0)
  torch.testing.assert_close(fused[4][1], rqd, rtol=0, atol=0)
  for a_, b_ in zip(split[:3], fused[:3]):
    torch.testing.assert_close(a_, b_, rtol=0, atol=0)
  o = Oracle(sys_, np.float64, exact_inverse=mode == 'exact')

  def loss(q0_, qd0_, u_):
    s = o.init(q0_, qd0_)
    tot = np.zeros(n)
    for t in range(H):
      s = o.env_step(s, u_[t], F)
      tot += np.sum(q_bar[t] * s.q, -1) + np.sum(qd_bar[t] * s.qd, -1)
    return tot

  errs = {}
  fd = np.zeros((n, sys_.qd_size()))
  for j in range(sys_.qd_size()):
    fd[:, j] = _fd_median(lambda x: loss(q0, x, u), qd0, (slice(None), j))
  errs['qd0'] = _rel(fused[2].cpu().numpy(), fd)
  fdu = np.zeros(u.shape)
  for t in range(H):
    for j in range(sys_.act_size()):
      fdu[t, :, j] = _fd_median(lambda x: loss(q0, qd0, x), u, (t, slice(None), j))
  errs['act'] = _rel(np.swapaxes(fused[0].cpu().numpy(), 0, 1), np.swapaxes(fdu, 0, 1))
  for k, e in errs.items():
    print(f'humanoid-like {pose} {mode} gradient vs FP64 FD ({k}; rows {rows.tolist()}): '
          f'per env {" ".join(f"{v:.2e}" for v in e)}')
  for e in errs.values():
    assert np.median(e) <= 1e-4 and e.max() <= 1e-3


# Two free bodies whose geoms overlap by about 1 cm at the start: the contact
# between two moving geoms (mujoco.mjx's sphere / capsule pairs), without a
# plane.
_PAIR_XML = {
    'capsule_capsule': '''<mujoco model="pair_cc"><option timestep="0.005"/><worldbody>
      <body name="a" pos="0 0 1"><freejoint/><geom type="capsule" fromto="-0.2 0 0 0.2 0 0" size="0.05"/></body>
      <body name="b" pos="0 0 1.09"><freejoint/><geom type="capsule" fromto="0 -0.2 0 0 0.2 0" size="0.05"/></body>
      </worldbody></mujoco>''',
    'sphere_sphere': '''<mujoco model="pair_ss"><option timestep="0.005"/><worldbody>
      <body name="a" pos="0 0 1"><freejoint/><geom type="sphere" size="0.06"/></body>
      <body name="b" pos="0.02 0 1.11"><freejoint/><geom type="sphere" size="0.06"/></body>
      </worldbody></mujoco>''',
    'sphere_capsule': '''<mujoco model="pair_sc"><option timestep="0.005"/><worldbody>
      <body name="a" pos="0.05 0 1.1"><freejoint/><geom type="sphere" size="0.06"/></body>
      <body name="b" pos="0 0 1"><freejoint/><geom type="capsule" fromto="-0.2 0 0 0.2 0 0" size="0.05"/></body>
      </worldbody></mujoco>''',
}


@pytest.mark.parametrize('mode', ['exact', 'newton_schulz'])
@pytest.mark.parametrize('pair', sorted(_PAIR_XML))
def test_two_geom_contact_gradient(pair, mode):
  """The reverse of a contact between two moving geoms (brax/contact.py:28-67
  with mujoco.mjx's sphere-sphere, sphere-capsule and capsule-capsule
  primitives; both links' point Jacobians in the rows, constraint.py:135-176):
  8 envs of two overlapping free bodies, positions and orientations jittered,
  2 env steps of 2 frames, against FP64 central differences of the FP64
  rollout (the median of three step sizes); the gradient kernel's forward is
  the plain rollout bit for bit.  Bar: median env within 1e-3, every env
  within 1e-2: where the first frame's projected-gradient solve stops at a
  different iteration in FP32 than in FP64 (sphere-capsule env 4: 124
  against 53 matvecs, the stopping test near the tolerance) the two
  gradients are of different branches (measured 4e-3 there, <= 6e-4
  elsewhere)."""
  P = _P()
  from brax_gb300 import mjcf
  from oracle.pipeline import Oracle
  sys_ = mjcf.loads(_PAIR_XML[pair])
  n, H, F = 8, 2, 2
  rng = np.random.default_rng(91)
  q0 = np.tile(sys_.init_q, (n, 1)).astype(np.float64)
  for b in range(2):  # free joint b: position q[7b:7b+3], quaternion q[7b+3:7b+7]
    q0[:, 7 * b:7 * b + 3] += rng.uniform(-0.01, 0.01, (n, 3))
    quat = q0[:, 7 * b + 3:7 * b + 7] + rng.uniform(-0.05, 0.05, (n, 4))
    q0[:, 7 * b + 3:7 * b + 7] = quat / np.linalg.norm(quat, axis=1, keepdims=True)
  qd0 = 0.1 * rng.normal(size=(n, sys_.qd_size()))
  q0, qd0 = q0.astype(np.float32).astype(np.float64), qd0.astype(np.float32).astype(np.float64)
  u = np.zeros((H, n, 0))
  q_bar = rng.normal(size=(H, n, sys_.q_size()))
  qd_bar = rng.normal(size=(H, n, sys_.qd_size()))
  inv = P.CHOLESKY if mode == 'exact' else P.NEWTON_SCHULZ
  fused = P.rollout_grad(sys_, _t(q0), _t(qd0), _t(u), _t(q_bar), _t(qd_bar), n_frames=F, ckpt_every=1,
                         trajectory=True, inverse_mode=inv)
  s0 = P.bare_state(_t(q0), _t(qd0)) if mode == 'exact' else P.init(sys_, _t(q0), _t(qd0))
  _, (rq, rqd) = P.rollout(sys_, s0, _t(u), n_frames=F, inverse_mode=inv, trajectory=True)
  full = P.init(sys_, _t(q0), _t(qd0), full=True)
  torch.cuda.synchronize()
  rows = (full.con_diag.cpu().numpy() != 0).sum(-1)
  assert (rows > 0).sum() >= n // 2, rows  # the pair touches in most envs
  assert (fused[3] == 0).all(), fused[3]
  torch.testing.assert_close(fused[4][0], rq, rtol=0, atol=0)
  torch.testing.assert_close(fused[4][1], rqd, rtol=0, atol=0)
  o = Oracle(sys_, np.float64, exact_inverse=mode == 'exact')

  def loss(q0_, qd0_):
    s = o.init(q0_, qd0_)
    tot = np.zeros(n)
    for t in range(H):
      s = o.env_step(s, u[t], F)
      tot += np.sum(q_bar[t] * s.q, -1) + np.sum(qd_bar[t] * s.qd, -1)
    return tot

  errs = {}
  for which, (x0, got) in enumerate(((q0, fused[1]), (qd0, fused[2]))):
    fd = np.zeros(x0.shape)
    f = (lambda x: loss(x, qd0)) if which == 0 else (lambda x: loss(q0, x))
    for j in range(x0.shape[1]):
      fd[:, j] = _fd_median(f, x0, (slice(None), j))
    errs[['q0', 'qd0'][which]] = _rel(got.cpu().numpy(), fd)
  for k, e in errs.items():
    print(f'{pair} {mode} gradient vs FP64 FD ({k}; rows {rows.tolist()}): per env {" ".join(f"{v:.2e}" for v in e)}')
  for e in errs.values():
    assert np.median(e) <= 1e-3 and e.max() <= 1e-2


@pytest.mark.parametrize('mode', ['exact', 'newton_schulz'])
def test_box_plane_gradient(mode):
  """The reverse of mjx's plane-box contact (the slot's manifold vertex, a
  point of the box, against the plane; the vertex choice piecewise
  constant): 16 randomly oriented boxes with their lowest vertex 2-6 mm into
  the plane, 2 env steps of 2 frames, against FP64 central differences of
  the FP64 rollout on the envs where those are determined."""
  P = _P()
  from brax_gb300 import mjcf
  from oracle.pipeline import Oracle
  from tests.test_gpu_parity import BOX_XML
  sys_ = mjcf.loads(BOX_XML)
  n, H, F = 16, 2, 2
  rng = np.random.default_rng(93)
  qv = rng.normal(size=(n, 4))
  qv /= np.linalg.norm(qv, axis=1, keepdims=True)
  h = np.array([0.2, 0.15, 0.1])
  verts = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]) * h
  q0 = np.zeros((n, 7))
  for e in range(n):  # the lowest vertex's height sets the box's
    w, x, y, z = qv[e]
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    low = (verts @ R.T)[:, 2].min()
    q0[e] = [rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5), -low - rng.uniform(0.002, 0.006), w, x, y, z]
  qd0 = 0.05 * rng.normal(size=(n, 6))
  q0, qd0 = q0.astype(np.float32).astype(np.float64), qd0.astype(np.float32).astype(np.float64)
  u = np.zeros((H, n, 0))
  q_bar = rng.normal(size=(H, n, 7))
  qd_bar = rng.normal(size=(H, n, 6))
  inv = P.CHOLESKY if mode == 'exact' else P.NEWTON_SCHULZ
  fused = P.rollout_grad(sys_, _t(q0), _t(qd0), _t(u), _t(q_bar), _t(qd_bar), n_frames=F, ckpt_every=1,
                         trajectory=True, inverse_mode=inv)
  s0 = P.bare_state(_t(q0), _t(qd0)) if mode == 'exact' else P.init(sys_, _t(q0), _t(qd0))
  _, (rq, rqd) = P.rollout(sys_, s0, _t(u), n_frames=F, inverse_mode=inv, trajectory=True)
  full = P.init(sys_, _t(q0), _t(qd0), full=True)
  torch.cuda.synchronize()
  rows = (full.con_diag.cpu().numpy() != 0).sum(-1)
  assert (rows > 0).all(), rows
  assert (fused[3] == 0).all(), fused[3]
  torch.testing.assert_close(fused[4][0], rq, rtol=0, atol=0)
  torch.testing.assert_close(fused[4][1], rqd, rtol=0, atol=0)
  o = Oracle(sys_, np.float64, exact_inverse=mode == 'exact')

  def loss(q0_, qd0_):
    s = o.init(q0_, qd0_)
    tot = np.zeros(n)
    for t in range(H):
      s = o.env_step(s, u[t], F)
      tot += np.sum(q_bar[t] * s.q, -1) + np.sum(qd_bar[t] * s.qd, -1)
    return tot

  # a box on one corner is often near the solve's stopping test: its loss has
  # kinks below 1e-5, and differences at 1e-5, 1e-6 and 1e-7 disagree; the
  # gradient is checked on the envs whose three differences agree to 1e-3
  errs, det = {}, np.ones(n, bool)
  for which, (x0, got) in enumerate(((q0, fused[1]), (qd0, fused[2]))):
    f = (lambda x: loss(x, qd0)) if which == 0 else (lambda x: loss(q0, x))
    est = []
    for eps in (1e-5, 1e-6, 1e-7):
      cols = []
      for jj in range(x0.shape[1]):
        a_, b_ = x0.copy(), x0.copy()
        a_[:, jj] += eps
        b_[:, jj] -= eps
        cols.append((f(a_) - f(b_)) / (2 * eps))
      est.append(np.stack(cols, 1))
    est = np.stack(est)
    fd = np.median(est, 0)
    spread = (est.max(0) - est.min(0)).max(-1) / np.maximum(np.abs(fd).max(-1), 1e-6)
    det &= spread <= 1e-3
    errs[['q0', 'qd0'][which]] = _rel(got.cpu().numpy(), fd)
  for k_, e in errs.items():
    print(f'box-plane {mode} gradient vs FP64 FD ({k_}; determined envs {det.astype(int).tolist()}): '
          f'per env {" ".join(f"{v:.2e}" for v in e)}')
  assert det.sum() >= 3, det
  for e in errs.values():  # as the two-body pairs: FP32 and FP64 solves may stop apart
    assert np.median(e[det]) <= 1e-3 and e[det].max() <= 1e-2
