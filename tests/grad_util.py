"""CPU side of the rollout-gradient checks (process-pool workers; no torch).

reverse_along: the FP64 reverse (oracle/adjoint.py StepAdjoint) of a rollout
chained backwards along a given trajectory: every env step is re-run in FP64
from the given state at its start (the GPU's state after the previous env
step), its frames taped, and their reverses chained, so the result is the
FP64 gradient of the same linearisation the GPU differentiated.

tail_fd: FP64 central differences of the APG loss's tail (env steps t..H-1)
with respect to the action of env step t, from a given state at step t.
"""

from __future__ import annotations

import numpy as np


def _sys(name):
  from brax_gb300 import mjcf
  return mjcf.load_asset(name)


def reverse_along(args):
  """(name, q_start [H, nq], qd_start [H, nv], act [H, nu], q_bar [H, nq],
  qd_bar [H, nv], n_frames, forced) for one env -> (act_bar [H, nu], q0_bar,
  qd0_bar, gap [H], mismatch [H]).  q_start[s] / qd_start[s] is the state at
  the start of env step s.  forced[s][f] = (iterations, active rows, step
  sizes) of another implementation's projected-gradient solve in frame f of
  env step s (None: the FP64 solve's own decisions); the FP64 re-run then
  takes that branch, and mismatch[s] records a frame whose FP64 active row
  count differs from the given one (a contact within rounding of the
  threshold).  gap[s] is the closest call, relative to the compared values'
  size, of any projected-gradient decision the FP64 re-run of env step s took
  itself (below about 1e-6 the same decision is a tie in FP32)."""
  from oracle.adjoint import StepAdjoint
  name, q_start, qd_start, act, q_bar, qd_bar, n_frames, forced = args
  sys_ = _sys(name)
  adj = StepAdjoint(sys_)
  H = act.shape[0]
  qb = q_bar[H - 1][None].astype(np.float64)
  qdb = qd_bar[H - 1][None].astype(np.float64)
  act_bar = np.zeros(act.shape)
  gaps = np.full(H, np.inf)
  mismatch = np.zeros(H, bool)
  for s in range(H - 1, -1, -1):
    q = q_start[s][None].astype(np.float64)
    qd = qd_start[s][None].astype(np.float64)
    a = act[s][None].astype(np.float64)
    tapes = []
    for f in range(n_frames):
      fr = None if forced is None else forced[s][f]
      adj.force = None if fr is None else (fr[0], fr[2])
      qn, qdn, T = adj.forward(q, qd, a)
      adj.force = None
      if fr is not None and int(np.count_nonzero(T['s'].con_diag[0])) != fr[1]:
        mismatch[s] = True
      tapes.append((T, T['s'].x_rot))
      gaps[s] = min(gaps[s], float(T['pg_gap'][0]))
      q, qd = qn, qdn
    for T, xr in reversed(tapes):
      adj._xr = xr
      qb, qdb, ab = adj.vjp(T, qb, qdb)
      act_bar[s] += ab[0]
    if s > 0:
      qb = qb + q_bar[s - 1][None]
      qdb = qdb + qd_bar[s - 1][None]
  return act_bar, qb[0], qdb[0], gaps, mismatch


def tail_fd(args):
  """(name, q_t [nq], qd_t [nv], act [H - t, nu], n_frames, eps_list, coords,
  horizon[, forced]) -> ({eps: [len(coords)]} central differences of -mean
  torso x-velocity over the env steps t..H-1 (each 1/horizon weighted) w.r.t.
  act[0, k] for k in coords, the FP64 tail trajectory of the unperturbed
  actions (q, qd after each env step), whether every frame's FP64 active
  row count matched the forced tape's, and the closest projection call of
  the unperturbed tail's solves (relative; below about 1e-5 the sign of that
  component is a tie at FP32 resolution)).  With `forced` ([H - t][n_frames]
  (iterations, active rows, step sizes) of another implementation's
  projected-gradient solves), every rollout of the difference takes those
  solver decisions: the difference quotient of the same branch."""
  from oracle.pipeline import Oracle
  name, q_t, qd_t, act, n_frames, eps_list, coords, horizon = args[:8]
  forced = args[8] if len(args) > 8 else None
  sys_ = _sys(name)
  o = Oracle(sys_, np.float64, exact_inverse=True)
  L = act.shape[0]
  # one batch: the unperturbed rollout, then +eps / -eps for every coordinate and eps
  rows = [act]
  for eps in eps_list:
    for k in coords:
      for sgn in (1.0, -1.0):
        a = act.copy()
        a[0, k] += sgn * eps
        rows.append(a)
  B = len(rows)
  acts = np.stack(rows, axis=1).astype(np.float64)  # [L, B, nu]
  q = np.repeat(q_t[None].astype(np.float64), B, 0)
  qd = np.repeat(qd_t[None].astype(np.float64), B, 0)
  loss = np.zeros(B)
  traj_q, traj_qd = [], []
  rows_ok = True
  proj_gap = np.inf
  if forced is None:
    s = o.init(q, qd)
    for j in range(L):
      s = o.env_step(s, acts[j], n_frames)
      loss += -s.qd[:, 0] / horizon
      traj_q.append(s.q[0].copy())
      traj_qd.append(s.qd[0].copy())
  else:
    from oracle.adjoint import StepAdjoint
    adj = StepAdjoint(sys_)
    for j in range(L):
      for f in range(n_frames):
        iters, rows, steps = forced[j][f]
        adj.force = (iters, steps)
        try:
          with np.errstate(all='ignore'):
            q, qd, T = adj.forward(q, qd, acts[j])
        except np.linalg.LinAlgError:  # a forced solve off its branch threw the state off
          rows_ok = False
          break
        finally:
          adj.force = None
        if not (np.count_nonzero(T['s'].con_diag, axis=1) == rows).all():
          rows_ok = False  # the tape belongs to another active set: forcing it means nothing
          break
        proj_gap = min(proj_gap, float(T['proj_gap'][0]))
      if not rows_ok:
        break
      loss += -qd[:, 0] / horizon
      traj_q.append(q[0].copy())
      traj_qd.append(qd[0].copy())
    if not rows_ok:
      nan = {eps: np.full(len(coords), np.nan) for eps in eps_list}
      return nan, np.full((L, q.shape[1]), np.nan), np.full((L, qd.shape[1]), np.nan), False, proj_gap
  out, i = {}, 1
  for eps in eps_list:
    fd = np.zeros(len(coords))
    for c in range(len(coords)):
      fd[c] = (loss[i] - loss[i + 1]) / (2 * eps)
      i += 2
    out[eps] = fd
  return out, np.array(traj_q), np.array(traj_qd), rows_ok, proj_gap
