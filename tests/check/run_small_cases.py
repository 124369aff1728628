"""Small cases (<= 64 envs) of every kernel path, for the checked-build test:
single-model init / step (both inverse modes, state caches carried, two
frames), the implicit solve (lying humanoid-like models), the fused env step,
an uneven batch and rollout gradients (including the implicit solve).
Writes every output to the .npz named on the command line.  Which library
runs is chosen by BRAXG_CHECK (brax_gb300._native)."""

import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from brax_gb300 import _native as N  # noqa: E402
from brax_gb300 import envs, pipeline as P, workloads as W  # noqa: E402
from brax_gb300.batch import Batch  # noqa: E402
from tests.parity_util import actions, load, seeded_inputs  # noqa: E402


def main(out_path):
  dev = torch.device('cuda')
  t = lambda x: torch.as_tensor(np.asarray(x, np.float32), device=dev)
  out = {'checked': np.array(N.CHECKED)}
  rng = np.random.default_rng(5)
  for name in ('chain3', 'quadruped', 'humanoid_like'):
    sys_ = load(name)
    n = 48
    q, qd = seeded_inputs(sys_, n, 3)
    for mode in (P.NEWTON_SCHULZ, P.CHOLESKY):
      s = P.init(sys_, t(q), t(qd))
      for k in range(3):
        s = P.step(sys_, s, t(actions(sys_, n, rng)), n_frames=2, inverse_mode=mode, full=(k == 2))
      torch.cuda.synchronize()
      for f in ('q', 'qd', 'mass_mx_inv', 'status', 'con_jac'):
        out[f'{name}_{mode}_{f}'] = getattr(s, f).cpu().numpy()
  # the implicit solve: lying humanoid-like models (more than 32 active rows)
  sys_ = load('humanoid_like')
  n = 32
  q = sys_.init_q[None] + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))
  q[:, 3:7] = [np.cos(np.pi / 4), np.sin(np.pi / 4), 0.0, 0.0]
  q[:, 2] = rng.uniform(0.05, 0.2, n)
  qd = 0.1 * rng.normal(size=(n, sys_.qd_size()))
  s = P.init(sys_, t(q), t(qd))
  s = P.step(sys_, s, t(actions(sys_, n, rng)), n_frames=2, inverse_mode=P.CHOLESKY, full=True)
  torch.cuda.synchronize()
  out['lying_q'], out['lying_status'] = s.q.cpu().numpy(), s.status.cpu().numpy()
  out['lying_rows'] = (s.con_diag.cpu().numpy() != 0).sum(-1)
  # fused env step
  env = envs.Locomotion(load('quadruped'), device=dev)
  g = torch.Generator(device=dev)
  g.manual_seed(9)
  st = env.reset(32, generator=g)
  for k in range(3):
    st = env.step(st, torch.rand(32, env.action_size, device=dev, generator=g) * 2 - 1)
  torch.cuda.synchronize()
  out['env_obs'], out['env_status'] = st.obs.cpu().numpy(), st.pipeline_state.status.cpu().numpy()
  # uneven batch
  mix = [(W.chain(4), 16, 1), (W.chain(20), 16, 1), (load('quadruped'), 16, 5), (load('humanoid_like'), 16, 5)]
  b = Batch([m[0] for m in mix], [m[1] for m in mix], [m[2] for m in mix], device=dev)
  qs, qds, acts = [], [], []
  for s_, n_, _ in mix:
    q_, qd_ = W.reset(s_, n_, rng)
    qs.append(q_)
    qds.append(qd_)
    acts.append(np.stack([W.actions(s_, n_, rng) for _ in range(3)]).astype(np.float32))
  s0 = b.init(b.concat(qs, 'q'), b.concat(qds, 'qd'))
  s1, _ = b.rollout(s0, b.concat_steps(acts, 'act'))
  torch.cuda.synchronize()
  out['batch_q'], out['batch_status'] = s1.q.cpu().numpy(), s1.status.cpu().numpy()
  # gradients: standing and lying quadrupeds (explicit and implicit solves)
  sys_ = load('quadruped')
  n = 16
  q, qd = seeded_inputs(sys_, n, 4)
  q[n // 2:, 2] = 0.05 + rng.uniform(0.0, 0.05, n - n // 2)
  u = t(rng.uniform(-1, 1, (4, n, sys_.act_size())))
  qdb = t(rng.normal(size=(4, n, sys_.qd_size())))
  ab, q0b, qd0b, st, _ = P.rollout_grad(sys_, t(q), t(qd), u, None, qdb, n_frames=2, ckpt_every=2)
  torch.cuda.synchronize()
  out['grad_act'], out['grad_qd0'], out['grad_status'] = ab.cpu().numpy(), qd0b.cpu().numpy(), st.cpu().numpy()
  np.savez(out_path, **out)


if __name__ == '__main__':
  main(sys.argv[1])
