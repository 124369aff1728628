"""APG through the hand-written adjoint (brax_gb300/apg.py): autograd chained
over per-env-step adjoint launches gives the gradient of the whole-rollout
adjoint for the same open-loop actions, and a few closed-loop training
iterations run with finite losses and move the policy."""

import numpy as np
import pytest

from tests.parity_util import load, seeded_inputs

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _setup():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import apg
  from brax_gb300 import pipeline
  return apg, pipeline


def test_chained_env_steps_match_rollout_adjoint():
  apg, P = _setup()
  sys_ = load('quadruped')
  n, H = 16, 4
  q0, qd0 = seeded_inputs(sys_, n, 71)
  rng = np.random.default_rng(72)
  u = torch.tensor(rng.uniform(-1, 1, (H, n, sys_.act_size())), dtype=torch.float32, device='cuda')
  w = torch.tensor(rng.normal(size=(H, n, sys_.qd_size())), dtype=torch.float32, device='cuda')
  # whole rollout
  u1 = u.clone().requires_grad_(True)
  qd1 = torch.tensor(qd0, dtype=torch.float32, device='cuda').requires_grad_(True)
  _, tqd = P.differentiable_rollout(sys_, torch.tensor(q0, dtype=torch.float32, device='cuda'), qd1, u1,
                                    n_frames=5, ckpt_every=2)
  (tqd * w).sum().backward()
  # the same as a chain of one-env-step functions
  u2 = u.clone().requires_grad_(True)
  qd2 = torch.tensor(qd0, dtype=torch.float32, device='cuda').requires_grad_(True)
  q, qd = torch.tensor(q0, dtype=torch.float32, device='cuda'), qd2
  loss = 0.0
  for t in range(H):
    q, qd = apg.env_step(sys_, q, qd, u2[t], 5)
    loss = loss + (qd * w[t]).sum()
  loss.backward()
  torch.cuda.synchronize()
  for a, b in ((u2.grad, u1.grad), (qd2.grad, qd1.grad)):
    rel = (a - b).abs().max() / b.abs().max().clamp_min(1e-6)
    assert float(rel) <= 1e-5, float(rel)


def test_apg_training_iterations():
  apg, _ = _setup()
  sys_ = load('quadruped')
  cfg = apg.Config(num_envs=64, horizon=8)
  policy = apg.make_policy(sys_.q_size() - 2 + sys_.qd_size(), sys_.act_size(), device='cuda')
  before = [p.detach().clone() for p in policy.parameters()]
  policy, losses = apg.train(sys_, cfg, iterations=3, policy=policy)
  assert len(losses) == 3 and np.isfinite(losses).all()
  moved = sum(float((p.detach() - b).abs().sum()) for p, b in zip(policy.parameters(), before))
  assert moved > 0
