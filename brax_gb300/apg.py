"""Analytic policy gradients through the hand-written adjoint.

The training step of brax/training/agents/apg/train.py:179-236 in torch: a
closed-loop policy acts on the observation for ``horizon`` env steps, the loss
is the negative mean reward, and the gradient flows back through every env
step to the policy parameters.  Each env step is ``EnvStep`` — a
``torch.autograd.Function`` whose forward is the forward half of the
gradient kernel for that env step (braxg_rollout_vjp_fwd: exact mass-matrix
inverse, its frame snapshots kept) and whose backward is the reverse half
(braxg_rollout_vjp_bwd) — so torch's autograd chains the physics adjoint with
the policy network's backward, as ``jax.grad`` chains them through
``lax.scan`` in the reference.

The reward is the locomotion task's (brax/envs/ant.py:238-262): forward
velocity of the torso (q[0] is its x position for a free-root model) over the
env step's duration, a healthy reward while the torso height is inside the
range, minus the control cost.  Observations are q[2:] ++ qd
(brax/envs/ant.py:271-279); there is no observation normaliser.
"""

from __future__ import annotations

import dataclasses
from typing import Callable, List, Optional

import torch

from brax_gb300 import pipeline as P


class EnvStep(torch.autograd.Function):
  """(q, qd, act) -> (q', qd') for one env step of n_frames pipeline steps."""

  @staticmethod
  def forward(ctx, q, qd, act, sys, n_frames):
    # one launch, the forward half of the gradient kernel: the env step's
    # frame snapshots stay in a workspace for the backward, which then runs
    # only the reverse (an exact-inverse step reads only q and qd of its
    # input, so no init launch precedes it)
    (tq, tqd), ctx.tape = P.rollout_vjp_fwd(sys, q.detach(), qd.detach(), act.detach()[None],
                                            n_frames=n_frames, ckpt_every=1, resident_segments=1)
    return tq[0], tqd[0]

  @staticmethod
  def backward(ctx, gq, gqd):
    act_bar, q_bar, qd_bar, _ = P.rollout_vjp_bwd(ctx.tape, None if gq is None else gq[None],
                                                  None if gqd is None else gqd[None])
    return q_bar, qd_bar, act_bar[0], None, None


def env_step(sys, q, qd, act, n_frames: int):
  """One env step, differentiable when a gradient is being taken (else a
  plain step launch)."""
  if torch.is_grad_enabled() and any(t.requires_grad for t in (q, qd, act)):
    return EnvStep.apply(q, qd, act, sys, n_frames)
  out = P.step(sys, P.bare_state(q, qd), act, n_frames=n_frames, inverse_mode=P.CHOLESKY)
  return out.q, out.qd


@dataclasses.dataclass
class Config:
  """The APG hyper-parameters of brax/training/agents/apg/train.py:47-80 that
  this loop uses."""
  num_envs: int = 256
  horizon: int = 32
  n_frames: int = 5
  learning_rate: float = 1e-3
  max_gradient_norm: float = 1e9
  ctrl_cost_weight: float = 0.5
  healthy_reward: float = 1.0
  healthy_z_range: tuple = (0.2, 1.0)
  reset_noise_scale: float = 0.1


def make_policy(obs_size: int, act_size: int, hidden=(64, 64), device=None) -> torch.nn.Module:
  """An MLP with a tanh output (actions in [-1, 1])."""
  layers: List[torch.nn.Module] = []
  d = obs_size
  for h in hidden:
    layers += [torch.nn.Linear(d, h), torch.nn.SiLU()]
    d = h
  layers += [torch.nn.Linear(d, act_size), torch.nn.Tanh()]
  return torch.nn.Sequential(*layers).to(device)


def loss(sys, policy: Callable, q0, qd0, cfg: Config):
  """-mean(reward) over cfg.horizon env steps from (q0, qd0) (train.py:187-196)."""
  dt = cfg.n_frames * sys.dt
  q, qd = q0, qd0
  rewards = []
  for _ in range(cfg.horizon):
    obs = torch.cat([q[:, 2:], qd], dim=-1)
    act = policy(obs)
    q2, qd2 = env_step(sys, q, qd, act, cfg.n_frames)
    z = q2[:, 2]
    healthy = ((z >= cfg.healthy_z_range[0]) & (z <= cfg.healthy_z_range[1])).to(q2.dtype)
    reward = (q2[:, 0] - q[:, 0]) / dt + cfg.healthy_reward * healthy - cfg.ctrl_cost_weight * (act * act).sum(-1)
    rewards.append(reward)
    q, qd = q2, qd2
  return -torch.stack(rewards).mean()


def train(sys, cfg: Config = Config(), iterations: int = 10, seed: int = 0,
          policy: Optional[torch.nn.Module] = None, device=None):
  """Runs APG updates (Adam, gradient clipping as train.py:158-162, 199-207);
  returns (policy, losses)."""
  device = torch.device('cuda') if device is None else torch.device(device)
  gen = torch.Generator(device=device).manual_seed(seed)
  nq, nv, nu = sys.q_size(), sys.qd_size(), sys.act_size()
  if policy is None:
    torch.manual_seed(seed)
    policy = make_policy(nq - 2 + nv, nu, device=device)
  opt = torch.optim.Adam(policy.parameters(), lr=cfg.learning_rate)
  init_q = torch.tensor(sys.init_q, dtype=torch.float32, device=device)
  s = cfg.reset_noise_scale
  losses = []
  for _ in range(iterations):
    q0 = init_q + (torch.rand(cfg.num_envs, nq, device=device, generator=gen) * 2 - 1) * s
    qd0 = s * torch.randn(cfg.num_envs, nv, device=device, generator=gen)
    opt.zero_grad()
    l = loss(sys, policy, q0, qd0, cfg)
    l.backward()
    torch.nn.utils.clip_grad_norm_(policy.parameters(), max(cfg.max_gradient_norm, 1e-12))
    opt.step()
    losses.append(float(l.detach()))
  return policy, losses
