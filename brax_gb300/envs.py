"""Locomotion env step fused with the physics (braxg_env_rollout).

Mirrors the env API brax trains on: ``reset(...) -> State`` and
``step(state, action) -> State`` of brax/envs/ant.py:205-279, wrapped by
EpisodeWrapper and AutoResetWrapper (brax/envs/wrappers/training.py:75-158)
as ``wrap_for_training`` composes them.  The task (forward reward, healthy
reward, control cost, healthy-z termination, obs = q[2:] ++ qd) runs in the
same kernel launch as the n_frames pipeline steps; done envs return to their
episode's first pipeline state inside that launch.

Arrays are torch CUDA tensors with a leading env axis.  Random resets use a
torch generator (the reference's jax.random stream is not reproduced).
"""

from __future__ import annotations

import ctypes
import dataclasses
from typing import Dict, Optional

import torch

from brax_gb300 import _native as N
from brax_gb300 import pipeline as P


@dataclasses.dataclass
class State:
  """brax.envs.base.State: pipeline_state, obs, reward, done, metrics, info."""
  pipeline_state: P.State
  obs: torch.Tensor
  reward: torch.Tensor
  done: torch.Tensor
  metrics: Dict[str, torch.Tensor]
  info: Dict[str, torch.Tensor]


class Locomotion:
  """brax/envs/ant.py's task on a System whose link 0 is the torso (the
  packaged quadruped by default), with brax's training wrappers fused in."""

  def __init__(self, sys, ctrl_cost_weight: float = 0.5, healthy_reward: float = 1.0,
               terminate_when_unhealthy: bool = True, healthy_z_range=(0.2, 1.0),
               reset_noise_scale: float = 0.1,
               exclude_current_positions_from_observation: bool = True, n_frames: int = 5,
               episode_length: int = 1000, action_repeat: int = 1, auto_reset: bool = True,
               inverse_mode: int = P.CHOLESKY, randomization: Optional[dict] = None, device=None):
    self.sys = sys
    self.model = P.model_for(sys, device)
    self.device = self.model.device
    self.n_frames = int(n_frames)
    self.reset_noise_scale = float(reset_noise_scale)
    self.inverse_mode = int(inverse_mode)
    # per-env System parameters (DomainRandomizationVmapWrapper,
    # brax/envs/wrappers/training.py:223-260): pipeline.randomize(...)
    self.randomization = randomization
    self.exclude = bool(exclude_current_positions_from_observation)
    self.task = N.Task(float(ctrl_cost_weight), float(healthy_reward), float(healthy_z_range[0]),
                       float(healthy_z_range[1]), int(terminate_when_unhealthy), int(self.exclude),
                       int(episode_length), int(action_repeat), int(auto_reset))

  @property
  def dt(self) -> float:  # PipelineEnv.dt
    return self.n_frames * self.sys.dt

  @property
  def observation_size(self) -> int:
    return self.model.nq - (2 if self.exclude else 0) + self.model.nv

  @property
  def action_size(self) -> int:
    return self.model.nu

  def _obs(self, ps: P.State) -> torch.Tensor:  # ant.py:271-279
    q = ps.q[:, 2:] if self.exclude else ps.q
    return torch.cat([q, ps.qd], dim=-1)

  def reset(self, n_env: int, generator: Optional[torch.Generator] = None, q=None, qd=None) -> State:
    """ant.py:205-231 for n_env envs (q / qd override the sampled reset)."""
    m = self.model
    s = self.reset_noise_scale
    if q is None:
      init_q = torch.tensor(self.sys.init_q, dtype=torch.float32, device=self.device)
      q = init_q + (torch.rand(n_env, m.nq, device=self.device, generator=generator) * 2 - 1) * s
    if qd is None:
      qd = s * torch.randn(n_env, m.nv, device=self.device, generator=generator)
    ps = P.init(self.sys, q.to(self.device, torch.float32), qd.to(self.device, torch.float32),
                randomization=self.randomization)
    z = lambda: torch.zeros(n_env, dtype=torch.float32, device=self.device)
    info = {'steps': z(), 'truncation': z(), 'first_q': ps.q.clone(), 'first_qd': ps.qd.clone(),
            'first_mass_mx_inv': ps.mass_mx_inv.clone(), 'first_obs': self._obs(ps)}
    metrics = {k: z() for k in N.METRICS}
    return State(ps, self._obs(ps), z(), z(), metrics, info)

  def rollout(self, state: State, act_seq: torch.Tensor, donate: bool = False):
    """len(act_seq) env steps in one launch; returns (State after the last,
    rewards [n_steps, n], dones [n_steps, n])."""
    m = self.model
    ps = state.pipeline_state
    n = ps.q.shape[0]
    act_seq = act_seq.to(self.device, torch.float32).contiguous()
    if act_seq.dim() == 2:
      act_seq = act_seq[None]
    if act_seq.shape[1:] != (n, m.nu):
      raise ValueError(f'act_seq must be (n_steps, {n}, {m.nu})')
    n_steps = act_seq.shape[0]
    out = ps if donate else P._alloc(m, n, False, self.device, ps.cache is not None)
    f = lambda *sh: torch.empty(*sh, dtype=torch.float32, device=self.device)
    obs, rewards, dones, met = f(n, self.observation_size), f(n_steps, n), f(n_steps, n), f(n, len(N.METRICS))
    steps = state.info['steps'].clone()
    trunc = state.info['truncation'].clone()
    last_done = state.done.clone()
    io = N.EnvIO(obs.data_ptr(), rewards.data_ptr(), dones.data_ptr(), met.data_ptr(), steps.data_ptr(),
                 trunc.data_ptr(), last_done.data_ptr(), state.info['first_q'].data_ptr(),
                 state.info['first_qd'].data_ptr(), state.info['first_mass_mx_inv'].data_ptr())
    cin, cout = P._cstate(ps), P._cstate(out)
    dr, _keep = P._randomization(m, n, self.randomization)
    stream = torch.cuda.current_stream(self.device).cuda_stream
    N.check(N.lib().braxg_env_rollout(m.handle, ctypes.c_void_p(stream), n, n_steps, self.n_frames,
                                      act_seq.data_ptr() if m.nu else None, ctypes.byref(cin),
                                      ctypes.byref(cout), ctypes.byref(self.task), ctypes.byref(io),
                                      ctypes.byref(P._opts(self.inverse_mode, 0, 0, dr=dr))),
            'braxg_env_rollout')
    info = dict(state.info, steps=steps, truncation=trunc)
    metrics = {k: met[:, i] for i, k in enumerate(N.METRICS)}
    return State(out, obs, rewards[-1], last_done, metrics, info), rewards, dones

  def step(self, state: State, action: torch.Tensor) -> State:
    """One env step: AutoResetWrapper(EpisodeWrapper(task)).step."""
    return self.rollout(state, action[None] if action.dim() == 2 else action)[0]
