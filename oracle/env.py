"""CPU restatement of brax's locomotion env step with its training wrappers.

TEST INFRASTRUCTURE ONLY: the checker for the fused env step
(braxg_env_rollout); nothing in the product imports it.

Restates, for a batch of envs (numpy, FP32 or FP64 through oracle.pipeline):
  brax/envs/ant.py:233-279          Ant.step / _get_obs (forward reward from the
                                    torso's x displacement over dt, healthy
                                    reward, control cost, healthy-z done)
  brax/envs/wrappers/training.py:97-125   EpisodeWrapper.step (step count,
                                    done at episode_length, truncation)
  brax/envs/wrappers/training.py:131-158  AutoResetWrapper.step (step count
                                    reset after a done, return to the first
                                    pipeline state)
composed as AutoResetWrapper(EpisodeWrapper(task)), brax's training order
(brax/envs/wrappers/training.py:32-72, wrap_for_training).
"""

from __future__ import annotations

import dataclasses
from typing import Dict

import numpy as np

from oracle.pipeline import Oracle
from oracle.pipeline import State as PState

METRICS = ('reward_forward', 'reward_survive', 'reward_ctrl', 'reward_contact', 'x_position',
           'y_position', 'distance_from_origin', 'x_velocity', 'y_velocity', 'forward_reward')


@dataclasses.dataclass
class TaskParams:
  ctrl_cost_weight: float = 0.5
  healthy_reward: float = 1.0
  healthy_z_range: tuple = (0.2, 1.0)
  terminate_when_unhealthy: bool = True
  exclude_current_positions: bool = True
  episode_length: int = 1000
  action_repeat: int = 1
  auto_reset: bool = True


@dataclasses.dataclass
class EnvState:
  pipeline_state: PState
  obs: np.ndarray
  reward: np.ndarray
  done: np.ndarray
  metrics: Dict[str, np.ndarray]
  steps: np.ndarray
  truncation: np.ndarray
  first: PState


class LocomotionOracle:
  """The env step of brax/envs/ant.py for any model whose link 0 is the torso."""

  def __init__(self, oracle: Oracle, n_frames: int, task: TaskParams):
    self.o = oracle
    self.n_frames = n_frames
    self.task = task
    self.t = oracle.dt_.type
    self.dt = self.t(n_frames) * self.t(oracle.sys.dt)  # PipelineEnv.dt

  def obs(self, s: PState) -> np.ndarray:  # ant.py:271-279
    q = s.q[:, 2:] if self.task.exclude_current_positions else s.q
    return np.concatenate([q, s.qd], axis=-1)

  def reset(self, q: np.ndarray, qd: np.ndarray) -> EnvState:  # ant.py:205-231 (q, qd given)
    s = self.o.init(q, qd)
    n = q.shape[0]
    z = np.zeros(n, self.o.dt_)
    return EnvState(s, self.obs(s), z.copy(), z.copy(), {k: z.copy() for k in METRICS}, z.copy(),
                    z.copy(), s)

  def _task_step(self, s0: PState, action: np.ndarray):  # ant.py:233-269
    k = self.task
    dt = self.t
    s = self.o.env_step(s0, action, self.n_frames)
    velocity = (s.x_pos[:, 0] - s0.x_pos[:, 0]) / self.dt
    forward = velocity[:, 0]
    zmin, zmax = (dt(v) for v in k.healthy_z_range)
    z = s.x_pos[:, 0, 2]
    healthy = np.where(z < zmin, dt(0), dt(1))
    healthy = np.where(z > zmax, dt(0), healthy)
    survive = (np.full_like(healthy, k.healthy_reward) if k.terminate_when_unhealthy
               else dt(k.healthy_reward) * healthy)
    ctrl = dt(k.ctrl_cost_weight) * np.sum(np.square(action.astype(dt)), axis=-1)
    reward = forward + survive - ctrl - dt(0)
    done = dt(1) - healthy if k.terminate_when_unhealthy else np.zeros_like(healthy)
    pos0 = s.x_pos[:, 0]
    metrics = dict(reward_forward=forward, reward_survive=survive, reward_ctrl=-ctrl,
                   reward_contact=np.zeros_like(forward), x_position=pos0[:, 0], y_position=pos0[:, 1],
                   distance_from_origin=np.sqrt(np.sum(pos0 * pos0, axis=-1)), x_velocity=velocity[:, 0],
                   y_velocity=velocity[:, 1], forward_reward=forward)
    return s, reward, done, metrics

  def step(self, st: EnvState, action: np.ndarray) -> EnvState:
    k = self.task
    dt = self.t
    # AutoResetWrapper.step (training.py:139-145): a new episode after a done
    steps = np.where(st.done != 0, dt(0), st.steps)
    s = st.pipeline_state
    rewards = []
    done = metrics = None
    for _ in range(k.action_repeat):  # EpisodeWrapper.step (training.py:98-104)
      s, r, done, metrics = self._task_step(s, action)
      rewards.append(r)
    reward = np.sum(np.stack(rewards), axis=0)
    steps = steps + dt(k.action_repeat)
    over = steps >= dt(k.episode_length)
    truncation = np.where(over, dt(1) - done, dt(0))
    done = np.where(over, dt(1), done)
    if k.auto_reset:  # AutoResetWrapper.step (training.py:146-158)
      m = done != 0
      s = _where_env(m, st.first, s)
    return EnvState(s, self.obs(s), reward, done, metrics, steps, truncation, st.first)


def _where_env(mask: np.ndarray, a: PState, b: PState) -> PState:
  """Per env, the fields of a where mask else those of b."""
  kw = {}
  for f in dataclasses.fields(PState):
    va, vb = getattr(a, f.name), getattr(b, f.name)
    if isinstance(va, np.ndarray) and isinstance(vb, np.ndarray) and va.shape == vb.shape and va.ndim >= 1:
      kw[f.name] = np.where(mask.reshape((-1,) + (1,) * (va.ndim - 1)), va, vb)
    else:
      kw[f.name] = vb
  return PState(**kw)
