"""The fused env step (braxg_env_rollout) against the oracle's restatement of
brax/envs/ant.py with EpisodeWrapper and AutoResetWrapper (oracle/env.py).

Quadruped, 48 envs, episode_length 4 so that truncation and the auto-reset run
inside the rollout, and two envs started above the healthy z range so that the
task's own done and reset run on the first step.  Compared per env step:
reward (|err| <= 1e-4 + 1e-4 |ref|), done / steps / truncation exactly (envs
whose torso height is within 1e-4 of a healthy-range edge excluded), obs and
the metrics of the last step (relative 1e-5 for 99 % of envs).  One launch of
6 env steps equals 6 single-step launches.
"""

import numpy as np
import pytest

from tests.parity_util import rel_err

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

N_ENV, N_STEPS, EP_LEN = 48, 6, 4


def _setup():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import envs as E
  from brax_gb300 import workloads as W
  return E, W


def _inputs(W, sys_):
  rng = np.random.default_rng(21)
  q, qd = W.reset(sys_, N_ENV, rng)
  q[3, 2] = 1.3   # above the healthy range: done on the first step
  q[7, 2] = 1.25
  acts = np.stack([W.actions(sys_, N_ENV, rng) for _ in range(N_STEPS)]).astype(np.float32)
  return q.astype(np.float32), qd.astype(np.float32), acts


def _oracle(sys_, q, qd, acts):
  from oracle.env import LocomotionOracle, TaskParams
  from oracle.pipeline import Oracle
  o = LocomotionOracle(Oracle(sys_, np.float32, exact_inverse=True), 5, TaskParams(episode_length=EP_LEN))
  st = o.reset(q, qd)
  out = []
  for k in range(N_STEPS):
    st = o.step(st, acts[k])
    out.append(st)
  return out


def test_env_rollout_matches_oracle():
  E, W = _setup()
  sys_ = W.asset('quadruped')
  env = E.Locomotion(sys_, episode_length=EP_LEN)
  q, qd, acts = _inputs(W, sys_)
  dev = env.device
  st0 = env.reset(N_ENV, q=torch.tensor(q, device=dev), qd=torch.tensor(qd, device=dev))
  got, rewards, dones = env.rollout(st0, torch.tensor(acts, device=dev))
  torch.cuda.synchronize()
  ref = _oracle(sys_, q, qd, acts)
  rewards, dones = rewards.cpu().numpy(), dones.cpu().numpy()
  z_edges = np.array([0.2, 1.0])
  for k in range(N_STEPS):
    r = ref[k]
    z = r.pipeline_state.q[:, 2]
    near = np.abs(z[:, None] - z_edges[None]).min(-1) <= 1e-4
    err = np.abs(rewards[k] - r.reward)
    assert (err <= 1e-4 + 1e-4 * np.abs(r.reward)).all(), (k, err.max())
    assert ((dones[k] == r.done) | near).all(), (k, np.nonzero(dones[k] != r.done))
  assert dones[0, 3] == 1 and dones[0, 7] == 1       # the task's own done
  fresh = ~(dones[:EP_LEN - 1] != 0).any(0)           # envs whose first episode ran EP_LEN steps
  assert fresh.sum() > N_ENV // 2 and (dones[EP_LEN - 1][fresh] == 1).all()  # truncated at EP_LEN
  last = ref[-1]
  np.testing.assert_array_equal(got.info['steps'].cpu().numpy(), last.steps)
  np.testing.assert_array_equal(got.info['truncation'].cpu().numpy(), last.truncation)
  e = rel_err(got.obs.cpu().numpy(), last.obs)
  print(f'obs after {N_STEPS} env steps: p50 {np.median(e):.2e} p99 {np.quantile(e, 0.99):.2e} max {e.max():.2e}')
  assert np.quantile(e, 0.99) <= 1e-5
  met = np.stack([got.metrics[k].cpu().numpy() for k in sorted(last.metrics)], -1)
  mref = np.stack([last.metrics[k] for k in sorted(last.metrics)], -1)
  e = np.abs(met - mref) / np.maximum(np.abs(mref), 1.0)
  assert np.quantile(e.max(-1), 0.99) <= 1e-4, e.max()
  # reset envs sit exactly at their first state
  for i in (3, 7):
    np.testing.assert_allclose(got.pipeline_state.q[i].cpu().numpy(), q[i], rtol=0, atol=0)


def test_one_launch_equals_per_step_launches():
  E, W = _setup()
  sys_ = W.asset('quadruped')
  env = E.Locomotion(sys_, episode_length=EP_LEN)
  q, qd, acts = _inputs(W, sys_)
  dev = env.device
  st0 = env.reset(N_ENV, q=torch.tensor(q, device=dev), qd=torch.tensor(qd, device=dev))
  one, rewards, _ = env.rollout(st0, torch.tensor(acts, device=dev))
  st = st0
  for k in range(N_STEPS):
    st = env.step(st, torch.tensor(acts[k], device=dev))
    torch.testing.assert_close(st.reward, rewards[k], rtol=0, atol=0)
  torch.cuda.synchronize()
  for a, b in ((one.obs, st.obs), (one.pipeline_state.q, st.pipeline_state.q), (one.done, st.done),
               (one.info['steps'], st.info['steps'])):
    torch.testing.assert_close(a, b, rtol=0, atol=0)
