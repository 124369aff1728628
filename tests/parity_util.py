"""Shared helpers for the GPU parity tests (kernel vs oracle)."""

import numpy as np

from brax_gb300 import mjcf

WORKLOADS = ('chain3', 'quadruped', 'humanoid_like')


def seeded_inputs(sys, n, seed=0):
  """Reset distribution of the workloads: q jitter U(-0.1, 0.1) on init_q
  (brax/envs/ant.py:209-213), qd ~ 0.1 N(0, 1); the chain uses
  q0 ~ U(-pi/4, pi/4), qd0 ~ N(0, 0.1)."""
  rng = np.random.default_rng(seed)
  if sys.name == 'chain3' or sys.name.startswith('chain'):
    q = rng.uniform(-np.pi / 4, np.pi / 4, (n, sys.q_size()))
    qd = rng.normal(0, 0.1, (n, sys.qd_size()))
  else:
    q = sys.init_q + rng.uniform(-0.1, 0.1, (n, sys.q_size()))
    qd = 0.1 * rng.normal(size=(n, sys.qd_size()))
  return q, qd


def actions(sys, n, rng):
  if sys.name == 'humanoid_like':
    return np.clip(rng.normal(0, 0.3, (n, sys.act_size())), -1, 1)
  if sys.name == 'chain3':
    return np.zeros((n, sys.act_size()))
  return rng.uniform(-1, 1, (n, sys.act_size()))


def rel_err(a, b):
  """Per-env relative error: max |a - b| / max(max |b|, 1) over the trailing axes."""
  a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
  b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
  return np.abs(a - b).max(-1) / np.maximum(np.abs(b).max(-1), 1.0)


def load(name):
  return mjcf.load_asset(name)
