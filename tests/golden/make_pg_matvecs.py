"""Writes pg_matvecs.json: the mean number of A-matvecs the FP64 oracle's
projected-gradient solve executes per pipeline step on each workload (seeded
resets, 20 env steps of 5 frames, 128 envs).  bench.py uses it in the fixed
algorithmic FLOP count (F_PG = 2 m^2 N_mv)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from brax_gb300 import mjcf  # noqa: E402
from oracle.pipeline import Oracle  # noqa: E402
from tests.parity_util import actions, seeded_inputs  # noqa: E402


def main():
  out = {}
  for name in ('chain3', 'quadruped', 'humanoid_like'):
    sys_ = mjcf.load_asset(name)
    o = Oracle(sys_, np.float64)
    n = 128
    q, qd = seeded_inputs(sys_, n, seed=0)
    rng = np.random.default_rng(1)
    s = o.init(q, qd)
    counts = []
    for _ in range(20):
      a = actions(sys_, n, rng)
      for _ in range(5):
        s = o.step(s, a)
        counts.append(float(np.mean(s.pg_matvecs)))
    out[name] = {'mean_matvecs_per_step': float(np.mean(counts)), 'envs': n, 'env_steps': 20,
                 'frames': 5, 'rows_m': sys_.n_constraint_rows(), 'ncon': sys_.contacts.n}
  with open(os.path.join(HERE, 'pg_matvecs.json'), 'w') as f:
    json.dump(out, f, indent=1)
  print(json.dumps(out, indent=1))


if __name__ == '__main__':
  main()
