"""The headline workload's non-finite envs are the reference algorithm's.

Over the benchmark's 210 env steps (4096 quadrupeds, U(-1, 1) actions at gear
150, 5 x 0.01 s per env step, the exact inverse) a few envs leave the ground,
spin up in flight, and the semi-implicit integrator (brax/generalized/
integrator.py:46-84) then diverges within a few env steps: the kernel flags
them BRAXG_ENV_NONFINITE (and BRAXG_ENV_NOT_SPD, the mass matrix of the
non-finite state).  The check: for every flagged env, the FP64 oracle run
from the GPU's state 8 env steps before the first non-finite one, with the
same actions, follows the GPU's trajectory (max |qd| within 1 % at each step
up to the blow-up) and diverges too (non-finite, a mass matrix that is not
positive definite, or max |qd| above 1e4).  Chaos separates the GPU's and
the oracle's whole-run trajectories long before (contacts amplify rounding),
so the replay starts from the GPU's own state.
"""

import warnings

import numpy as np
import pytest

from tests.parity_util import load

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def test_blowups_are_the_reference_algorithms():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import pipeline as P
  from oracle.pipeline import Oracle
  sys_ = load('quadruped')
  dev = torch.device('cuda')
  n, total, back = 4096, 210, 8
  rng = np.random.default_rng(1234)  # the benchmark's resets and actions
  q0 = (sys_.init_q + rng.uniform(-0.1, 0.1, (n, sys_.q_size()))).astype(np.float32)
  qd0 = (0.1 * rng.normal(size=(n, sys_.qd_size()))).astype(np.float32)
  gen = torch.Generator(device=dev)
  gen.manual_seed(77)
  acts = torch.rand(total, n, sys_.act_size(), device=dev, generator=gen) * 2 - 1
  s = P.init(sys_, torch.tensor(q0, device=dev), torch.tensor(qd0, device=dev))
  tq, tqd, flags = [], [], []
  for i in range(total):
    s = P.step(sys_, s, acts[i], n_frames=5, inverse_mode=P.CHOLESKY)
    tq.append(s.q.cpu().numpy())
    tqd.append(s.qd.cpu().numpy())
    flags.append(s.status.cpu().numpy())
  tq, tqd, flags = np.stack(tq), np.stack(tqd), np.stack(flags)
  act = acts.cpu().numpy().astype(np.float64)
  finite = np.isfinite(tq).all(-1) & np.isfinite(tqd).all(-1)
  flagged = np.nonzero((flags != 0).any(0))[0]
  # every flag is a non-finite state and every non-finite state is flagged
  np.testing.assert_array_equal((flags & 1) != 0, ~finite)
  assert len(flagged) <= 16, f'{len(flagged)} envs flagged'
  o = Oracle(sys_, np.float64, exact_inverse=True)
  for e in flagged:
    first = int(np.argmax(~finite[:, e]))
    assert first > back, f'env {e} is non-finite after {first} env steps'
    s0 = first - back
    st = o.init(tq[s0, e][None].astype(np.float64), tqd[s0, e][None].astype(np.float64))
    diverged, log = False, []
    with warnings.catch_warnings():
      warnings.simplefilter('ignore')
      for i in range(s0 + 1, first + 1):
        try:
          st = o.env_step(st, act[i, e][None], 5)
        except np.linalg.LinAlgError:
          diverged = True
          log.append(f'{i}: not positive definite')
          break
        qd = np.asarray(st.qd[0], np.float64)
        if not np.isfinite(qd).all():
          diverged = True
          log.append(f'{i}: non-finite')
          break
        big, gpu = np.abs(qd).max(), np.abs(tqd[i, e]).max()
        log.append(f'{i}: |qd| {big:.3g} (GPU {gpu:.3g})')
        if big > 1e4:
          diverged = True
          break
        assert abs(big - gpu) <= 1e-2 * gpu, f'env {e}: ' + '; '.join(log)
    print(f'env {e}: GPU non-finite at env step {first}; FP64 oracle from env step {s0}: ' + '; '.join(log))
    assert diverged, f'env {e}: the oracle stays finite: ' + '; '.join(log)
