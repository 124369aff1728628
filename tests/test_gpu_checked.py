"""The bounds-checked build (-DBRAXG_CHECK) on the GPU.

Runs tests/check/run_small_cases.py (every kernel path on <= 64 envs) twice,
in child processes: with the checked library (BRAXG_CHECK=1) and with the
default one.  The checked run must set BRAXG_ENV_BOUNDS on no env (every
scratch carve-out, Jacobian row index, float4 alignment and arena canary
held), and its results must equal the default build's bit for bit: the checks
read and compare but change no arithmetic.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(path, checked):
  env = dict(os.environ, BRAXG_CHECK='1' if checked else '0')
  r = subprocess.run([sys.executable, os.path.join(ROOT, 'tests', 'check', 'run_small_cases.py'), str(path)],
                     env=env, capture_output=True, text=True, timeout=900)
  assert r.returncode == 0, r.stderr[-3000:]
  return dict(np.load(path))


def test_checked_build_flags_nothing_and_changes_nothing(tmp_path):
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import build
  build.build(check=True)
  chk = _run(tmp_path / 'checked.npz', True)
  ref = _run(tmp_path / 'default.npz', False)
  assert bool(chk['checked']) and not bool(ref['checked'])
  assert (chk['lying_rows'] > 32).any()
  for k, v in chk.items():
    if k == 'checked':
      continue
    if k.endswith('status'):
      assert not (v & 16).any(), (k, np.nonzero(v & 16))
    np.testing.assert_array_equal(v, ref[k], err_msg=k)
