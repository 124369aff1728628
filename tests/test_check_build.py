"""The checked build (-DBRAXG_CHECK): host-side test of its scratch checks.

tests/check/layout_check.cu includes the kernels' own layout and check code
(make_layout, the stages' ScratchUse declarations, scratch_use_ok) compiled
for the host, and shows that every stage's scratch use fits the real arena of
each model below while an undersized arena fails the check that sets
BRAXG_ENV_BOUNDS in the kernels.  nvcc compiles it as host code; no GPU runs.
"""

import os
import shutil
import subprocess

import pytest

from brax_gb300 import workloads
from tests.parity_util import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
  cand = os.path.join(os.environ.get('CUDA_HOME', '/usr/local/cuda'), 'bin', 'nvcc')
  return cand if os.path.exists(cand) else shutil.which('nvcc')


def _dims(sys):
  return [sys.num_links(), sys.q_size(), sys.qd_size(), sys.act_size(), sys.contacts.n, sys.n_limit_rows(),
          sys.matrix_inv_iterations, 1 if sys.enable_fluid else 0]


def test_scratch_checks_flag_an_undersized_arena(tmp_path):
  nvcc = _nvcc()
  if nvcc is None:
    pytest.skip('nvcc not available')
  exe = tmp_path / 'layout_check'
  cmd = [nvcc, '-x', 'cu', '-std=c++17', '-DBRAXG_CHECK', '-I', os.path.join(ROOT, 'include'),
         '-I', os.path.join(ROOT, 'brax_gb300', 'csrc'), os.path.join(ROOT, 'tests', 'check', 'layout_check.cu'),
         '-o', str(exe)]
  r = subprocess.run(cmd, capture_output=True, text=True)
  assert r.returncode == 0, r.stderr
  models = [load('chain3'), load('quadruped'), load('humanoid_like'), workloads.chain(32)]
  args = [str(v) for s in models for v in _dims(s)]
  r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=60)
  assert r.returncode == 0, r.stderr + r.stdout
  assert r.stdout.startswith('ok ')
