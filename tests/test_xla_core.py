"""The XLA FFI handlers' core (brax_gb300/csrc/xla/xla_core.h), host only.

The handlers of brax_gb300/csrc/xla/braxg_xla.cc compile only where jaxlib's
FFI headers exist; everything they do besides unpacking XLA buffers lives in
xla_core.h.  This test compiles that core with g++ against a stub of the
braxg C calls (tests/xla/core_test.cc) and runs its cases: batch axes as
jax.vmap leaves them, time axes of sequences, shape errors that name the
argument, and the pointers / env counts / options forwarded to each call.
"""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_xla_core_against_stub(tmp_path):
  gxx = shutil.which('g++')
  if gxx is None:
    pytest.skip('g++ not available')
  exe = tmp_path / 'core_test'
  cmd = [gxx, '-std=c++17', '-O1', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'),
         '-I', os.path.join(ROOT, 'brax_gb300', 'csrc', 'xla'),
         os.path.join(ROOT, 'tests', 'xla', 'core_test.cc'), '-o', str(exe)]
  r = subprocess.run(cmd, capture_output=True, text=True)
  assert r.returncode == 0, r.stderr
  r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
  assert r.returncode == 0, r.stderr
  assert r.stdout.startswith('ok ')


def test_jax_ops_without_jax_refuses_cleanly():
  """brax_gb300.jax_ops imports without jax and raises ImportError from every
  entry point (there is no other path to fall back to)."""
  from brax_gb300 import jax_ops
  if jax_ops.jax is not None and jax_ops.AVAILABLE:
    pytest.skip('jax and libbraxg_xla.so are present')
  assert not jax_ops.AVAILABLE
  with pytest.raises(ImportError):
    jax_ops.register()
  with pytest.raises(ImportError):
    jax_ops.rollout(None, None, None, None)


def test_handler_symbols_match_registration():
  """Every target jax_ops registers is a handler symbol braxg_xla.cc defines,
  and each handler binds the attributes jax_ops passes."""
  import re
  from brax_gb300 import jax_ops
  src = open(os.path.join(ROOT, 'brax_gb300', 'csrc', 'xla', 'braxg_xla.cc')).read()
  defined = set(re.findall(r'XLA_FFI_DEFINE_HANDLER_SYMBOL\((\w+),', src))
  assert set(jax_ops.TARGETS.values()) == defined
  for attr in ('model', 'n_frames', 'inverse_mode', 'ckpt_every'):
    assert f'.Attr<' in src and f'("{attr}")' in src
