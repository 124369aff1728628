"""Builds libbraxg.so in-tree with nvcc for sm_103a (no CPU fallback exists)."""

from __future__ import annotations

import concurrent.futures
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'brax_gb300', 'csrc')
OUT_DIR = os.path.join(ROOT, 'brax_gb300', '_lib')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# one translation unit per group of kernel instantiations so they compile in
# parallel; braxg.cu holds the C ABI
UNITS = ['braxg.cu', 'braxg_grad.cu', 'braxg_batch.cu', 'inst_t32_nv16.cu', 'inst_t32_nv32.cu', 'inst_t32_nv64.cu',
         'inst_t16.cu', 'inst_vjp_nv16.cu', 'inst_vjp_nv32.cu', 'inst_batch.cu']


def _nvcc():
  cand = os.environ.get('NVCC') or os.path.join(
      os.environ.get('CUDA_HOME', '/usr/local/cuda'), 'bin', 'nvcc')
  return cand if os.path.exists(cand) else 'nvcc'


def _flags(extra=()):
  return [*ARCH, '-lineinfo', '-O3', '-std=c++17', '-Xcompiler', '-fPIC',
          '-I', os.path.join(ROOT, 'include'), '-I', CSRC, *extra]


def _sources_newer(target, deps):
  if not os.path.exists(target):
    return True
  t = os.path.getmtime(target)
  return any(os.path.getmtime(d) > t for d in deps)


CHECK_DIR = os.path.join(OUT_DIR, 'check')


def build(verbose: bool = False, force: bool = False, check: bool = False) -> str:
  """Compiles (if stale) and returns the path of libbraxg.so.  check=True
  builds the bounds-checked variant (-DBRAXG_CHECK) into _lib/check/ instead;
  brax_gb300._native loads it when BRAXG_CHECK=1 is set."""
  out_dir = CHECK_DIR if check else OUT_DIR
  build_dir = os.path.join(out_dir, 'obj')
  os.makedirs(build_dir, exist_ok=True)
  headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
  headers.append(os.path.join(ROOT, 'include', 'braxg.h'))
  nvcc = _nvcc()
  jobs = []
  objs = []
  extra = ['-DBRAXG_CHECK'] if check else []
  for u in UNITS:
    src = os.path.join(CSRC, u)
    obj = os.path.join(build_dir, u.replace('.cu', '.o'))
    objs.append(obj)
    if force or _sources_newer(obj, [src, *headers]):
      jobs.append([nvcc, *_flags(extra + (['-Xptxas', '-v'] if verbose else [])), '-c', src, '-o', obj])

  def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError(f'nvcc failed: {" ".join(cmd)}\n{r.stdout}\n{r.stderr}')
    return r.stdout + r.stderr

  with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
    for log in ex.map(run, jobs):
      if verbose and log:
        print(log, file=sys.stderr)
  lib = os.path.join(out_dir, 'libbraxg.so')
  if force or jobs or _sources_newer(lib, objs):
    run([nvcc, *ARCH, '-shared', '-o', lib, *objs, '-lcudart'])
  return lib


def xla_include_dir():
  """jaxlib's FFI header directory ($BRAXG_XLA_INCLUDE, else
  jax.ffi.include_dir()), or None where jax is not installed."""
  d = os.environ.get('BRAXG_XLA_INCLUDE')
  if d:
    return d if os.path.exists(os.path.join(d, 'xla', 'ffi', 'api', 'ffi.h')) else None
  try:
    import jax  # noqa: F401
    from jax import ffi
    d = ffi.include_dir()
  except Exception:  # jax absent or too old for jax.ffi
    return None
  return d if os.path.exists(os.path.join(d, 'xla', 'ffi', 'api', 'ffi.h')) else None


XLA_LIB = os.path.join(OUT_DIR, 'libbraxg_xla.so')


def build_xla(verbose: bool = False):
  """Builds libbraxg_xla.so (the XLA FFI handlers of csrc/xla/braxg_xla.cc,
  linked against libbraxg.so) when jaxlib's FFI headers are present; returns
  its path, or None without them."""
  inc = xla_include_dir()
  if inc is None:
    return None
  lib = build(verbose)
  src = os.path.join(CSRC, 'xla', 'braxg_xla.cc')
  deps = [src, os.path.join(CSRC, 'xla', 'xla_core.h'), os.path.join(ROOT, 'include', 'braxg.h'), lib]
  if _sources_newer(XLA_LIB, deps):
    cmd = [_nvcc(), '-x', 'cu', *ARCH, '-O3', '-std=c++17', '-Xcompiler', '-fPIC', '-shared',
           '-I', inc, '-I', os.path.join(ROOT, 'include'), '-I', os.path.join(CSRC, 'xla'), src,
           '-o', XLA_LIB, '-L', OUT_DIR, '-lbraxg', '-Xlinker', '-rpath,$ORIGIN', '-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError(f'nvcc failed: {" ".join(cmd)}\n{r.stdout}\n{r.stderr}')
  return XLA_LIB


if __name__ == '__main__':
  print(build(verbose='-v' in sys.argv, force='-f' in sys.argv, check='--check' in sys.argv))
