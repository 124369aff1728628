"""The allocation-free rollout gradient, braxg_rollout_vjp_noalloc.

Some callers cannot allocate device memory (an XLA custom call without the
scratch allocator, a plugin inside a framework that owns every allocation, a
control loop that must stay out of the CUDA allocator).  For them the library
keeps the gradient's checkpoint scratch in one fixed device array.  This test
calls that entry point through the C ABI, twice in a row, and checks that
each result equals, bit for bit, braxg_rollout_vjp given a caller-allocated
workspace: the two entry points run the same kernel, and the gradient does
not depend on how many segments the workspace keeps resident (the fixed
array holds more than the smallest workspace), so any difference would be a
wrong scratch offset or stale scratch contents.  It also checks that an
oversized request is refused with a clear error.  This file is collected
last on purpose, and passes on its own in a fresh process as well.
"""

import ctypes

import numpy as np
import pytest

from tests.parity_util import load, seeded_inputs

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _setup():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from brax_gb300 import _native as N
  from brax_gb300 import pipeline
  return N, pipeline


@pytest.mark.parametrize('mode', ['exact', 'newton_schulz'])
def test_noalloc_rollout_vjp_matches_workspace_variant(mode):
  N, P = _setup()
  lib = N.lib()
  sys_ = load('quadruped')
  m = P.model_for(sys_)
  n, steps, frames, ckpt = 32, 4, 5, 2
  dev = m.device
  q0, qd0 = seeded_inputs(sys_, n, 41)
  q0 = torch.tensor(q0.astype(np.float32), device=dev)
  qd0 = torch.tensor(qd0.astype(np.float32), device=dev)
  rng = np.random.default_rng(42)
  u = torch.tensor(rng.uniform(-1, 1, (steps, n, m.nu)).astype(np.float32), device=dev)
  qd_bar = torch.tensor(rng.normal(size=(steps, n, m.nv)).astype(np.float32), device=dev)
  stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
  inv = N.INV_CHOLESKY if mode == 'exact' else N.INV_NEWTON_SCHULZ
  opt = N.Options(inv, 0, 0, 0, None)

  need = ctypes.c_size_t()  # one resident segment, as the noalloc entry point sizes its request
  N.check(lib.braxg_rollout_vjp_workspace_mode(m.handle, n, steps, frames, ckpt, 1, inv, ctypes.byref(need)),
          'workspace')
  assert need.value <= lib.braxg_rollout_vjp_noalloc_capacity()

  def outputs():
    return (torch.zeros(steps, n, m.nu, device=dev), torch.zeros(n, m.nq, device=dev),
            torch.zeros(n, m.nv, device=dev), torch.zeros(n, dtype=torch.int32, device=dev))

  # reference: the workspace entry point
  ws = torch.empty(need.value, dtype=torch.uint8, device=dev)
  ref = outputs()
  N.check(lib.braxg_rollout_vjp(m.handle, stream, n, steps, frames, ckpt, u.data_ptr(),
                                q0.data_ptr(), qd0.data_ptr(), None, qd_bar.data_ptr(),
                                ref[0].data_ptr(), ref[1].data_ptr(), ref[2].data_ptr(), None, None,
                                ws.data_ptr(), need.value, ref[3].data_ptr(), ctypes.byref(opt)),
          'braxg_rollout_vjp')
  torch.cuda.synchronize()
  for call in range(2):  # two calls in a row share the fixed scratch
    got = outputs()
    N.check(lib.braxg_rollout_vjp_noalloc(m.handle, stream, n, steps, frames, ckpt, u.data_ptr(),
                                          q0.data_ptr(), qd0.data_ptr(), None, qd_bar.data_ptr(),
                                          got[0].data_ptr(), got[1].data_ptr(), got[2].data_ptr(),
                                          None, None, got[3].data_ptr(), ctypes.byref(opt)),
            'braxg_rollout_vjp_noalloc')
    torch.cuda.synchronize()
    assert torch.equal(got[3], ref[3])
    for name, g, r in zip(('act_bar', 'q0_bar', 'qd0_bar'), got[:3], ref[:3]):
      assert torch.isfinite(g).all(), (call, name)
      # rtol = atol = 0: the same kernel on the same inputs
      assert torch.equal(g, r), (call, name, (g - r).abs().max().item())


def test_noalloc_rejects_oversized_request():
  N, P = _setup()
  lib = N.lib()
  m = P.model_for(load('quadruped'))
  cap = lib.braxg_rollout_vjp_noalloc_capacity()
  n, steps, frames, ckpt = 65536, 64, 5, 64
  need = ctypes.c_size_t()
  N.check(lib.braxg_rollout_vjp_workspace(m.handle, n, steps, frames, ckpt, ctypes.byref(need)), 'ws')
  assert need.value > cap
  rc = lib.braxg_rollout_vjp_noalloc(m.handle, None, n, steps, frames, ckpt, None, None, None, None,
                                     None, None, None, None, None, None, None, None)
  assert rc == N.ERR_INVALID
  assert b'fixed array holds' in lib.braxg_last_error()
