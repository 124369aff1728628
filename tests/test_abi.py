"""CPU-side checks of the C ABI boundary: the library loads, exports every
symbol include/braxg.h declares, validates descriptors before touching a GPU,
and the descriptor layout agrees between model_layout.h and model_pack.py."""

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
  text = open(os.path.join(ROOT, 'include', 'braxg.h')).read()
  text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
  return sorted(set(re.findall(r'\b(braxg_\w+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
  from brax_gb300 import _native, build
  build.build()
  return _native.lib()


def test_exports_every_declared_symbol(lib):
  names = _declared()
  assert 'braxg_step' in names and 'braxg_init' in names
  for n in names:
    assert hasattr(lib, n), n


def test_native_binding_covers_header():
  from brax_gb300 import _native
  for n in _declared():
    assert n in _native.EXPORTS, n


def test_descriptor_validation_without_gpu(lib):
  from brax_gb300 import _native as N
  from brax_gb300 import mjcf, model_pack
  desc = model_pack.pack(mjcf.load_asset('quadruped'))
  h = ctypes.c_void_p()
  bad = desc.copy()
  bad[0] = 0
  assert lib.braxg_model_create(bad.ctypes.data, bad.nbytes, 0, ctypes.byref(h)) == N.ERR_INVALID
  assert b'magic' in lib.braxg_last_error()
  assert lib.braxg_model_create(desc.ctypes.data, desc.nbytes - 4, 0, ctypes.byref(h)) == N.ERR_INVALID
  bad = desc.copy()
  bad[model_pack.H['BXM_H_M']] += 1
  assert lib.braxg_model_create(bad.ctypes.data, bad.nbytes, 0, ctypes.byref(h)) == N.ERR_INVALID
  assert lib.braxg_model_create(None, 0, 0, ctypes.byref(h)) == N.ERR_INVALID
  with pytest.raises(ValueError):
    N.check(N.ERR_INVALID, 'x')
  with pytest.raises(NotImplementedError):
    N.check(N.ERR_UNSUPPORTED, 'x')
  with pytest.raises(RuntimeError):
    N.check(N.ERR_CUDA, 'x')


def test_null_arguments_rejected(lib):
  from brax_gb300 import _native as N
  st = N.State()
  assert lib.braxg_step(None, None, 1, 1, None, ctypes.byref(st), ctypes.byref(st), None) == N.ERR_INVALID
  assert lib.braxg_init(None, None, 1, None, None, ctypes.byref(st), None) == N.ERR_INVALID


def test_layout_enum_parses():
  from brax_gb300 import model_pack
  H = model_pack.H
  assert H['BXM_H_MAGIC'] == 0 and H['BXM_HEADER_WORDS'] == 128
  assert max(v for k, v in H.items() if k != 'BXM_HEADER_WORDS') < 128


@pytest.mark.parametrize('name', ['chain3', 'quadruped', 'humanoid_like'])
def test_pack_roundtrip(name):
  from brax_gb300 import mjcf, model_pack
  sys_ = mjcf.load_asset(name)
  d = model_pack.pack(sys_)
  H = model_pack.H
  assert d[H['BXM_H_WORDS']] == d.shape[0]
  assert d[H['BXM_H_NV']] == sys_.qd_size() and d[H['BXM_H_M']] == sys_.n_constraint_rows()
  f = d.view(np.float32)
  o = d[H['BXM_O_LI_MASS']]
  np.testing.assert_allclose(f[o:o + sys_.num_links()], sys_.link.inertia.mass, rtol=1e-6)
  o = d[H['BXM_O_LINK_PARENT']]
  assert tuple(d[o:o + sys_.num_links()]) == tuple(sys_.link_parents)
  # every array offset is 16-byte aligned
  for k, v in H.items():
    if k.startswith('BXM_O_'):
      assert d[v] % 4 == 0


def test_batch_argument_validation_without_gpu(lib):
  from brax_gb300 import _native as N
  h = ctypes.c_void_p()
  assert lib.braxg_batch_create(None, None, None, 0, None, 0, 0, ctypes.byref(h)) == N.ERR_INVALID
  assert b'n_models' in lib.braxg_last_error()
  ne = (ctypes.c_int32 * 1)(4)
  models = (ctypes.c_void_p * 1)(None)
  assert lib.braxg_batch_create(models, ne, None, 1, None, 0, 0, ctypes.byref(h)) == N.ERR_INVALID
  assert b'NULL' in lib.braxg_last_error()
  assert lib.braxg_batch_rollout(None, None, 1, None, None, None, None, None, None) == N.ERR_INVALID
  assert lib.braxg_batch_init(None, None, None, None, None, None) == N.ERR_INVALID


def test_chain_workloads_and_uneven_mix():
  from brax_gb300 import workloads as W
  for k in (2, 9, 32):
    s = W.chain(k)
    assert (s.num_links(), s.q_size(), s.qd_size(), s.act_size()) == (k, k, k, k)
    assert s.contacts.n == 2  # the last capsule against the plane: two end points
  mix = W.uneven_mix(8192, 0)
  assert sum(n for _, n, _ in mix) == 8192
  names = [s.name for s, _, _ in mix]
  assert names[-2:] == ['quadruped', 'humanoid_like']
  n_chain = sum(n for s, n, _ in mix if s.name.startswith('chain'))
  assert abs(n_chain - 0.6 * 8192) <= 1
  assert max(s.qd_size() for s, _, _ in mix) == 32 and min(s.qd_size() for s, _, _ in mix) == 2

