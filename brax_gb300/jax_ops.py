"""JAX binding: the braxg kernels as XLA FFI custom calls.

The reference runs ``jax.jit(jax.vmap(pipeline.step))``
(brax/envs/wrappers/training.py:66-72) and differentiates ``lax.scan`` of
env steps with ``jax.grad`` (brax/training/agents/apg/train.py:188-198).
Here:

* ``step(sys, state, act, n_frames)`` is one XLA custom call
  (``braxg_step`` -> braxg_step of the C ABI); ``state`` is a ``JaxState``
  with the reference's field names.  Arrays carry the env batch as leading
  axes (an unbatched call is one env); under ``jax.vmap`` the batch axes are
  moved to the front and passed through (``vmap_method='broadcast_all'``).
* ``rollout(sys, q0, qd0, act_seq, n_frames, ckpt_every)`` returns the
  trajectory ``(traj_q [T, n, nq], traj_qd [T, n, nv])`` of ``act_seq
  [T, n, nu]`` from the state of ``pipeline.init(q0, qd0)`` and is a
  ``jax.custom_vjp``: its forward under differentiation is the gradient
  kernel's forward half (``braxg_rollout_vjp_fwd``), whose checkpoints and
  frame snapshots are the residual, and its backward the reverse half
  (``braxg_rollout_vjp_bwd``), which the APG training step can call through
  ``jax.grad`` unchanged; ``rollout_grad`` is the fused launch
  (``braxg_rollout_vjp``) for callers that hold the cotangents up front.

The handlers live in ``libbraxg_xla.so`` (brax_gb300/csrc/xla/braxg_xla.cc),
which ``brax_gb300.build.build_xla`` compiles only where jaxlib's FFI headers
are installed.  Without jax (or without that library) ``AVAILABLE`` is False
and every function raises ImportError; nothing falls back to another path.
"""

from __future__ import annotations

import ctypes
import functools
import os
import threading
from typing import NamedTuple

import numpy as np

try:  # jax is optional: the torch binding (pipeline.py) does not need it
  import jax
  import jax.numpy as jnp
except ImportError:  # pragma: no cover - exercised where jax is installed
  jax = None
  jnp = None

from brax_gb300 import _native as N
from brax_gb300 import model_pack

XLA_LIB = os.path.join(N.LIB_DIR, 'libbraxg_xla.so')
TARGETS = {'braxg_step': 'BraxgStepFfi', 'braxg_rollout': 'BraxgRolloutFfi',
           'braxg_rollout_vjp': 'BraxgRolloutVjpFfi', 'braxg_rollout_vjp_fwd': 'BraxgRolloutVjpFwdFfi',
           'braxg_rollout_vjp_bwd': 'BraxgRolloutVjpBwdFfi'}

AVAILABLE = jax is not None and os.path.exists(XLA_LIB)

NEWTON_SCHULZ = N.INV_NEWTON_SCHULZ
CHOLESKY = N.INV_CHOLESKY


class JaxState(NamedTuple):
  """The carried and returned fields of brax.generalized.base.State
  (brax/generalized/base.py:25-92) for the XLA path (a pytree)."""
  q: object
  qd: object
  mass_mx_inv: object
  x_pos: object = None
  x_rot: object = None
  xd_ang: object = None
  xd_vel: object = None
  qf_smooth: object = None
  qf_constraint: object = None
  qdd: object = None
  status: object = None


_lock = threading.Lock()
_registered = False
_models = {}


def _require():
  if jax is None:
    raise ImportError('brax_gb300.jax_ops needs jax (not installed)')
  if not os.path.exists(XLA_LIB):
    raise ImportError(f'{XLA_LIB} is not built: brax_gb300.build.build_xla() needs jaxlib\'s FFI '
                      'headers (jax.ffi.include_dir())')


def register():
  """Registers the custom-call targets for the CUDA platform (once)."""
  global _registered
  _require()
  with _lock:
    if _registered:
      return
    N.lib()  # libbraxg.so first: libbraxg_xla.so links against it
    lib = ctypes.CDLL(XLA_LIB)
    for name, sym in TARGETS.items():
      jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, sym)), platform='CUDA')
    _registered = True


def model_handle(sys, device_id: int = 0) -> int:
  """The braxg model of ``sys`` on CUDA device ``device_id`` (created once,
  kept for the process), as the int64 custom-call attribute."""
  key = (id(sys), int(device_id))
  with _lock:
    ent = _models.get(key)
    if ent is None or ent[0] is not sys:
      desc = model_pack.pack(sys)
      h = ctypes.c_void_p()
      N.check(N.lib().braxg_model_create(desc.ctypes.data, desc.nbytes, int(device_id), ctypes.byref(h)),
              'braxg_model_create')
      ent = (sys, h, desc)
      _models[key] = ent
    return int(ent[1].value)


def _dims(sys):
  return sys.num_links(), sys.q_size(), sys.qd_size(), sys.act_size()


def step(sys, state: JaxState, act, n_frames: int = 1, inverse_mode: int = NEWTON_SCHULZ,
         device_id: int = 0) -> JaxState:
  """n_frames x brax/generalized/pipeline.py:64-94 with one action
  (brax/envs/base.py:128-137) as one XLA custom call."""
  register()
  nl, nq, nv, nu = _dims(sys)
  q = jnp.asarray(state.q, jnp.float32)
  batch = q.shape[:-1]
  f32 = lambda *s: jax.ShapeDtypeStruct(batch + s, jnp.float32)
  out_types = (f32(nq), f32(nv), f32(nv, nv), f32(nl, 3), f32(nl, 4), f32(nl, 3), f32(nl, 3), f32(nv),
               f32(nv), f32(nv), jax.ShapeDtypeStruct(batch, jnp.int32))
  if act is None:
    act = jnp.zeros(batch + (nu,), jnp.float32)
  call = jax.ffi.ffi_call('braxg_step', out_types, vmap_method='broadcast_all')
  outs = call(q, jnp.asarray(state.qd, jnp.float32), jnp.asarray(state.mass_mx_inv, jnp.float32),
              jnp.asarray(act, jnp.float32), model=np.int64(model_handle(sys, device_id)),
              n_frames=np.int32(n_frames), inverse_mode=np.int32(inverse_mode))
  return JaxState(*outs)


def _rollout_call(handle, nq, nv, n_frames, q0, qd0, act_seq, inverse_mode=CHOLESKY):
  T, batch = act_seq.shape[0], q0.shape[:-1]
  out_types = (jax.ShapeDtypeStruct((T,) + batch + (nq,), jnp.float32),
               jax.ShapeDtypeStruct((T,) + batch + (nv,), jnp.float32),
               jax.ShapeDtypeStruct(batch, jnp.int32))
  call = jax.ffi.ffi_call('braxg_rollout', out_types, vmap_method='sequential')
  return call(q0, qd0, act_seq, model=np.int64(handle), n_frames=np.int32(n_frames),
              inverse_mode=np.int32(inverse_mode))


def _vjp_call(handle, nq, nv, nu, n_frames, ckpt_every, q0, qd0, act_seq, q_bar, qd_bar, inverse_mode=CHOLESKY):
  batch = q0.shape[:-1]
  out_types = (jax.ShapeDtypeStruct(act_seq.shape, jnp.float32),
               jax.ShapeDtypeStruct(batch + (nq,), jnp.float32),
               jax.ShapeDtypeStruct(batch + (nv,), jnp.float32),
               jax.ShapeDtypeStruct(batch, jnp.int32))
  call = jax.ffi.ffi_call('braxg_rollout_vjp', out_types, vmap_method='sequential')
  return call(q0, qd0, act_seq, q_bar, qd_bar, model=np.int64(handle), n_frames=np.int32(n_frames),
              ckpt_every=np.int32(ckpt_every), inverse_mode=np.int32(inverse_mode))


def _residual_bytes(handle, n_env, n_steps, n_frames, ckpt_every, inverse_mode=CHOLESKY) -> int:
  """Bytes of the gradient workspace with every segment resident (the
  residual of the split forward), for the inverse mode's records."""
  nbytes = ctypes.c_size_t()
  N.check(N.lib().braxg_rollout_vjp_workspace_mode(ctypes.c_void_p(handle), int(n_env), int(n_steps),
                                                   int(n_frames), int(ckpt_every), 0, int(inverse_mode),
                                                   ctypes.byref(nbytes)),
          'braxg_rollout_vjp_workspace_mode')
  return int(nbytes.value)


def _vjp_fwd_call(handle, nq, nv, n_frames, ckpt_every, q0, qd0, act_seq, inverse_mode=CHOLESKY):
  T, batch = act_seq.shape[0], q0.shape[:-1]
  n = int(np.prod(batch)) if batch else 1
  out_types = (jax.ShapeDtypeStruct((T,) + batch + (nq,), jnp.float32),
               jax.ShapeDtypeStruct((T,) + batch + (nv,), jnp.float32),
               jax.ShapeDtypeStruct(batch, jnp.int32),
               jax.ShapeDtypeStruct((_residual_bytes(handle, n, T, n_frames, ckpt_every, inverse_mode),),
                                    jnp.uint8))
  call = jax.ffi.ffi_call('braxg_rollout_vjp_fwd', out_types, vmap_method='sequential')
  return call(q0, qd0, act_seq, model=np.int64(handle), n_frames=np.int32(n_frames),
              ckpt_every=np.int32(ckpt_every), inverse_mode=np.int32(inverse_mode))


def _vjp_bwd_call(handle, nq, nv, n_frames, ckpt_every, q0, qd0, act_seq, residual, status, q_bar, qd_bar,
                  inverse_mode=CHOLESKY):
  batch = q0.shape[:-1]
  out_types = (jax.ShapeDtypeStruct(act_seq.shape, jnp.float32),
               jax.ShapeDtypeStruct(batch + (nq,), jnp.float32),
               jax.ShapeDtypeStruct(batch + (nv,), jnp.float32),
               jax.ShapeDtypeStruct(batch, jnp.int32))
  # the forward's status (argument 6) is the status result: the reverse ORs its bits in
  call = jax.ffi.ffi_call('braxg_rollout_vjp_bwd', out_types, vmap_method='sequential',
                          input_output_aliases={6: 3})
  return call(q0, qd0, act_seq, residual, q_bar, qd_bar, status, model=np.int64(handle),
              n_frames=np.int32(n_frames), ckpt_every=np.int32(ckpt_every), inverse_mode=np.int32(inverse_mode))


@functools.lru_cache(maxsize=None)
def _rollout_fn(handle: int, nq: int, nv: int, nu: int, n_frames: int, ckpt_every: int, inverse_mode: int):
  """jax.custom_vjp rollout for one model and static configuration."""

  @jax.custom_vjp
  def roll(q0, qd0, act_seq):
    tq, tqd, _ = _rollout_call(handle, nq, nv, n_frames, q0, qd0, act_seq, inverse_mode)
    return tq, tqd

  def fwd(q0, qd0, act_seq):
    tq, tqd, status, residual = _vjp_fwd_call(handle, nq, nv, n_frames, ckpt_every, q0, qd0, act_seq,
                                              inverse_mode)
    return (tq, tqd), (q0, qd0, act_seq, residual, status)

  def bwd(res, g):
    q0, qd0, act_seq, residual, status = res
    gq, gqd = g
    act_bar, q0_bar, qd0_bar, _ = _vjp_bwd_call(handle, nq, nv, n_frames, ckpt_every, q0, qd0, act_seq, residual,
                                                status, jnp.asarray(gq, jnp.float32), jnp.asarray(gqd, jnp.float32),
                                                inverse_mode)
    return q0_bar, qd0_bar, act_bar

  roll.defvjp(fwd, bwd)
  return roll


def rollout_grad(sys, q0, qd0, act_seq, q_bar, qd_bar, n_frames: int = 1, ckpt_every: int = 16,
                 device_id: int = 0, inverse_mode: int = CHOLESKY):
  """(act_bar, q0_bar, qd0_bar, status) of the rollout for cotangents q_bar
  [T, n, nq], qd_bar [T, n, nv] in one fused launch (braxg_rollout_vjp)."""
  register()
  nl, nq, nv, nu = _dims(sys)
  return _vjp_call(model_handle(sys, device_id), nq, nv, nu, int(n_frames), int(ckpt_every),
                   jnp.asarray(q0, jnp.float32), jnp.asarray(qd0, jnp.float32), jnp.asarray(act_seq, jnp.float32),
                   jnp.asarray(q_bar, jnp.float32), jnp.asarray(qd_bar, jnp.float32), int(inverse_mode))


def rollout(sys, q0, qd0, act_seq, n_frames: int = 1, ckpt_every: int = 16, device_id: int = 0,
            inverse_mode: int = CHOLESKY):
  """Differentiable rollout: ``(traj_q, traj_qd)`` of act_seq [T, n, nu]
  from q0 [n, nq], qd0 [n, nv]; gradients through the hand-written adjoint.
  inverse_mode CHOLESKY (default) computes the exact inverse every frame;
  NEWTON_SCHULZ carries init's exact inverse through the reference's
  Newton-Schulz update, and the gradient differentiates that update."""
  register()
  nl, nq, nv, nu = _dims(sys)
  fn = _rollout_fn(model_handle(sys, device_id), nq, nv, nu, int(n_frames), int(ckpt_every), int(inverse_mode))
  return fn(jnp.asarray(q0, jnp.float32), jnp.asarray(qd0, jnp.float32), jnp.asarray(act_seq, jnp.float32))
