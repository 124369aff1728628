"""ctypes binding of the braxg C ABI (include/braxg.h).

The shared library is built in-tree by ``brax_gb300.build``; if it is missing
every entry point raises instead of falling back to any CPU path.
"""

from __future__ import annotations

import ctypes
import os
import threading

LIB_DIR = os.path.join(os.path.dirname(__file__), '_lib')
# BRAXG_CHECK=1 selects the bounds-checked build (brax_gb300.build.build(check=True))
CHECKED = os.environ.get('BRAXG_CHECK') == '1'
LIB_PATH = os.path.join(LIB_DIR, 'check', 'libbraxg.so') if CHECKED else os.path.join(LIB_DIR, 'libbraxg.so')

STATE_FIELDS = (
    'q', 'qd', 'mass_mx_inv', 'x_pos', 'x_rot', 'xd_ang', 'xd_vel', 'qf_smooth',
    'qf_constraint', 'qdd', 'root_com', 'cinr_pos', 'cinr_rot', 'cinr_i', 'cd',
    'cdof', 'cdofd', 'mass_mx', 'con_jac', 'con_diag', 'con_aref', 'status', 'cache',
    'contact_dist', 'contact_pos', 'contact_frame', 'solver_maxiter')

EXPORTS = ('braxg_model_create', 'braxg_model_destroy', 'braxg_model_dims', 'braxg_model_cache_words', 'braxg_model_cache_span',
           'braxg_init', 'braxg_step', 'braxg_rollout', 'braxg_rollout_vjp_workspace',
           'braxg_rollout_vjp_workspace_resident', 'braxg_rollout_vjp_workspace_mode',
           'braxg_rollout_vjp', 'braxg_rollout_vjp_fwd', 'braxg_rollout_vjp_bwd', 'braxg_rollout_vjp_noalloc',
           'braxg_rollout_vjp_noalloc_capacity', 'braxg_launch_shape',
           'braxg_batch_create', 'braxg_batch_destroy', 'braxg_batch_get_offsets',
           'braxg_batch_launch_info', 'braxg_batch_init', 'braxg_batch_rollout',
           'braxg_env_rollout',
           'braxg_last_launch_count', 'braxg_last_error')

OK, ERR_INVALID, ERR_CUDA, ERR_UNSUPPORTED = 0, 1, 2, 3
INV_NEWTON_SCHULZ, INV_CHOLESKY = 0, 1
ENV_NONFINITE, ENV_NOT_SPD, ENV_NO_GRADIENT, ENV_SKIPPED, ENV_BOUNDS = 1, 2, 4, 8, 16


class State(ctypes.Structure):
  _fields_ = [(n, ctypes.c_void_p) for n in STATE_FIELDS]


class Dims(ctypes.Structure):
  _fields_ = [(n, ctypes.c_int32) for n in ('nl', 'nq', 'nv', 'nu', 'ncon', 'nlim', 'm')]


RANDOMIZATION_FIELDS = ('friction', 'act_gain', 'act_bias_q', 'act_bias_qd', 'link_mass', 'link_inertia',
                        'dof_armature', 'dof_damping', 'dof_stiffness')


class Randomization(ctypes.Structure):
  _fields_ = [(n, ctypes.c_void_p) for n in RANDOMIZATION_FIELDS]


class Options(ctypes.Structure):
  _fields_ = [('inverse_mode', ctypes.c_int32), ('threads_per_env', ctypes.c_int32),
              ('envs_per_cta', ctypes.c_int32), ('relax_barriers', ctypes.c_int32),
              ('stage_cycles', ctypes.c_void_p), ('randomization', ctypes.POINTER(Randomization))]


class BucketShape(ctypes.Structure):
  _fields_ = [('nv_max', ctypes.c_int32), ('threads_per_env', ctypes.c_int32),
              ('envs_per_cta', ctypes.c_int32), ('reserved', ctypes.c_int32)]


OFFSET_FIELDS = ('env', 'q', 'qd', 'mass_mx', 'link', 'act', 'row', 'jac')


class BatchOffsets(ctypes.Structure):
  _fields_ = [(n, ctypes.c_int64) for n in OFFSET_FIELDS]


class Task(ctypes.Structure):
  _fields_ = [('ctrl_cost_weight', ctypes.c_float), ('healthy_reward', ctypes.c_float),
              ('healthy_z_min', ctypes.c_float), ('healthy_z_max', ctypes.c_float),
              ('terminate_when_unhealthy', ctypes.c_int32),
              ('exclude_current_positions', ctypes.c_int32), ('episode_length', ctypes.c_int32),
              ('action_repeat', ctypes.c_int32), ('auto_reset', ctypes.c_int32),
              ('reserved', ctypes.c_int32 * 3)]


ENV_IO_FIELDS = ('obs', 'reward', 'done', 'metrics', 'steps', 'truncation', 'last_done',
                 'first_q', 'first_qd', 'first_mass_mx_inv')


class EnvIO(ctypes.Structure):
  _fields_ = [(n, ctypes.c_void_p) for n in ENV_IO_FIELDS]


METRICS = ('reward_forward', 'reward_survive', 'reward_ctrl', 'reward_contact', 'x_position',
           'y_position', 'distance_from_origin', 'x_velocity', 'y_velocity', 'forward_reward')


PROFILE_SLOTS = ('fk', 'com', 'crba', 'inverse', 'jacobian', 'smooth', 'constraint',
                 'integrate', 'io', 'matvecs', 'rows', 'ns_resets', 'substeps')
VJP_PROFILE_SLOTS = {16: 'checkpoint_pass', 17: 'segment_recompute', 18: 'restore',
                     19: 'rev_integrate', 20: 'rev_qdd', 21: 'rev_constraint', 22: 'rev_smooth',
                     23: 'rev_inverse', 24: 'rev_crba', 25: 'rev_rows', 26: 'rev_com', 27: 'rev_fk',
                     28: 'pg_build', 29: 'pg_iterate'}
N_PROFILE_SLOTS = 32


_lib = None
_lock = threading.Lock()


def lib() -> ctypes.CDLL:
  """Loads libbraxg.so (raises if it has not been built)."""
  global _lib
  with _lock:
    if _lib is not None:
      return _lib
    if not os.path.exists(LIB_PATH):
      raise RuntimeError(
          f'braxg CUDA library not built ({LIB_PATH} missing); run '
          f'`python -c "import brax_gb300.build as b; b.build(check={CHECKED})"`')
    l = ctypes.CDLL(LIB_PATH)
    vp, i32, P = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER
    l.braxg_model_create.argtypes = [vp, ctypes.c_size_t, i32, P(vp)]
    l.braxg_model_destroy.argtypes = [vp]
    l.braxg_model_dims.argtypes = [vp, P(Dims)]
    l.braxg_model_cache_words.argtypes = [vp, P(ctypes.c_int32)]
    l.braxg_model_cache_span.argtypes = [vp, P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_int32)]
    l.braxg_init.argtypes = [vp, vp, i32, vp, vp, P(State), P(Options)]
    l.braxg_step.argtypes = [vp, vp, i32, i32, vp, P(State), P(State), P(Options)]
    l.braxg_rollout.argtypes = [vp, vp, i32, i32, i32, vp, P(State), P(State), vp, vp,
                                P(Options)]
    l.braxg_rollout_vjp_workspace.argtypes = [vp, i32, i32, i32, i32, P(ctypes.c_size_t)]
    l.braxg_rollout_vjp_workspace_resident.argtypes = [vp, i32, i32, i32, i32, i32,
                                                       P(ctypes.c_size_t)]
    l.braxg_rollout_vjp_workspace_mode.argtypes = [vp, i32, i32, i32, i32, i32, i32, P(ctypes.c_size_t)]
    l.braxg_rollout_vjp.argtypes = [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp,
                                    vp, vp, vp, ctypes.c_size_t, vp, P(Options)]
    l.braxg_rollout_vjp_fwd.argtypes = [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp,
                                        ctypes.c_size_t, vp, P(Options)]
    l.braxg_rollout_vjp_bwd.argtypes = [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp,
                                        vp, ctypes.c_size_t, vp, P(Options)]
    l.braxg_rollout_vjp_noalloc.argtypes = [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp,
                                            vp, vp, vp, vp, vp, P(Options)]
    l.braxg_rollout_vjp_noalloc_capacity.restype = ctypes.c_size_t
    l.braxg_rollout_vjp_noalloc_capacity.argtypes = []
    l.braxg_launch_shape.argtypes = [vp, P(Options), i32, P(ctypes.c_int32), P(ctypes.c_int32),
                                     P(ctypes.c_int32)]
    l.braxg_batch_create.argtypes = [P(vp), P(ctypes.c_int32), P(ctypes.c_int32), i32,
                                     P(BucketShape), i32, ctypes.c_int32, P(vp)]
    l.braxg_batch_destroy.argtypes = [vp]
    l.braxg_batch_get_offsets.argtypes = [vp, i32, P(BatchOffsets)]
    l.braxg_batch_launch_info.argtypes = [vp, P(ctypes.c_int32), P(ctypes.c_int32),
                                          P(ctypes.c_int32), P(ctypes.c_int32)]
    l.braxg_batch_init.argtypes = [vp, vp, vp, vp, P(State), P(Options)]
    l.braxg_batch_rollout.argtypes = [vp, vp, i32, vp, P(State), P(State), vp, vp, P(Options)]
    l.braxg_env_rollout.argtypes = [vp, vp, i32, i32, i32, vp, P(State), P(State), P(Task),
                                    P(EnvIO), P(Options)]
    l.braxg_last_error.restype = ctypes.c_char_p
    l.braxg_last_launch_count.restype = ctypes.c_int
    for n in EXPORTS:
      if n not in ('braxg_last_error', 'braxg_last_launch_count',
                   'braxg_rollout_vjp_noalloc_capacity'):
        getattr(l, n).restype = ctypes.c_int
    _lib = l
    return l


def check(rc: int, what: str):
  """Maps a braxg status code onto the exception the reference would raise."""
  if rc == OK:
    return
  msg = f'{what}: {lib().braxg_last_error().decode()}'
  if rc == ERR_INVALID:
    raise ValueError(msg)
  if rc == ERR_UNSUPPORTED:
    raise NotImplementedError(msg)
  raise RuntimeError(msg)
