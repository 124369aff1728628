"""Drop-in for brax.generalized.pipeline (init / step) on the GB300 kernels.

Mirrors brax/generalized/pipeline.py:32-94: ``init(sys, q, qd)`` and
``step(sys, state, act)`` with the same argument meaning, except that arrays
are torch CUDA tensors and may carry a leading batch axis (the axis brax adds
with ``jax.vmap``).  ``state`` fields follow brax/generalized/base.py:25-92.

Every call goes through the braxg C ABI (include/braxg.h); there is no CPU
fallback: without the built CUDA library or a CUDA device the calls raise.
"""

from __future__ import annotations

import ctypes
import dataclasses
from typing import Optional

import torch

from brax_gb300 import _native as N
from brax_gb300 import model_pack
from brax_gb300.system import Inertia, Motion, System, Transform

NEWTON_SCHULZ = N.INV_NEWTON_SCHULZ
CHOLESKY = N.INV_CHOLESKY


class Model:
  """A System resident on one CUDA device (braxg_model_create)."""

  def __init__(self, sys: System, device: Optional[torch.device] = None):
    device = torch.device('cuda') if device is None else torch.device(device)
    if device.type != 'cuda':
      raise RuntimeError('braxg runs on CUDA devices only')
    self.sys = sys
    self.device = torch.device('cuda', device.index if device.index is not None
                               else torch.cuda.current_device())
    self.desc = model_pack.pack(sys)
    h = ctypes.c_void_p()
    lib = N.lib()
    N.check(lib.braxg_model_create(self.desc.ctypes.data, self.desc.nbytes,
                                   self.device.index, ctypes.byref(h)),
            'braxg_model_create')
    self._h = h
    d = N.Dims()
    N.check(lib.braxg_model_dims(h, ctypes.byref(d)), 'braxg_model_dims')
    self.nl, self.nq, self.nv, self.nu = d.nl, d.nq, d.nv, d.nu
    self.ncon, self.nlim, self.m = d.ncon, d.nlim, d.m
    w = ctypes.c_int32()
    N.check(lib.braxg_model_cache_words(h, ctypes.byref(w)), 'braxg_model_cache_words')
    self.cache_words = w.value
    fw, rw, rf = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    N.check(lib.braxg_model_cache_span(h, ctypes.byref(fw), ctypes.byref(rw), ctypes.byref(rf)),
            'braxg_model_cache_span')
    # floats per env a call copies each way: fixed + row_words per active row past rows_in_fixed
    self.cache_span = (fw.value, rw.value, rf.value)

  @property
  def handle(self):
    return self._h

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        N.lib().braxg_model_destroy(h)
      except Exception:  # interpreter shutdown
        pass
      self._h = None

  def launch_shape(self, inverse_mode=NEWTON_SCHULZ, threads_per_env=0, envs_per_cta=0, n_env=0):
    """(threads_per_env, envs_per_cta, smem_bytes) of a call on n_env envs
    (0: the largest CTA)."""
    t, e, s = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    opt = N.Options(inverse_mode, threads_per_env, envs_per_cta)
    N.check(N.lib().braxg_launch_shape(self._h, ctypes.byref(opt), int(n_env), ctypes.byref(t),
                                       ctypes.byref(e), ctypes.byref(s)), 'braxg_launch_shape')
    return t.value, e.value, s.value


_MODELS = {}


def model_for(sys, device=None) -> Model:
  """Returns (and caches) the device-resident Model of a System."""
  if isinstance(sys, Model):
    return sys
  dev = torch.device('cuda') if device is None else torch.device(device)
  idx = dev.index if dev.index is not None else torch.cuda.current_device()
  key = (id(sys), idx)
  m = _MODELS.get(key)
  if m is None or m.sys is not sys:
    m = Model(sys, torch.device('cuda', idx))
    _MODELS[key] = m
  return m


@dataclasses.dataclass
class Contact:
  """brax.base.Contact (brax/base.py:359-368: mujoco.mjx's Contact plus
  link_idx and elasticity) of every contact slot, with the batch axis:
  dist [n, ncon], pos [n, ncon, 3], frame [n, ncon, 3, 3] from the kernel;
  the per-slot constants of the model broadcast over envs."""
  dist: torch.Tensor
  pos: torch.Tensor
  frame: torch.Tensor
  includemargin: torch.Tensor
  friction: torch.Tensor       # [n, ncon, 5]
  solref: torch.Tensor         # [n, ncon, 2]
  solreffriction: torch.Tensor  # [n, ncon, 2] (zero: MuJoCo's default)
  solimp: torch.Tensor         # [n, ncon, 5]
  dim: torch.Tensor            # [n, ncon] condim 3 (pyramid rows)
  geom1: torch.Tensor
  geom2: torch.Tensor
  geom: torch.Tensor           # [n, ncon, 2]
  link_idx: tuple              # ([n, ncon], [n, ncon]); -1 is the world
  elasticity: torch.Tensor     # [n, ncon]


# packed [ang(3), vel(3)] storage of the Motion fields; the C ABI names them
# cd / cdof / cdofd
_PACKED = {'cd': 'cd_packed', 'cdof': 'cdof_packed', 'cdofd': 'cdofd_packed'}


def _motion(t: Optional[torch.Tensor]):
  return None if t is None else Motion(ang=t[..., :3], vel=t[..., 3:])


@dataclasses.dataclass
class State:
  """brax.generalized.base.State with a leading batch axis (torch tensors).

  The reference's nested pytree (brax/generalized/base.py:25-92 on
  brax/base.py:396-412) is available as views of the flat device arrays:
  ``x.pos`` / ``x.rot``, ``xd.ang`` / ``xd.vel``, ``cinr.transform.pos`` /
  ``.rot``, ``cinr.i``, ``cinr.mass``, ``cd`` / ``cdof`` / ``cdofd`` ``.ang`` /
  ``.vel`` (slices of the packed [..., 6] arrays, no copies), and ``contact``
  after a ``debug=True`` call.  Fields that the call did not produce (the
  position-level terms unless ``full=True``) are None."""
  q: torch.Tensor
  qd: torch.Tensor
  x_pos: torch.Tensor
  x_rot: torch.Tensor
  xd_ang: torch.Tensor
  xd_vel: torch.Tensor
  mass_mx_inv: torch.Tensor
  qf_smooth: torch.Tensor
  qf_constraint: torch.Tensor
  qdd: torch.Tensor
  status: torch.Tensor
  root_com: Optional[torch.Tensor] = None
  cinr_pos: Optional[torch.Tensor] = None
  cinr_rot: Optional[torch.Tensor] = None
  cinr_i: Optional[torch.Tensor] = None
  cinr_mass: Optional[torch.Tensor] = None  # [n, nl] the links' masses (constants of the System)
  cd_packed: Optional[torch.Tensor] = None     # [n, nl, 6]
  cdof_packed: Optional[torch.Tensor] = None   # [n, nv, 6]
  cdofd_packed: Optional[torch.Tensor] = None  # [n, nv, 6]
  mass_mx: Optional[torch.Tensor] = None
  con_jac: Optional[torch.Tensor] = None
  con_diag: Optional[torch.Tensor] = None
  con_aref: Optional[torch.Tensor] = None
  contact: Optional[Contact] = None
  # kernel outputs behind ``contact`` (debug=True)
  contact_dist: Optional[torch.Tensor] = None
  contact_pos: Optional[torch.Tensor] = None
  contact_frame: Optional[torch.Tensor] = None
  # [n] int32: pipeline steps of the call whose projected-gradient solve
  # stopped at solver_iterations with its error above tol (``solver_stats``)
  solver_maxiter: Optional[torch.Tensor] = None
  # [n, Model.cache_words] position-level terms of this state, computed by
  # the call that made it; a step from this state reuses them for every env
  # whose q / qd / parameters are unchanged (bit for bit) instead of
  # recomputing them.  Not part of brax's State.
  cache: Optional[torch.Tensor] = None

  def replace(self, **kw) -> 'State':
    return dataclasses.replace(self, **kw)

  # ---- the reference's nested views -------------------------------------
  @property
  def x(self) -> Optional[Transform]:
    return None if self.x_pos is None else Transform(pos=self.x_pos, rot=self.x_rot)

  @property
  def xd(self) -> Optional[Motion]:
    return None if self.xd_ang is None else Motion(ang=self.xd_ang, vel=self.xd_vel)

  @property
  def cinr(self) -> Optional[Inertia]:
    if self.cinr_pos is None:
      return None
    return Inertia(transform=Transform(pos=self.cinr_pos, rot=self.cinr_rot), i=self.cinr_i,
                   mass=self.cinr_mass)

  @property
  def cd(self) -> Optional[Motion]:
    return _motion(self.cd_packed)

  @property
  def cdof(self) -> Optional[Motion]:
    return _motion(self.cdof_packed)

  @property
  def cdofd(self) -> Optional[Motion]:
    return _motion(self.cdofd_packed)


def _alloc(m: Model, n: int, full: bool, dev, cache: bool = False) -> State:
  f = lambda *s: torch.empty(*s, dtype=torch.float32, device=dev)
  s = State(q=f(n, m.nq), qd=f(n, m.nv), x_pos=f(n, m.nl, 3), x_rot=f(n, m.nl, 4),
            xd_ang=f(n, m.nl, 3), xd_vel=f(n, m.nl, 3), mass_mx_inv=f(n, m.nv, m.nv),
            qf_smooth=f(n, m.nv), qf_constraint=f(n, m.nv), qdd=f(n, m.nv),
            status=torch.empty(n, dtype=torch.int32, device=dev),
            cache=f(n, m.cache_words) if cache else None)
  if full:
    mass = torch.as_tensor(m.sys.link.inertia.mass, dtype=torch.float32, device=dev)
    s = s.replace(root_com=f(n, m.nl, 3), cinr_pos=f(n, m.nl, 3), cinr_rot=f(n, m.nl, 4),
                  cinr_i=f(n, m.nl, 3, 3), cinr_mass=mass.reshape(1, m.nl).expand(n, m.nl),
                  cd_packed=f(n, m.nl, 6), cdof_packed=f(n, m.nv, 6),
                  cdofd_packed=f(n, m.nv, 6), mass_mx=f(n, m.nv, m.nv), con_jac=f(n, m.m, m.nv),
                  con_diag=f(n, m.m), con_aref=f(n, m.m))
  return s


def _alloc_contacts(m: Model, s: State) -> State:
  """Adds the debug contact outputs to a state about to be written."""
  n, k = s.q.shape[0], m.ncon
  f = lambda *sh: torch.empty(*sh, dtype=torch.float32, device=s.q.device)
  return s.replace(contact_dist=f(n, k), contact_pos=f(n, k, 3), contact_frame=f(n, k, 3, 3))


def _contact(m: Model, s: State) -> Optional[Contact]:
  """brax.base.Contact of the kernel's contact outputs (None without contact
  slots, as brax/contact.py:39-40)."""
  k = m.ncon
  if k == 0:
    return None
  n, dev = s.q.shape[0], s.q.device
  c = m.sys.contacts

  def const(a, dt=torch.float32):
    t = torch.as_tensor(a, dtype=dt, device=dev)
    return t.reshape(1, *t.shape).expand(n, *t.shape)

  g1, g2 = const(c.geom1, torch.int32), const(c.geom2, torch.int32)
  return Contact(
      dist=s.contact_dist, pos=s.contact_pos, frame=s.contact_frame,
      includemargin=const(torch.zeros(k)), friction=const(c.friction), solref=const(c.solref),
      solreffriction=const(torch.zeros(k, 2)), solimp=const(c.solimp),
      dim=const(torch.full((k,), 3), torch.int32), geom1=g1, geom2=g2, geom=torch.stack([g1, g2], -1),
      link_idx=(const(c.link_a, torch.int32), const(c.link_b, torch.int32)),
      elasticity=const(c.elasticity))


def _ptr(t):
  return None if t is None else t.data_ptr()


def _cstate(s: State) -> N.State:
  return N.State(*[_ptr(getattr(s, _PACKED.get(f, f))) for f in N.STATE_FIELDS])


def _as_batch(x: torch.Tensor, width: int, name: str, dev) -> torch.Tensor:
  if not isinstance(x, torch.Tensor):
    x = torch.as_tensor(x)
  if x.dim() == 1:
    x = x[None]
  if x.dim() != 2 or x.shape[1] != width:
    raise ValueError(f'{name} must have shape (..., {width}), got {tuple(x.shape)}')
  if x.device != dev:
    raise ValueError(f'{name} is on {x.device}, the model on {dev}')
  return x.to(torch.float32).contiguous()


_DR_FIELDS = N.RANDOMIZATION_FIELDS


def _dr_width(m: 'Model', k: str) -> int:
  return {'friction': m.ncon, 'link_mass': m.nl, 'link_inertia': 9 * m.nl, 'dof_armature': m.nv,
          'dof_damping': m.nv, 'dof_stiffness': m.nv}.get(k, m.nu)


def _randomization(m: 'Model', n: int, randomization):
  """A C Randomization struct for a dict of per-env tensors (friction
  [n, ncon]; act_gain / act_bias_q / act_bias_qd [n, nu]; link_mass [n, nl];
  link_inertia [n, nl, 3, 3]; dof_armature / dof_damping / dof_stiffness
  [n, nv]), with the tensors it points to (kept alive by the caller for the
  call)."""
  if not randomization:
    return None, []
  keep = []
  ptrs = {}
  for k, v in randomization.items():
    if k not in _DR_FIELDS:
      raise ValueError(f'unknown randomization field {k!r}; expected one of {_DR_FIELDS}')
    v = torch.as_tensor(v, dtype=torch.float32, device=m.device).reshape(n, _dr_width(m, k)).contiguous()
    keep.append(v)
    ptrs[k] = v.data_ptr()
  return N.Randomization(*[ptrs.get(k) for k in _DR_FIELDS]), keep


def randomize(sys, n: int, generator: Optional[torch.Generator] = None, friction_range=(0.6, 1.4),
              gain_scale_range=(1.0, 1.0), mass_scale_range=(1.0, 1.0), damping_scale_range=(1.0, 1.0),
              device=None) -> dict:
  """Per-env parameters in the manner of brax's domain randomisation
  examples: one sliding friction per env, uniform in friction_range, for
  every contact slot (every geom gets it, so every pair's mixed friction is
  it); the actuator gains scaled by a per-env factor; the link masses and
  inertias scaled together by a per-env factor (a uniformly denser body); the
  dof damping scaled by a per-env factor."""
  m = model_for(sys, device)
  dev = m.device

  def scale(rng):
    g = torch.rand(n, 1, device=dev, generator=generator)
    return rng[0] + (rng[1] - rng[0]) * g

  f = scale(friction_range)
  out = {'friction': f.expand(n, m.ncon).contiguous()}
  if m.nu and gain_scale_range != (1.0, 1.0):
    gain = torch.tensor(sys.actuator.gain, dtype=torch.float32, device=dev)[None]
    out['act_gain'] = (gain * scale(gain_scale_range)).contiguous()
  if mass_scale_range != (1.0, 1.0):
    s = scale(mass_scale_range)
    mass = torch.tensor(sys.link.inertia.mass, dtype=torch.float32, device=dev)[None]
    inertia = torch.tensor(sys.link.inertia.i, dtype=torch.float32, device=dev).reshape(1, -1)
    out['link_mass'] = (mass * s).contiguous()
    out['link_inertia'] = (inertia * s).reshape(n, m.nl, 3, 3).contiguous()
  if damping_scale_range != (1.0, 1.0):
    damp = torch.tensor(sys.dof.damping, dtype=torch.float32, device=dev)[None]
    out['dof_damping'] = (damp * scale(damping_scale_range)).contiguous()
  return out


def _opts(inverse_mode, threads_per_env, envs_per_cta, profile=None, relax_barriers=0, dr=None):
  o = N.Options(int(inverse_mode), int(threads_per_env), int(envs_per_cta), int(relax_barriers),
                None if profile is None else profile.data_ptr())
  if dr is not None:
    o.randomization = ctypes.pointer(dr)
  return o


def profile_buffer(device=None) -> torch.Tensor:
  """A zeroed per-stage profile buffer to pass as ``profile=``."""
  return torch.zeros(N.N_PROFILE_SLOTS, dtype=torch.int64,
                     device=device if device is not None else 'cuda')


def profile_report(buf: torch.Tensor) -> dict:
  v = buf.cpu().tolist()
  out = {k: v[i] for i, k in enumerate(N.PROFILE_SLOTS)}
  out.update({k: v[i] for i, k in N.VJP_PROFILE_SLOTS.items() if v[i]})
  return out


def init(sys, q, qd, unused_act=None, unused_ctrl=None, debug: bool = False,
         full: bool = False, threads_per_env: int = 0, envs_per_cta: int = 0,
         randomization: Optional[dict] = None, cache: bool = True) -> State:
  """brax/generalized/pipeline.py:32-61 for a batch of envs.  ``cache``
  gives the state (and the states stepped from it) a position-term cache;
  ``debug`` adds ``state.contact`` (contact.get of the state, as the
  reference's debug flag does)."""
  m = model_for(sys, q.device if isinstance(q, torch.Tensor) else None)
  q = _as_batch(q, m.nq, 'q', m.device)
  qd = _as_batch(qd, m.nv, 'qd', m.device)
  if q.shape[0] != qd.shape[0]:
    raise ValueError('q and qd batch sizes differ')
  out = _alloc(m, q.shape[0], full, m.device, cache)
  if debug:
    out = _alloc_contacts(m, out)
  cs = _cstate(out)
  dr, _keep = _randomization(m, q.shape[0], randomization)
  stream = torch.cuda.current_stream(m.device).cuda_stream
  N.check(N.lib().braxg_init(m.handle, ctypes.c_void_p(stream), q.shape[0], q.data_ptr(),
                             qd.data_ptr(), ctypes.byref(cs),
                             ctypes.byref(_opts(NEWTON_SCHULZ, threads_per_env, envs_per_cta, dr=dr))),
          'braxg_init')
  return out.replace(contact=_contact(m, out)) if debug else out


def bare_state(q: torch.Tensor, qd: torch.Tensor) -> State:
  """A State holding only q and qd: the input of an exact-inverse
  (``CHOLESKY``) step or rollout, which reads nothing else of its input state
  (a Newton-Schulz step also needs the carried ``mass_mx_inv``)."""
  if q.dim() != 2 or qd.dim() != 2 or q.shape[0] != qd.shape[0]:
    raise ValueError('q and qd must be [n, nq] and [n, nv]')
  return State(q=q.to(torch.float32).contiguous(), qd=qd.to(torch.float32).contiguous(), x_pos=None,
               x_rot=None, xd_ang=None, xd_vel=None, mass_mx_inv=None, qf_smooth=None, qf_constraint=None,
               qdd=None, status=None)


def step(sys, state: State, act, debug: bool = False, n_frames: int = 1,
         full: bool = False, inverse_mode: int = NEWTON_SCHULZ, out: Optional[State] = None,
         threads_per_env: int = 0, envs_per_cta: int = 0,
         profile: Optional[torch.Tensor] = None, relax_barriers: int = 0,
         randomization: Optional[dict] = None, solver_stats: bool = False) -> State:
  """brax/generalized/pipeline.py:64-94; n_frames > 1 repeats it with the same
  action (PipelineEnv.pipeline_step, brax/envs/base.py:128-137).  ``debug``
  adds ``state.contact`` of the output state; ``solver_stats`` fills
  ``state.solver_maxiter``."""
  m = model_for(sys, state.q.device)
  n = state.q.shape[0]
  act_p = None
  if act is not None and m.nu > 0:
    act = _as_batch(act, m.nu, 'act', m.device)
    if act.shape[0] != n:
      raise ValueError(f'act batch {act.shape[0]} != state batch {n}')
    act_p = act.data_ptr()
  if out is None:
    out = _alloc(m, n, full, m.device, state.cache is not None)
  if solver_stats and out.solver_maxiter is None:
    out = out.replace(solver_maxiter=torch.empty(n, dtype=torch.int32, device=m.device))
  if debug and out.contact_dist is None:
    out = _alloc_contacts(m, out)
  elif not debug and (out.contact_dist is not None or out.contact is not None):
    out = out.replace(contact=None, contact_dist=None, contact_pos=None, contact_frame=None)
  cin = _cstate(state)
  cout = _cstate(out)
  dr, _keep = _randomization(m, n, randomization)
  stream = torch.cuda.current_stream(m.device).cuda_stream
  N.check(N.lib().braxg_step(m.handle, ctypes.c_void_p(stream), n, int(n_frames), act_p,
                             ctypes.byref(cin), ctypes.byref(cout),
                             ctypes.byref(_opts(inverse_mode, threads_per_env, envs_per_cta,
                                                profile, relax_barriers, dr))),
          'braxg_step')
  return out.replace(contact=_contact(m, out)) if debug else out


def rollout(sys, state: State, act_seq, n_frames: int = 1, inverse_mode: int = NEWTON_SCHULZ,
            trajectory: bool = False, threads_per_env: int = 0, envs_per_cta: int = 0,
            randomization: Optional[dict] = None):
  """len(act_seq) env steps in one launch; returns (final State, (traj_q, traj_qd))."""
  m = model_for(sys, state.q.device)
  n = state.q.shape[0]
  act_seq = act_seq.to(torch.float32).contiguous()
  if act_seq.dim() != 3 or act_seq.shape[1] != n or act_seq.shape[2] != m.nu:
    raise ValueError(f'act_seq must be (n_steps, {n}, {m.nu})')
  n_steps = act_seq.shape[0]
  out = _alloc(m, n, False, m.device, state.cache is not None)
  tq = tqd = None
  if trajectory:
    tq = torch.empty(n_steps, n, m.nq, dtype=torch.float32, device=m.device)
    tqd = torch.empty(n_steps, n, m.nv, dtype=torch.float32, device=m.device)
  cin, cout = _cstate(state), _cstate(out)
  dr, _keep = _randomization(m, n, randomization)
  stream = torch.cuda.current_stream(m.device).cuda_stream
  N.check(N.lib().braxg_rollout(m.handle, ctypes.c_void_p(stream), n, n_steps, int(n_frames),
                                act_seq.data_ptr() if m.nu else None, ctypes.byref(cin),
                                ctypes.byref(cout), _ptr(tq), _ptr(tqd),
                                ctypes.byref(_opts(inverse_mode, threads_per_env, envs_per_cta,
                                                   dr=dr))),
          'braxg_rollout')
  return out, (tq, tqd)


def rollout_grad(sys, q0, qd0, act_seq, q_bar=None, qd_bar=None, n_frames: int = 1,
                 ckpt_every: int = 16, trajectory: bool = False,
                 profile: Optional[torch.Tensor] = None, resident_segments: Optional[int] = None,
                 inverse_mode: int = CHOLESKY):
  """Reverse-mode gradient of a rollout through the hand-written adjoint.

  Replaces ``jax.grad`` through ``lax.scan`` of ``pipeline_step``
  (brax/training/agents/apg/train.py:188-198).  ``q_bar`` / ``qd_bar``
  [n_steps, n, nq|nv] are the loss cotangents of the state after every env step.
  ``resident_segments``: checkpoint segments whose frame snapshots stay
  resident from the checkpoint pass (the others are recomputed); None keeps
  as many as fit a quarter of the free device memory.  ``inverse_mode``
  NEWTON_SCHULZ differentiates the reference's carried Newton-Schulz inverse
  (exact at the first frame, as init computes it); CHOLESKY the exact one.
  Returns (act_bar, q0_bar, qd0_bar, status, (traj_q, traj_qd)).
  """
  m = model_for(sys, q0.device)
  q0 = _as_batch(q0, m.nq, 'q0', m.device)
  qd0 = _as_batch(qd0, m.nv, 'qd0', m.device)
  n = q0.shape[0]
  act_seq = act_seq.to(torch.float32).contiguous()
  if act_seq.dim() != 3 or act_seq.shape[1] != n or act_seq.shape[2] != m.nu:
    raise ValueError(f'act_seq must be (n_steps, {n}, {m.nu})')
  n_steps = act_seq.shape[0]
  dev = m.device
  f = lambda *s: torch.zeros(*s, dtype=torch.float32, device=dev)
  qb = None if q_bar is None else q_bar.to(torch.float32).contiguous()
  qdb = None if qd_bar is None else qd_bar.to(torch.float32).contiguous()
  act_bar, q0_bar, qd0_bar = f(n_steps, n, m.nu), f(n, m.nq), f(n, m.nv)
  tq = tqd = None
  if trajectory:
    tq, tqd = f(n_steps, n, m.nq), f(n_steps, n, m.nv)
  status = torch.zeros(n, dtype=torch.int32, device=dev)
  lib = N.lib()
  ws, nbytes = _vjp_workspace(m, n, n_steps, n_frames, ckpt_every, resident_segments, inverse_mode)
  stream = torch.cuda.current_stream(dev).cuda_stream
  N.check(lib.braxg_rollout_vjp(
      m.handle, ctypes.c_void_p(stream), n, n_steps, int(n_frames), int(ckpt_every),
      act_seq.data_ptr() if m.nu else None, q0.data_ptr(), qd0.data_ptr(), _ptr(qb), _ptr(qdb),
      act_bar.data_ptr() if m.nu else None, q0_bar.data_ptr(), qd0_bar.data_ptr(), _ptr(tq),
      _ptr(tqd), ws.data_ptr(), nbytes, status.data_ptr(),
      ctypes.byref(_opts(inverse_mode, 0, 0, profile))), 'braxg_rollout_vjp')
  return act_bar, q0_bar, qd0_bar, status, (tq, tqd)


def _vjp_workspace(m: 'Model', n: int, n_steps: int, n_frames: int, ckpt_every: int,
                   resident_segments: Optional[int], inverse_mode: int = CHOLESKY):
  """(workspace tensor, bytes) of a gradient launch; resident_segments None
  keeps as many checkpoint segments resident as fit a quarter of the free
  device memory."""
  lib = N.lib()
  nbytes = ctypes.c_size_t()
  n_ckpt = (n_steps + int(ckpt_every) - 1) // int(ckpt_every)
  size = lambda r: lib.braxg_rollout_vjp_workspace_mode(m.handle, n, n_steps, int(n_frames), int(ckpt_every), int(r),
                                                        int(inverse_mode), ctypes.byref(nbytes))
  if resident_segments is None:
    free = torch.cuda.mem_get_info(m.device)[0]
    resident_segments = 1
    for r in range(n_ckpt, 0, -1):
      N.check(size(r), 'workspace')
      if nbytes.value <= free // 4:
        resident_segments = r
        break
  N.check(size(resident_segments), 'braxg_rollout_vjp_workspace_mode')
  return torch.empty(max(nbytes.value, 4), dtype=torch.uint8, device=m.device), nbytes.value


@dataclasses.dataclass
class VjpTape:
  """What rollout_vjp_fwd leaves for rollout_vjp_bwd: the inputs, the sizes
  and the workspace holding the forward's checkpoints and frame snapshots
  (the residuals of a jax.custom_vjp forward)."""
  model: 'Model'
  q0: torch.Tensor
  qd0: torch.Tensor
  act_seq: torch.Tensor
  n_frames: int
  ckpt_every: int
  workspace: torch.Tensor
  nbytes: int
  status: torch.Tensor
  inverse_mode: int = CHOLESKY


def rollout_vjp_fwd(sys, q0, qd0, act_seq, n_frames: int = 1, ckpt_every: int = 16,
                    resident_segments: Optional[int] = None, inverse_mode: int = CHOLESKY):
  """The forward half of rollout_grad (braxg_rollout_vjp_fwd): the rollout's
  trajectory (traj_q [n_steps, n, nq], traj_qd [n_steps, n, nv]) and a
  VjpTape for rollout_vjp_bwd.  The two halves give bitwise the result of
  one rollout_grad call, and the reverse does not re-run the forward."""
  m = model_for(sys, q0.device)
  q0 = _as_batch(q0, m.nq, 'q0', m.device)
  qd0 = _as_batch(qd0, m.nv, 'qd0', m.device)
  n = q0.shape[0]
  act_seq = act_seq.to(torch.float32).contiguous()
  if act_seq.dim() != 3 or act_seq.shape[1] != n or act_seq.shape[2] != m.nu:
    raise ValueError(f'act_seq must be (n_steps, {n}, {m.nu})')
  n_steps = act_seq.shape[0]
  ws, nbytes = _vjp_workspace(m, n, n_steps, n_frames, ckpt_every, resident_segments, inverse_mode)
  tq = torch.empty(n_steps, n, m.nq, dtype=torch.float32, device=m.device)
  tqd = torch.empty(n_steps, n, m.nv, dtype=torch.float32, device=m.device)
  status = torch.zeros(n, dtype=torch.int32, device=m.device)
  stream = torch.cuda.current_stream(m.device).cuda_stream
  N.check(N.lib().braxg_rollout_vjp_fwd(
      m.handle, ctypes.c_void_p(stream), n, n_steps, int(n_frames), int(ckpt_every),
      act_seq.data_ptr() if m.nu else None, q0.data_ptr(), qd0.data_ptr(), tq.data_ptr(), tqd.data_ptr(),
      ws.data_ptr(), nbytes, status.data_ptr(), ctypes.byref(_opts(inverse_mode, 0, 0))), 'braxg_rollout_vjp_fwd')
  return (tq, tqd), VjpTape(m, q0, qd0, act_seq, int(n_frames), int(ckpt_every), ws, nbytes, status,
                            int(inverse_mode))


def rollout_vjp_bwd(tape: VjpTape, q_bar=None, qd_bar=None):
  """The reverse half (braxg_rollout_vjp_bwd) on a VjpTape: q_bar / qd_bar
  [n_steps, n, nq|nv] (None = zero) -> (act_bar, q0_bar, qd0_bar, status)."""
  m, n, n_steps = tape.model, tape.q0.shape[0], tape.act_seq.shape[0]
  f = lambda *sh: torch.zeros(*sh, dtype=torch.float32, device=m.device)
  qb = None if q_bar is None else q_bar.to(torch.float32).contiguous()
  qdb = None if qd_bar is None else qd_bar.to(torch.float32).contiguous()
  act_bar, q0_bar, qd0_bar = f(n_steps, n, m.nu), f(n, m.nq), f(n, m.nv)
  stream = torch.cuda.current_stream(m.device).cuda_stream
  N.check(N.lib().braxg_rollout_vjp_bwd(
      m.handle, ctypes.c_void_p(stream), n, n_steps, tape.n_frames, tape.ckpt_every,
      tape.act_seq.data_ptr() if m.nu else None, tape.q0.data_ptr(), tape.qd0.data_ptr(), _ptr(qb), _ptr(qdb),
      act_bar.data_ptr() if m.nu else None, q0_bar.data_ptr(), qd0_bar.data_ptr(), tape.workspace.data_ptr(),
      tape.nbytes, tape.status.data_ptr(), ctypes.byref(_opts(tape.inverse_mode, 0, 0))), 'braxg_rollout_vjp_bwd')
  return act_bar, q0_bar, qd0_bar, tape.status


class Rollout(torch.autograd.Function):
  """Differentiable rollout for torch: (q0, qd0, act_seq) -> (traj_q, traj_qd).

  The forward runs braxg_rollout_vjp_fwd (the checkpoints and frame
  snapshots stay in a workspace held by the graph); the backward runs the
  hand-written reverse on it (braxg_rollout_vjp_bwd).
  """

  @staticmethod
  def forward(ctx, q0, qd0, act_seq, sys, n_frames, ckpt_every, inverse_mode=CHOLESKY):
    (tq, tqd), ctx.tape = rollout_vjp_fwd(sys, q0.detach(), qd0.detach(), act_seq.detach(), n_frames=n_frames,
                                          ckpt_every=ckpt_every, inverse_mode=inverse_mode)
    return tq, tqd

  @staticmethod
  def backward(ctx, gq, gqd):
    act_bar, q0_bar, qd0_bar, _ = rollout_vjp_bwd(ctx.tape, gq, gqd)
    return q0_bar, qd0_bar, act_bar, None, None, None, None


def differentiable_rollout(sys, q0, qd0, act_seq, n_frames: int = 1, ckpt_every: int = 16,
                           inverse_mode: int = CHOLESKY):
  """torch.autograd-enabled rollout returning (traj_q, traj_qd).  With a
  gradient to take, the forward is braxg_rollout_vjp_fwd (its checkpoints and
  frame snapshots kept for the backward, which runs only the reverse);
  without one, a plain braxg_rollout.  inverse_mode CHOLESKY computes the
  exact inverse every frame; NEWTON_SCHULZ carries pipeline.init's exact
  inverse through the reference's Newton-Schulz update (and differentiates
  it)."""
  if torch.is_grad_enabled() and any(t.requires_grad for t in (q0, qd0, act_seq)):
    return Rollout.apply(q0, qd0, act_seq, sys, n_frames, ckpt_every, int(inverse_mode))
  s0 = bare_state(q0, qd0) if inverse_mode == CHOLESKY else init(sys, q0, qd0)
  _, (tq, tqd) = rollout(sys, s0, act_seq, n_frames=n_frames, inverse_mode=inverse_mode, trajectory=True)
  return tq, tqd
