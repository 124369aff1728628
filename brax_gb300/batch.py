"""Uneven batches: envs of several Systems stepped by one persistent launch.

brax steps one System per jitted function (``jax.vmap`` over envs of the same
System); a batch of different Systems has no counterpart there.  Each model in
a batch keeps the meaning of ``pipeline.init`` / ``pipeline.step`` /
``pipeline.rollout`` for its own envs; the state arrays are flat (every
model's envs one contiguous run of each field) and ``Batch.split`` returns the
per-model views with the single-model shapes.
"""

from __future__ import annotations

import ctypes
from typing import Callable, List, Optional, Sequence

import torch

from brax_gb300 import _native as N
from brax_gb300 import pipeline as P

# field -> (offset class, elements per unit, trailing shape given the dims)
FIELD_CLASS = {
    'q': ('q', 1), 'qd': ('qd', 1), 'mass_mx_inv': ('mass_mx', 1), 'x_pos': ('link', 3),
    'x_rot': ('link', 4), 'xd_ang': ('link', 3), 'xd_vel': ('link', 3),
    'qf_smooth': ('qd', 1), 'qf_constraint': ('qd', 1), 'qdd': ('qd', 1),
    'root_com': ('link', 3), 'cinr_pos': ('link', 3), 'cinr_rot': ('link', 4),
    'cinr_i': ('link', 9), 'cd_packed': ('link', 6), 'cdof_packed': ('qd', 6), 'cdofd_packed': ('qd', 6),
    'mass_mx': ('mass_mx', 1), 'con_jac': ('jac', 1), 'con_diag': ('row', 1),
    'con_aref': ('row', 1), 'status': ('env', 1),
}
BASIC = ('q', 'qd', 'x_pos', 'x_rot', 'xd_ang', 'xd_vel', 'mass_mx_inv', 'qf_smooth',
         'qf_constraint', 'qdd', 'status')


def _shape(m: P.Model, field: str):
  return {
      'q': (m.nq,), 'qd': (m.nv,), 'mass_mx_inv': (m.nv, m.nv), 'x_pos': (m.nl, 3),
      'x_rot': (m.nl, 4), 'xd_ang': (m.nl, 3), 'xd_vel': (m.nl, 3), 'qf_smooth': (m.nv,),
      'qf_constraint': (m.nv,), 'qdd': (m.nv,), 'root_com': (m.nl, 3), 'cinr_pos': (m.nl, 3),
      'cinr_rot': (m.nl, 4), 'cinr_i': (m.nl, 3, 3), 'cd_packed': (m.nl, 6), 'cdof_packed': (m.nv, 6),
      'cdofd_packed': (m.nv, 6), 'mass_mx': (m.nv, m.nv), 'con_jac': (m.m, m.nv), 'con_diag': (m.m,),
      'con_aref': (m.m,), 'status': (),
  }[field]


class Batch:
  """``n_env[g]`` envs of ``systems[g]`` with ``n_frames[g]`` pipeline steps per
  env step, on one device (braxg_batch_create).

  ``shapes``: [(nv_max, threads_per_env, envs_per_cta)], first match per model
  (``brax_gb300.autotune.tune_batch`` picks them); ``smem_per_cta`` 0 = up to
  227 KB per CTA (one CTA per SM).
  """

  def __init__(self, systems: Sequence, n_env: Sequence[int], n_frames: Optional[Sequence[int]] = None,
               shapes=None, smem_per_cta: int = 0, device=None):
    if len(systems) != len(n_env) or not systems:
      raise ValueError('systems and n_env must be non-empty and of equal length')
    self.models: List[P.Model] = [P.model_for(s, device) for s in systems]
    self.device = self.models[0].device
    self.systems = list(systems)
    self.n_env = [int(n) for n in n_env]
    self.n_frames = [1] * len(systems) if n_frames is None else [int(f) for f in n_frames]
    self.shapes = [tuple(int(v) for v in s) for s in (shapes or [])]
    k = len(systems)
    handles = (ctypes.c_void_p * k)(*[m.handle.value for m in self.models])
    ne = (ctypes.c_int32 * k)(*self.n_env)
    nf = (ctypes.c_int32 * k)(*self.n_frames)
    sh = (N.BucketShape * max(1, len(self.shapes)))(
        *[N.BucketShape(a, b, c, 0) for a, b, c in self.shapes])
    h = ctypes.c_void_p()
    lib = N.lib()
    N.check(lib.braxg_batch_create(handles, ne, nf, k, sh, len(self.shapes), int(smem_per_cta),
                                   ctypes.byref(h)), 'braxg_batch_create')
    self._h = h
    self.offsets = []
    for g in range(k + 1):
      o = N.BatchOffsets()
      N.check(lib.braxg_batch_get_offsets(h, g, ctypes.byref(o)), 'braxg_batch_get_offsets')
      self.offsets.append({f: getattr(o, f) for f in N.OFFSET_FIELDS})
    self.totals = self.offsets[-1]

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        N.lib().braxg_batch_destroy(h)
      except Exception:  # interpreter shutdown
        pass
      self._h = None

  @property
  def handle(self):
    return self._h

  @property
  def total_envs(self) -> int:
    return self.totals['env']

  def launch_info(self) -> dict:
    g, b, s, n = (ctypes.c_int32() for _ in range(4))
    N.check(N.lib().braxg_batch_launch_info(self._h, ctypes.byref(g), ctypes.byref(b),
                                            ctypes.byref(s), ctypes.byref(n)),
            'braxg_batch_launch_info')
    return {'grid': g.value, 'block': b.value, 'smem_bytes': s.value, 'n_items': n.value}

  # ---- flat <-> per-model -------------------------------------------------
  def field_size(self, field: str) -> int:
    cls, k = FIELD_CLASS[field]
    return self.totals[cls] * k

  def _span(self, field: str, g: int):
    cls, k = FIELD_CLASS[field]
    return self.offsets[g][cls] * k, self.offsets[g + 1][cls] * k

  def split(self, flat: torch.Tensor, field: str) -> List[torch.Tensor]:
    """Per-model views [n_env[g], ...] of a flat field array."""
    out = []
    for g, m in enumerate(self.models):
      a, b = self._span(field, g)
      out.append(flat[a:b].view(self.n_env[g], *_shape(m, field)))
    return out

  def concat(self, parts: Sequence, field: str) -> torch.Tensor:
    """The flat array of a field from per-model arrays [n_env[g], ...]."""
    dt = torch.int32 if field == 'status' else torch.float32
    return torch.cat([torch.as_tensor(p, dtype=dt).reshape(-1).to(self.device) for p in parts])

  def concat_steps(self, parts: Sequence, field: str) -> torch.Tensor:
    """[n_steps, total] from per-model arrays [n_steps, n_env[g], ...]."""
    dt = torch.float32
    ps = [torch.as_tensor(p, dtype=dt).to(self.device) for p in parts]
    n_steps = ps[0].shape[0]
    return torch.cat([p.reshape(n_steps, -1) for p in ps], dim=1).contiguous()

  def alloc(self, full: bool = False) -> P.State:
    fields = FIELD_CLASS.keys() if full else BASIC
    kw = {}
    for f in FIELD_CLASS:
      if f in fields:
        dt = torch.int32 if f == 'status' else torch.float32
        kw[f] = torch.empty(self.field_size(f), dtype=dt, device=self.device)
      else:
        kw[f] = None
    return P.State(**kw)

  # ---- stepping -----------------------------------------------------------
  def init(self, q: torch.Tensor, qd: torch.Tensor, full: bool = False) -> P.State:
    """pipeline.init for every env (flat q [total q], qd [total qd])."""
    q = q.to(self.device, torch.float32).reshape(-1).contiguous()
    qd = qd.to(self.device, torch.float32).reshape(-1).contiguous()
    if q.numel() != self.totals['q'] or qd.numel() != self.totals['qd']:
      raise ValueError(f'q / qd must hold {self.totals["q"]} / {self.totals["qd"]} values')
    out = self.alloc(full)
    cs = P._cstate(out)
    stream = torch.cuda.current_stream(self.device).cuda_stream
    N.check(N.lib().braxg_batch_init(self._h, ctypes.c_void_p(stream), q.data_ptr(), qd.data_ptr(),
                                     ctypes.byref(cs), ctypes.byref(P._opts(P.NEWTON_SCHULZ, 0, 0))),
            'braxg_batch_init')
    return out

  def rollout(self, state: P.State, act_seq: Optional[torch.Tensor], n_steps: Optional[int] = None,
              inverse_mode: int = P.CHOLESKY, out: Optional[P.State] = None, full: bool = False,
              trajectory: bool = False, profile: Optional[torch.Tensor] = None):
    """n_steps env steps of every env in one launch; act_seq [n_steps, total act]
    (None = no actuation).  Returns (final State, (traj_q, traj_qd))."""
    if act_seq is not None:
      if act_seq.dim() == 1:
        act_seq = act_seq[None]
      act_seq = act_seq.to(self.device, torch.float32).contiguous()
      if act_seq.shape[1] != self.totals['act']:
        raise ValueError(f'act_seq must be (n_steps, {self.totals["act"]})')
      n_steps = act_seq.shape[0] if n_steps is None else n_steps
      if act_seq.shape[0] < n_steps:
        raise ValueError('act_seq holds fewer steps than n_steps')
    n_steps = 1 if n_steps is None else int(n_steps)
    out = self.alloc(full) if out is None else out
    tq = tqd = None
    if trajectory:
      tq = torch.empty(n_steps, self.totals['q'], dtype=torch.float32, device=self.device)
      tqd = torch.empty(n_steps, self.totals['qd'], dtype=torch.float32, device=self.device)
    cin, cout = P._cstate(state), P._cstate(out)
    stream = torch.cuda.current_stream(self.device).cuda_stream
    N.check(N.lib().braxg_batch_rollout(
        self._h, ctypes.c_void_p(stream), n_steps, P._ptr(act_seq), ctypes.byref(cin),
        ctypes.byref(cout), P._ptr(tq), P._ptr(tqd),
        ctypes.byref(P._opts(inverse_mode, 0, 0, profile))), 'braxg_batch_rollout')
    return out, (tq, tqd)

  def step(self, state: P.State, act: Optional[torch.Tensor], inverse_mode: int = P.CHOLESKY,
           out: Optional[P.State] = None) -> P.State:
    return self.rollout(state, act, 1, inverse_mode, out)[0]


class GraphRollout:
  """``n_steps`` env steps of a batch captured as ONE CUDA graph: every step
  runs ``policy(step, state, act)`` (torch ops that fill the static action
  buffer ``act`` [total act] from the static state) and then one batch step
  (a counter memset and one kernel).  ``replay()`` re-runs all n_steps from
  the state in ``self.state``; the final state is in ``self.state`` again.
  """

  def __init__(self, batch: Batch, state: P.State, n_steps: int,
               policy: Callable[[int, P.State, torch.Tensor], None],
               inverse_mode: int = P.CHOLESKY):
    if n_steps < 1:
      raise ValueError('n_steps must be >= 1')
    self.batch = batch
    self.n_steps = n_steps
    self.inverse_mode = inverse_mode
    self.act = torch.zeros(max(1, batch.totals['act']), dtype=torch.float32, device=batch.device)
    self.state = batch.alloc()
    self._other = batch.alloc()
    for f in BASIC:
      getattr(self.state, f).copy_(getattr(state, f))
    self.policy = policy
    # warm-up outside capture (first-call device attributes, torch kernels)
    side = torch.cuda.Stream(batch.device)
    side.wait_stream(torch.cuda.current_stream(batch.device))
    with torch.cuda.stream(side):
      self._body(self._copy_of(self.state), 1)
    torch.cuda.current_stream(batch.device).wait_stream(side)
    torch.cuda.synchronize(batch.device)
    self.graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(self.graph):
      self._body(self.state, n_steps)

  def _copy_of(self, s: P.State) -> P.State:
    c = self.batch.alloc()
    for f in BASIC:
      getattr(c, f).copy_(getattr(s, f))
    return c

  def _body(self, s: P.State, n_steps: int):
    a, b = s, self._other
    for k in range(n_steps):
      self.policy(k, a, self.act)
      self.batch.step(a, self.act if self.batch.totals['act'] else None, self.inverse_mode, out=b)
      a, b = b, a
    if a is not s:  # the final state back into the static input buffers
      for f in BASIC:
        getattr(s, f).copy_(getattr(a, f))

  def replay(self):
    self.graph.replay()
    return self.state
