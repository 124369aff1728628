"""Batched numpy restatement of brax.generalized.pipeline.init/step.

TEST INFRASTRUCTURE ONLY (the checker / the timed CPU restatement).

Every function cites the reference file:line it follows.  Arrays carry a
leading batch axis B (the reference's ``jax.vmap`` axis).  ``dtype`` selects
float32 (the reference's default) or float64 (``jax_enable_x64``).
"""

from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from brax_gb300 import system as S

# ---------------------------------------------------------------------------
# math primitives: brax/math.py
# ---------------------------------------------------------------------------


def cross(a, b):
  return np.cross(a, b)


def dot(a, b):
  return np.sum(a * b, axis=-1)


def rotate(v, q):
  """brax/math.py:25-40."""
  s, u = q[..., 0:1], q[..., 1:]
  r = 2 * (dot(u, v)[..., None] * u) + (s * s - dot(u, u)[..., None]) * v
  return r + 2 * s * cross(u, v)


def quat_mul(u, v):
  """brax/math.py:86-101."""
  return np.stack([
      u[..., 0] * v[..., 0] - u[..., 1] * v[..., 1] - u[..., 2] * v[..., 2] - u[..., 3] * v[..., 3],
      u[..., 0] * v[..., 1] + u[..., 1] * v[..., 0] + u[..., 2] * v[..., 3] - u[..., 3] * v[..., 2],
      u[..., 0] * v[..., 2] - u[..., 1] * v[..., 3] + u[..., 2] * v[..., 0] + u[..., 3] * v[..., 1],
      u[..., 0] * v[..., 3] + u[..., 1] * v[..., 2] - u[..., 2] * v[..., 1] + u[..., 3] * v[..., 0],
  ], axis=-1)


def quat_inv(q):
  """brax/math.py:122-131."""
  return q * np.array([1, -1, -1, -1], dtype=q.dtype)


def quat_rot_axis(axis, angle):
  """brax/math.py:134-148; axis (..., 3), angle (...)."""
  s = np.sin(angle / 2)
  return np.stack([np.cos(angle / 2), axis[..., 0] * s, axis[..., 1] * s,
                   axis[..., 2] * s], axis=-1)


def quat_to_3x3(q):
  """brax/math.py:151-165."""
  d = dot(q, q)
  w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
  s = 2 / d
  xs, ys, zs = x * s, y * s, z * s
  wx, wy, wz = w * xs, w * ys, w * zs
  xx, xy, xz = x * xs, x * ys, x * zs
  yy, yz, zz = y * ys, y * zs, z * zs
  return np.stack([
      np.stack([1 - (yy + zz), xy - wz, xz + wy], -1),
      np.stack([xy + wz, 1 - (xx + zz), yz - wx], -1),
      np.stack([xz - wy, yz + wx, 1 - (xx + yy)], -1),
  ], -2)


def safe_norm(x, nd=1):
  """brax/math.py:308-328 over the trailing ``nd`` axes (allclose: atol 1e-8)."""
  axes = tuple(range(-nd, 0))
  is_zero = np.all(np.abs(x) <= 1e-8, axis=axes).astype(x.dtype)
  xs = x + is_zero.reshape(is_zero.shape + (1,) * nd) * 1.0
  return np.sqrt(np.sum(xs * xs, axis=axes)) * (1 - is_zero)


def normalize(x):
  """brax/math.py:331-345, trailing axis."""
  n = safe_norm(x)
  return x / (n + 1e-6 * (n == 0.0).astype(x.dtype))[..., None]


def orthogonals(a):
  """brax/math.py:247-254 (identical in mujoco.mjx math)."""
  dt = a.dtype
  y = np.array([0, 1, 0], dtype=dt)
  z = np.array([0, 0, 1], dtype=dt)
  sel = ((-0.5 < a[..., 1]) & (a[..., 1] < 0.5))[..., None]
  b = np.where(sel, y, z)
  b = b - a * dot(a, b)[..., None]
  b = normalize(b) * np.any(a != 0, axis=-1, keepdims=True).astype(dt)
  return b, cross(a, b)


def make_frame(a):
  """mujoco.mjx math.make_frame: rows (normal, tangent1, tangent2)."""
  a = normalize(a)
  b, c = orthogonals(a)
  return np.stack([a, b, c], axis=-2)


def _norm_with_norm(x):
  """mujoco.mjx math.normalize_with_norm (plain norm, 1e-6 guard at 0)."""
  n = np.sqrt(dot(x, x))
  return x / (n + 1e-6 * (n == 0.0).astype(x.dtype))[..., None], n


# spatial algebra: brax/base.py:546-614 ---------------------------------------


def tf_do_tf(ap, ar, bp, br):
  """Transform.do(Transform), brax/base.py:566-570."""
  return ap + rotate(bp, ar), quat_mul(ar, br)


def motion_cross(s_ang, s_vel, o_ang, o_vel):
  """self.cross(other) for Motions, brax/base.py:604-608."""
  return cross(s_ang, o_ang), cross(s_ang, o_vel) + cross(s_vel, o_ang)


def force_cross(s_ang, s_vel, f_ang, f_vel):
  """Motion x Force, brax/base.py:611-614 -> (ang, vel)."""
  return cross(s_ang, f_ang) + cross(s_vel, f_vel), cross(s_ang, f_vel)


def inertia_mul(i, tpos, mass, m_ang, m_vel):
  """Inertia.mul, brax/base.py:297-302 -> Force (ang, vel)."""
  ang = np.einsum('...ij,...j->...i', i, m_ang) + cross(tpos, m_vel)
  vel = mass[..., None] * m_vel - cross(tpos, m_ang)
  return ang, vel


# ---------------------------------------------------------------------------
# model-derived static structure (brax/scan.py level order, System helpers)
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class _Static:
  nl: int
  nq: int
  nv: int
  types: str
  parents: tuple
  levels: list
  qadr: list
  dadr: list
  dof_link: np.ndarray
  children: list
  roots: list


def static(sys: S.System) -> _Static:
  nl = sys.num_links()
  depth = sys.link_depth()
  levels = [[] for _ in range(max(depth) + 1 if nl else 0)]
  for i in range(nl):
    levels[depth[i]].append(i)
  qadr, dadr = [], []
  qa = da = 0
  for t in sys.link_types:
    qadr.append(qa)
    dadr.append(da)
    qa += S.Q_WIDTHS[t]
    da += S.QD_WIDTHS[t]
  children = [[c for c in range(nl) if sys.link_parents[c] == i] for i in range(nl)]
  roots = sys.link_root()
  return _Static(nl, qa, da, sys.link_types, tuple(sys.link_parents), levels,
                 qadr, dadr, sys.dof_link(), children, roots)


@dataclasses.dataclass
class State:
  """brax/generalized/base.py:25-92 (+ base.State q, qd, x, xd)."""
  q: np.ndarray
  qd: np.ndarray
  x_pos: np.ndarray
  x_rot: np.ndarray
  xd_ang: np.ndarray
  xd_vel: np.ndarray
  root_com: Optional[np.ndarray] = None
  cinr_pos: Optional[np.ndarray] = None   # cinr.transform.pos (= offset * mass)
  cinr_rot: Optional[np.ndarray] = None
  cinr_i: Optional[np.ndarray] = None
  cinr_mass: Optional[np.ndarray] = None
  cd_ang: Optional[np.ndarray] = None
  cd_vel: Optional[np.ndarray] = None
  cdof_ang: Optional[np.ndarray] = None
  cdof_vel: Optional[np.ndarray] = None
  cdofd_ang: Optional[np.ndarray] = None
  cdofd_vel: Optional[np.ndarray] = None
  mass_mx: Optional[np.ndarray] = None
  mass_mx_inv: Optional[np.ndarray] = None
  con_jac: Optional[np.ndarray] = None
  con_diag: Optional[np.ndarray] = None
  con_aref: Optional[np.ndarray] = None
  qf_smooth: Optional[np.ndarray] = None
  qf_constraint: Optional[np.ndarray] = None
  qdd: Optional[np.ndarray] = None
  # diagnostics of the last constraint solve
  contact_dist: Optional[np.ndarray] = None
  pg_matvecs: Optional[np.ndarray] = None
  pg_maxiter: Optional[np.ndarray] = None  # the solve stopped at maxiter with err > tol
  pg_err: Optional[np.ndarray] = None      # its final stopping error

  def replace(self, **kw):
    return dataclasses.replace(self, **kw)


class Oracle:
  """Holds a System cast to ``dtype`` plus its static schedule."""

  # half-width, in ulps of the operands' magnitude, of the decision margin
  # of the rounding envelope (about sqrt(n) for sums of tens of terms)
  DECISION_ULPS = 8

  # evaluation orders of the dense products (see __init__)
  ORDERS = ('reference', 'right', 'rounded', 'fma')

  def __init__(self, sys: S.System, dtype=np.float64, exact_inverse: bool = False, perturb_seed=None,
               perturb_bias: int = 0, order: str = 'reference'):
    """exact_inverse=True replaces the Newton-Schulz update of mass_mx_inv by
    the exact SPD inverse (the kernel's Cholesky mode); the reference path is
    exact_inverse=False.

    perturb_seed (for the parity tests' rounding envelope): when set, every
    step moves the intermediates whose rounding depends on the summation
    order (the link poses and velocities of forward kinematics, the
    constraint rows' Jacobian, diagonal and reference acceleration,
    qf_smooth, the mass matrix, mass_mx_inv and the Newton-Schulz iterates,
    and the projected-gradient problem's A and b; the symmetric ones
    symmetrically)
    by -1, 0 or +1 ulp at random, and every discrete decision
    taken on two computed values (the line search's sufficient-decrease test,
    the solver's stopping test, the Newton-Schulz acceptance and reset tests,
    the capsule-capsule closest-point choice) sees its two sides shifted by
    up to DECISION_ULPS ulps of their magnitude: decisions whose sides agree
    that closely may go either way in another operation order.
    perturb_bias -1 / +1 shifts every such decision the same way (a draw
    biased to one side), 0 draws each shift at random.  This emulates an
    evaluation of the same algorithm in another operation order; it is not
    part of the reference's algorithm.

    order (also for the envelope; float32 only): how the dense products
    whose terms cancel are evaluated -- J Minv J^T and J Minv qf_smooth of
    the constraint problem, Minv (qf_smooth + qf_constraint) of the
    integrator, the Newton-Schulz products and the exact inverse.
    'reference' associates them as the reference's code does ((J Minv) J^T)
    in numpy's summation order; 'right' associates them the other way
    (J (Minv J^T)); 'rounded' evaluates each in float64 and rounds once (the
    correctly rounded FP32 result); 'fma' sums every dot product as two
    interleaved chains of fused multiply-adds (even and odd terms, added at
    the end), as vectorised hardware commonly does.  Each is an exact
    evaluation of the same formula; on ill-conditioned models (long hanging
    chains: mass matrices of condition 1e4) they differ by far more than one
    ulp of the result."""
    if order not in self.ORDERS:
      raise ValueError(f'order must be one of {self.ORDERS}')
    self.order = order if np.dtype(dtype) == np.float32 else 'reference'
    self.sys = sys
    self.exact_inverse = exact_inverse
    self._rng = None if perturb_seed is None else np.random.default_rng(perturb_seed)
    self._bias = perturb_bias
    self.dt_ = np.dtype(dtype)
    self.st = static(sys)
    f = lambda a: np.asarray(a, dtype=self.dt_)
    self.c = dict(
        gravity=f(sys.gravity), dt=self.dt_.type(sys.dt),
        lt_pos=f(sys.link.transform.pos), lt_rot=f(sys.link.transform.rot),
        lj_pos=f(sys.link.joint.pos), lj_rot=f(sys.link.joint.rot),
        li_pos=f(sys.link.inertia.transform.pos), li_rot=f(sys.link.inertia.transform.rot),
        li_i=f(sys.link.inertia.i), li_mass=f(sys.link.inertia.mass),
        l_invw=f(sys.link.invweight),
        m_ang=f(sys.dof.motion.ang), m_vel=f(sys.dof.motion.vel),
        armature=f(sys.dof.armature), stiffness=f(sys.dof.stiffness),
        damping=f(sys.dof.damping), d_invw=f(sys.dof.invweight),
        solp=f(sys.dof.solver_params),
        lo=None if sys.dof.limit is None else f(sys.dof.limit[0]),
        hi=None if sys.dof.limit is None else f(sys.dof.limit[1]),
        geom_pos=f(sys.geom_pos), geom_quat=f(sys.geom_quat), geom_size=f(sys.geom_size),
        c_fric=f(sys.contacts.friction), c_solref=f(sys.contacts.solref),
        c_solimp=f(sys.contacts.solimp),
        a_cr=f(sys.actuator.ctrl_range), a_fr=f(sys.actuator.force_range),
        a_gain=f(sys.actuator.gain), a_gear=f(sys.actuator.gear),
        a_bq=f(sys.actuator.bias_q), a_bqd=f(sys.actuator.bias_qd),
        viscosity=self.dt_.type(sys.viscosity), density=self.dt_.type(sys.density))
    self.matvecs = 0

  def _margin(self, scale):
    """Shift of a decision's comparison (zero unless perturbing): up to
    DECISION_ULPS ulps of `scale` (the magnitude of the compared values)."""
    if self._rng is None:
      return np.zeros_like(scale)
    u = self._rng.uniform(-1, 1, np.shape(scale)) if self._bias == 0 else float(self._bias)
    return (u * self.DECISION_ULPS * np.finfo(self.dt_).eps * np.abs(scale)).astype(self.dt_)

  def _nudge(self, x, symmetric=False):
    """x moved by -1, 0 or +1 ulp per entry (identity unless perturbing)."""
    if self._rng is None:
      return x
    d = self._rng.integers(-1, 2, x.shape)
    if symmetric:  # the same move for (i, j) and (j, i)
      d = np.tril(d) + np.swapaxes(np.tril(d, -1), -1, -2)
    up, dn = np.nextafter(x, self.dt_.type(np.inf)), np.nextafter(x, self.dt_.type(-np.inf))
    return np.where(d > 0, up, np.where(d < 0, dn, x)).astype(self.dt_)

  def _fma2(self, x, y):
    """Dot products over the last axis of x and y (broadcast) as two
    interleaved fused multiply-add chains: s0 over the even terms, s1 over
    the odd ones, then s0 + s1; each fma rounded once to this dtype (the
    float64 product of two float32 values is exact)."""
    n = x.shape[-1]
    shape = np.broadcast_shapes(x.shape[:-1], y.shape[:-1])
    s = [np.zeros(shape, self.dt_), np.zeros(shape, self.dt_)]
    for d in range(n):
      k = d & 1
      s[k] = (x[..., d].astype(np.float64) * y[..., d].astype(np.float64) + s[k]).astype(self.dt_)
    return (s[0] + s[1]).astype(self.dt_)

  def _mm(self, a, b):
    """a @ b in this oracle's evaluation order ('rounded': float64, rounded once)."""
    if self.order == 'rounded':
      return (a.astype(np.float64) @ b.astype(np.float64)).astype(self.dt_)
    if self.order == 'fma':
      return self._fma2(a[..., :, None, :], np.swapaxes(b, -1, -2)[..., None, :, :])
    return a @ b

  def _mv(self, a, v):
    """a [B, n, m] times v [B, m] in this oracle's evaluation order."""
    if self.order == 'rounded':
      return np.einsum('bij,bj->bi', a.astype(np.float64), v.astype(np.float64)).astype(self.dt_)
    if self.order == 'fma':
      return self._fma2(a, v[:, None, :])
    return np.einsum('bij,bj->bi', a, v)

  # -------------------------------------------------------------------------
  # kinematics.forward: brax/kinematics.py:31-108
  # -------------------------------------------------------------------------
  def kinematics(self, q, qd):
    st, c = self.st, self.c
    B = q.shape[0]
    dt = self.dt_
    jp = np.zeros((B, st.nl, 3), dt)
    jr = np.zeros((B, st.nl, 4), dt)
    ja = np.zeros((B, st.nl, 3), dt)
    jv = np.zeros((B, st.nl, 3), dt)
    for i, t in enumerate(st.types):
      qa, da = st.qadr[i], st.dadr[i]
      if t == 'f':  # kinematics.py:47-50
        jp[:, i], jr[:, i] = q[:, qa:qa + 3], q[:, qa + 3:qa + 7]
        ja[:, i], jv[:, i] = qd[:, da + 3:da + 6], qd[:, da:da + 3]
        continue
      for k in range(int(t)):  # kinematics.py:51-76
        d = da + k
        ang, vel = c['m_ang'][d], c['m_vel'][d]
        rk = normalize(quat_rot_axis(np.broadcast_to(ang, (B, 3)), q[:, qa + k]))
        pk = vel * q[:, qa + k, None]
        dak = ang * qd[:, d, None]
        dvk = vel * qd[:, d, None]
        if k == 0:
          p_, r_, a_, v_ = pk, rk, dak, dvk
        else:
          p_, r_ = tf_do_tf(p_, r_, pk, rk)
          a_ = a_ + rotate(dak, rk)
          v_ = v_ + rotate(dvk + cross(pk, dak), rk)
      jp[:, i], jr[:, i], ja[:, i], jv[:, i] = p_, r_, a_, v_
    # joint anchor offset and link transform: kinematics.py:80-82
    anchor = rotate(np.broadcast_to(c['lj_pos'], jp.shape), jr)
    jp = jp + c['lj_pos'] - anchor
    jp, jr = tf_do_tf(c['lt_pos'], c['lt_rot'], jp, jr)
    # world: kinematics.py:84-102, root-to-leaf level order (scan.py:120-131)
    xp = np.zeros_like(jp)
    xr = np.zeros_like(jr)
    xa = np.zeros_like(ja)
    xv = np.zeros_like(jv)
    for lvl in st.levels:
      for i in lvl:
        p = st.parents[i]
        if p < 0:
          xp[:, i], xr[:, i] = jp[:, i], jr[:, i]
          xa[:, i] = rotate(ja[:, i], jr[:, i])
          xv[:, i] = jv[:, i]
          continue
        xp[:, i], xr[:, i] = tf_do_tf(xp[:, p], xr[:, p], jp[:, i], jr[:, i])
        vel = xv[:, p] + cross(xa[:, p], xp[:, i] - xp[:, p])
        vel = vel + rotate(jv[:, i], xr[:, p])
        xa[:, i] = xa[:, p] + rotate(ja[:, i], xr[:, i])
        xv[:, i] = vel
        # rounding envelope: every link's pose and velocity one ulp either
        # way, carried down the tree as the rounding of each level is (the
        # contact distances taken from them cancel to far below the positions)
        xp[:, i], xr[:, i] = self._nudge(xp[:, i]), self._nudge(xr[:, i])
        xa[:, i], xv[:, i] = self._nudge(xa[:, i]), self._nudge(xv[:, i])
    xr = normalize(xr)  # kinematics.py:106
    return xp, xr, xa, xv

  # -------------------------------------------------------------------------
  # dynamics.transform_com: brax/generalized/dynamics.py:27-134
  # -------------------------------------------------------------------------
  def transform_com(self, s: State) -> State:
    st, c = self.st, self.c
    B, dt = s.q.shape[0], self.dt_
    xi_p, xi_r = tf_do_tf(s.x_pos, s.x_rot, c['li_pos'], c['li_rot'])  # :37
    m = c['li_mass']
    mass_xi = m[:, None] * xi_p  # :40
    root_com = np.zeros_like(xi_p)
    for r in set(st.roots):  # segment_sum :41-43
      mem = [i for i in range(st.nl) if st.roots[i] == r]
      msum = np.zeros((), dt)
      mxs = np.zeros((B, 3), dt)
      for i in mem:
        msum = msum + m[i]
        mxs = mxs + mass_xi[:, i]
      for i in mem:
        root_com[:, i] = mxs / msum
    # cinr = x_i.replace(pos=x_i.pos - root_com).do(inertia): :44, base.py:589-595
    off = xi_p - root_com
    eye = np.eye(3, dtype=dt)
    h = cross(off[:, :, None, :], -eye)  # (B, nl, 3, 3)
    rot = quat_to_3x3(xi_r)
    cinr_i = rot @ c['li_i'] @ np.swapaxes(rot, -1, -2) + (h @ np.swapaxes(h, -1, -2)) * m[:, None, None]
    cinr_pos = off * m[:, None]
    # parent transform for cdof: :47-52
    ident_p = np.zeros((B, 3), dt)
    ident_r = np.broadcast_to(np.array([1, 0, 0, 0], dt), (B, 4))
    jj_p = np.zeros((B, st.nl, 3), dt)
    jj_r = np.zeros((B, st.nl, 4), dt)
    for i, t in enumerate(st.types):
      pi = i if t == 'f' else st.parents[i]
      pp, pr = (s.x_pos[:, pi], s.x_rot[:, pi]) if pi >= 0 else (ident_p, ident_r)
      a_p, a_r = tf_do_tf(pp, pr, c['lt_pos'][i], c['lt_rot'][i])
      jj_p[:, i], jj_r[:, i] = tf_do_tf(a_p, a_r, c['lj_pos'][i], c['lj_rot'][i])
    # cdof via stacked joints: :55-85
    nv = st.nv
    cang = np.zeros((B, nv, 3), dt)
    cvel = np.zeros((B, nv, 3), dt)
    for i, t in enumerate(st.types):
      qa, da = st.qadr[i], st.dadr[i]
      if t == 'f':
        cang[:, da:da + 6] = c['m_ang'][da:da + 6]
        cvel[:, da:da + 6] = c['m_vel'][da:da + 6]
        continue
      ap, ar = np.zeros((B, 3), dt), ident_r.copy()
      for k in range(int(t)):
        d = da + k
        ang, vel = c['m_ang'][d], c['m_vel'][d]
        # inv_do(Motion): base.py:580-584
        a_ = rotate(np.broadcast_to(ang, (B, 3)), ar)
        cang[:, d] = a_
        cvel[:, d] = rotate(np.broadcast_to(vel, (B, 3)), ar) + cross(ap, a_)
        rk = normalize(quat_rot_axis(np.broadcast_to(ang, (B, 3)), s.q[:, qa + k]))
        pk = vel * s.q[:, qa + k, None]
        ap, ar = tf_do_tf(ap, ar, pk, rk)
    dl = st.dof_link
    cang = rotate(cang, jj_r[:, dl])  # :86-87
    offp = root_com - jj_p  # :88-89 (Transform.do(Motion) with identity rot)
    cvel = cvel - cross(offp[:, dl], cang)
    qd = s.qd
    cq_a = cang * qd[:, :, None]
    cq_v = cvel * qd[:, :, None]
    # cd: root-to-leaf, cd = cd[parent] + sum(cdof * qd): :93-103
    cd_a = np.zeros((B, st.nl, 3), dt)
    cd_v = np.zeros((B, st.nl, 3), dt)
    for lvl in st.levels:
      for i in lvl:
        p = st.parents[i]
        a_ = cd_a[:, p].copy() if p >= 0 else np.zeros((B, 3), dt)
        v_ = cd_v[:, p].copy() if p >= 0 else np.zeros((B, 3), dt)
        for d in range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[st.types[i]]):
          a_ = a_ + cq_a[:, d]
          v_ = v_ + cq_v[:, d]
        cd_a[:, i], cd_v[:, i] = a_, v_
    # cdofd: :106-130
    dd_a = np.zeros((B, nv, 3), dt)
    dd_v = np.zeros((B, nv, 3), dt)
    for i, t in enumerate(st.types):
      da = st.dadr[i]
      if t == 'f':
        sa = cq_a[:, da] + cq_a[:, da + 1] + cq_a[:, da + 2]
        sv = cq_v[:, da] + cq_v[:, da + 1] + cq_v[:, da + 2]
        for k in range(3, 6):
          dd_a[:, da + k], dd_v[:, da + k] = motion_cross(sa, sv, cang[:, da + k], cvel[:, da + k])
        continue
      p = st.parents[i]
      sa = cd_a[:, p] if p >= 0 else np.zeros((B, 3), dt)
      sv = cd_v[:, p] if p >= 0 else np.zeros((B, 3), dt)
      for k in range(int(t)):
        d = da + k
        dd_a[:, d], dd_v[:, d] = motion_cross(sa, sv, cang[:, d], cvel[:, d])
        sa, sv = sa + cq_a[:, d], sv + cq_v[:, d]
    return s.replace(root_com=root_com, cinr_pos=cinr_pos, cinr_rot=xi_r,
                     cinr_i=cinr_i, cinr_mass=np.broadcast_to(m, (B, st.nl)).copy(),
                     cd_ang=cd_a, cd_vel=cd_v, cdof_ang=cang, cdof_vel=cvel,
                     cdofd_ang=dd_a, cdofd_vel=dd_v)

  # -------------------------------------------------------------------------
  # mass.matrix (CRBA) and matrix_inv: brax/generalized/mass.py:27-106
  # -------------------------------------------------------------------------
  def mass_matrix(self, s: State):
    st, c = self.st, self.c
    B, dt = s.q.shape[0], self.dt_
    crb_i = s.cinr_i.copy()
    crb_p = s.cinr_pos.copy()
    crb_m = s.cinr_mass.copy()
    for lvl in reversed(st.levels):  # leaf-to-root: crb = cinr + sum(children)
      for i in lvl:
        if not st.children[i]:
          continue
        si = np.zeros((B, 3, 3), dt)
        sp = np.zeros((B, 3), dt)
        sm = np.zeros((B,), dt)
        for ch in st.children[i]:
          si, sp, sm = si + crb_i[:, ch], sp + crb_p[:, ch], sm + crb_m[:, ch]
        crb_i[:, i], crb_p[:, i], crb_m[:, i] = crb_i[:, i] + si, crb_p[:, i] + sp, crb_m[:, i] + sm
    dl = st.dof_link
    fa, fv = inertia_mul(crb_i[:, dl], crb_p[:, dl], crb_m[:, dl], s.cdof_ang, s.cdof_vel)
    # mx[r, c] = cdof_c . f_r  (Motion.dot: vel.vel + ang.ang)
    mx = (np.einsum('bcj,brj->brc', s.cdof_vel, fv) + np.einsum('bcj,brj->brc', s.cdof_ang, fa))
    mask = np.zeros((st.nv, st.nv), dt)
    ranges = []
    for i, t in enumerate(st.types):
      ranges.append(list(range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[t])))
    for i in range(st.nl):
      j = i
      while j > -1:
        for a in ranges[i]:
          for b_ in ranges[j]:
            mask[a, b_] = 1
        j = st.parents[j]
    mx = mx * mask
    mx = np.tril(mx) + np.swapaxes(np.tril(mx, -1), -1, -2)
    mx = mx + np.diag(c['armature'])
    return mx

  def inv_approximate(self, a, a_inv, num_iter):
    """brax/math.py:278-305 (Newton-Schulz with best-iterate acceptance)."""
    dt = self.dt_
    n = a.shape[-1]
    eye = np.eye(n, dtype=dt)
    r0 = eye - self._mm(a, a_inv)
    n0 = safe_norm(r0, 2)
    reset = n0 > 1 + self._margin(np.maximum(n0, 1))
    tr = np.trace(a @ np.swapaxes(a, -1, -2), axis1=-2, axis2=-1)
    alt = 0.5 * np.swapaxes(a, -1, -2) / tr[:, None, None]
    a_inv = np.where(reset[:, None, None], alt, a_inv)
    r, err = r0, np.ones(a.shape[0], dt)
    for _ in range(num_iter):
      nxt = self._nudge(self._mm(a_inv, eye + r))
      r_next = self._nudge(eye - self._mm(a, nxt))
      err_next = safe_norm(r_next, 2)
      take = err_next < err + self._margin(np.maximum(err_next, err))
      a_inv = np.where(take[:, None, None], nxt, a_inv)
      r, err = r_next, err_next
    return a_inv

  def spd_inverse(self, a):
    """jax.scipy.linalg.solve(a, I, assume_a='pos') (mass.py:104)."""
    if self.order == 'rounded':
      a64 = a.astype(np.float64)
      l = np.linalg.cholesky(a64)
      linv = np.linalg.solve(l, np.broadcast_to(np.eye(a.shape[-1]), a.shape))
      return (np.swapaxes(linv, -1, -2) @ linv).astype(self.dt_)
    l = np.linalg.cholesky(a)
    n = a.shape[-1]
    linv = np.linalg.solve(l, np.broadcast_to(np.eye(n, dtype=a.dtype), a.shape))
    return np.swapaxes(linv, -1, -2) @ linv

  def matrix_inv(self, s: State, num_iter: int) -> State:
    mx = self._nudge(self.mass_matrix(s), symmetric=True)
    if self.st.nv == 0:
      return s.replace(mass_mx=mx, mass_mx_inv=mx)
    if num_iter > 0 and not self.exact_inverse:
      minv = self.inv_approximate(mx, s.mass_mx_inv, num_iter)
    else:
      minv = self.spd_inverse(mx)
    return s.replace(mass_mx=mx, mass_mx_inv=self._nudge(minv, symmetric=True))

  # -------------------------------------------------------------------------
  # contact.get (+ mujoco.mjx primitive collisions): brax/contact.py:28-67
  # -------------------------------------------------------------------------
  def contacts(self, x_pos, x_rot):
    sys, c = self.sys, self.c
    B, dt = x_pos.shape[0], self.dt_
    cs = sys.contacts
    n = cs.n
    zp = np.zeros((B, 1, 3), dt)
    zr = np.broadcast_to(np.array([1, 0, 0, 0], dt), (B, 1, 4))
    xp = np.concatenate([x_pos, zp], axis=1)
    xr = np.concatenate([x_rot, zr], axis=1)
    bid = sys.geom_bodyid - 1  # -1 -> the appended zero transform
    gxp = xp[:, bid] + rotate(np.broadcast_to(c['geom_pos'], xp[:, bid].shape), xr[:, bid])
    gxm = quat_to_3x3(quat_mul(xr[:, bid], np.broadcast_to(c['geom_quat'], xr[:, bid].shape)))
    dist = np.zeros((B, n), dt)
    pos = np.zeros((B, n, 3), dt)
    frame = np.zeros((B, n, 3, 3), dt)
    size = c['geom_size']
    for k in range(n):
      g1, g2, kind, sub = cs.geom1[k], cs.geom2[k], cs.kind[k], cs.sub[k]
      p1, m1, p2, m2 = gxp[:, g1], gxm[:, g1], gxp[:, g2], gxm[:, g2]
      if kind == S.CON_PLANE_SPHERE:
        nrm = m1[..., :, 2]
        d, ps = _plane_sphere(nrm, p1, p2, size[g2, 0])
        dist[:, k], pos[:, k], frame[:, k] = d, ps, make_frame(nrm)
      elif kind == S.CON_PLANE_CAPSULE:
        nrm, axis = m1[..., :, 2], m2[..., :, 2]
        b, bn = _norm_with_norm(axis - nrm * dot(nrm, axis)[..., None])
        yv = np.array([0.0, 1.0, 0.0], dt)
        zv = np.array([0.0, 0.0, 1.0], dt)
        alt = np.where(((-0.5 < nrm[..., 1]) & (nrm[..., 1] < 0.5))[..., None], yv, zv)
        b = np.where((bn < 0.5)[..., None], alt, b)
        seg = axis * size[g2, 1]
        center = p2 + seg if sub == 0 else p2 - seg
        d, ps = _plane_sphere(nrm, p1, center, size[g2, 0])
        dist[:, k], pos[:, k] = d, ps
        frame[:, k] = np.stack([nrm, b, cross(nrm, b)], axis=-2)
      elif kind == S.CON_PLANE_BOX:
        d, ps, fr = _plane_box(p1, m1, p2, m2, size[g2], sub, None if self._rng is None else self._margin)
        dist[:, k], pos[:, k], frame[:, k] = d, ps, fr
      elif kind == S.CON_SPHERE_SPHERE:
        d, ps, nrm = _sphere_sphere(p1, size[g1, 0], p2, size[g2, 0])
        dist[:, k], pos[:, k], frame[:, k] = d, ps, make_frame(nrm)
      elif kind == S.CON_SPHERE_CAPSULE:
        seg = m2[..., :, 2] * size[g2, 1]
        pt = _closest_segment_point(p2 - seg, p2 + seg, p1)
        d, ps, nrm = _sphere_sphere(p1, size[g1, 0], pt, size[g2, 0])
        dist[:, k], pos[:, k], frame[:, k] = d, ps, make_frame(nrm)
      elif kind == S.CON_CAPSULE_CAPSULE:
        s1 = m1[..., :, 2] * size[g1, 1]
        s2 = m2[..., :, 2] * size[g2, 1]
        a_, b_ = _closest_segment_to_segment_points(p1 - s1, p1 + s1, p2 - s2, p2 + s2, self._margin)
        d, ps, nrm = _sphere_sphere(a_, size[g1, 0], b_, size[g2, 0])
        dist[:, k], pos[:, k], frame[:, k] = d, ps, make_frame(nrm)
      else:
        raise NotImplementedError(kind)
    return dist, pos, frame

  # -------------------------------------------------------------------------
  # constraint: brax/generalized/constraint.py:29-240
  # -------------------------------------------------------------------------
  @staticmethod
  def imp_aref(params, pos, vel):
    """constraint.py:29-65; params (..., 7)."""
    timeconst, dampratio, dmin, dmax, width, mid, power = [params[..., k] for k in range(7)]
    imp_x = np.abs(pos) / width
    imp_a = (1.0 / np.power(mid, power - 1)) * np.power(imp_x, power)
    imp_b = 1 - (1.0 / np.power(1 - mid, power - 1)) * np.power(1 - imp_x, power)
    imp_y = np.where(imp_x < mid, imp_a, imp_b)
    imp = dmin + imp_y * (dmax - dmin)
    imp = np.clip(imp, dmin, dmax)
    imp = np.where(imp_x > 1.0, dmax, imp)
    b = 2 / (dmax * timeconst)
    k = 1 / (dmax * dmax * timeconst * timeconst * dampratio * dampratio)
    stiffness, damping = params[..., 0], params[..., 1]
    b = np.where(damping <= 0, -damping / dmax, b)
    k = np.where(stiffness <= 0, -stiffness / (dmax * dmax), k)
    aref = -b * vel - k * imp * pos
    return imp, aref

  def point_jacobian(self, s: State, pos, link_idx: int):
    """constraint.py:68-98 -> Motion (ang, vel) of shape (B, nv, 3)."""
    st = self.st
    anc = set()
    j = link_idx
    while j >= 0:
      anc.add(j)
      j = st.parents[j]
    mask = np.array([1.0 if st.dof_link[d] in anc else 0.0 for d in range(st.nv)], self.dt_)
    ca = s.cdof_ang * mask[:, None]
    cv = s.cdof_vel * mask[:, None]
    off = pos - s.root_com[:, link_idx]  # com[-1] wraps, as jax indexing does
    return ca, cv - cross(off[:, None, :], ca)

  def jac_contact(self, s: State):
    """constraint.py:135-176."""
    sys, c = self.sys, self.c
    cs = sys.contacts
    B, dt, nv = s.q.shape[0], self.dt_, self.st.nv
    if cs.n == 0:
      z = np.zeros((B, 0), dt)
      return np.zeros((B, 0, nv), dt), z, z, z
    dist, pos, frame = self.contacts(s.x_pos, s.x_rot)
    jac = np.zeros((B, 4 * cs.n, nv), dt)
    diag = np.zeros((B, 4 * cs.n), dt)
    aref = np.zeros((B, 4 * cs.n), dt)
    invw = c['l_invw']
    for k in range(cs.n):
      la, lb = int(cs.link_a[k]), int(cs.link_b[k])
      _, a_vel = self.point_jacobian(s, pos[:, k], la)
      _, b_vel = self.point_jacobian(s, pos[:, k], lb)
      diff = b_vel - a_vel  # (B, nv, 3)
      mu = c['c_fric'][k, 0]
      rows = []
      for t in (-frame[:, k, 1], -frame[:, k, 2]):
        for f in (-mu, mu):
          rows.append(np.einsum('bvj,bj->bv', diff, t * f + frame[:, k, 0]))
      rows = np.stack(rows, axis=1)  # (B, 4, nv)
      p4 = np.repeat(dist[:, k, None], 4, axis=1)
      params = np.concatenate([c['c_solref'][k], c['c_solimp'][k]])
      imp, ar = self.imp_aref(params, p4, np.einsum('brv,bv->br', rows, s.qd))
      tw = invw[la] * (1.0 if la > -1 else 0.0) + invw[lb]
      dg = np.repeat(np.asarray(tw + mu * mu * tw, dt)[None, None], 4, axis=1)
      dg = dg * (2 * mu * mu * (1 - imp) / (imp + 1e-8))
      act = (dist[:, k] < 0).astype(dt)
      jac[:, 4 * k:4 * k + 4] = rows * act[:, None, None]
      diag[:, 4 * k:4 * k + 4] = dg * act[:, None]
      aref[:, 4 * k:4 * k + 4] = ar * act[:, None]
    return jac, diag, aref, dist

  def jac_limit(self, s: State):
    """constraint.py:101-132."""
    sys, c = self.sys, self.c
    B, dt, nv = s.q.shape[0], self.dt_, self.st.nv
    if sys.dof.limit is None:
      z = np.zeros((B, 0), dt)
      return np.zeros((B, 0, nv), dt), z, z
    q_idx, qd_idx = sys.q_idx('123'), sys.qd_idx('123')
    pos_min = s.q[:, q_idx] - c['lo'][qd_idx]
    pos_max = c['hi'][qd_idx] - s.q[:, q_idx]
    pos = np.minimum(np.minimum(pos_min, pos_max), 0)
    side = ((pos_min < pos_max) * 2 - 1).astype(dt) * (pos < 0).astype(dt)
    jac = np.eye(nv, dtype=dt)[qd_idx][None] * side[:, :, None]
    params = c['solp'][qd_idx]
    imp, aref = self.imp_aref(params, pos, np.einsum('brv,bv->br', jac, s.qd))
    act = (pos < 0).astype(dt)
    diag = c['d_invw'][qd_idx] * act * (1 - imp) / (imp + 1e-8)
    aref = aref * act
    return jac, diag, aref

  def jacobian(self, s: State) -> State:
    """constraint.py:179-191."""
    jc, dc, ac, dist = self.jac_contact(s)
    jl, dl, al = self.jac_limit(s)
    # (rounding envelope: the rows one ulp either way; J Minv J^T cancels)
    return s.replace(con_jac=self._nudge(np.concatenate([jc, jl], axis=1)),
                     con_diag=self._nudge(np.concatenate([dc, dl], axis=1)),
                     con_aref=self._nudge(np.concatenate([ac, al], axis=1)),
                     contact_dist=dist)

  def pg_solve(self, a, b, maxiter, maxls, tol=1e-3):
    """jaxopt.ProjectedGradient(fun=0.5|Ax+b|^2, projection_non_negative).

    Restates jaxopt's ProximalGradient with acceleration=True (FISTA),
    stepsize<=0 (backtracking, decrease_factor 0.5, the step grown by 1/0.5
    after each accepted search and reset to 1 at <=1e-6), x0=0, stopping when
    |P(x - grad f(x)) - x| <= tol after the first (unconditional) update;
    at most ``maxiter`` updates and ``maxls`` halvings per search.  Used at
    brax/generalized/constraint.py:229-238.
    """
    dt = self.dt_
    B, m = b.shape
    cnt = np.zeros(B, np.int64)

    def resid(x, on):
      cnt[on] += 1
      return np.einsum('bij,bj->bi', a, x) + b

    def fun(x, on):
      r = resid(x, on)
      return np.sum(0.5 * r ** 2, axis=-1)

    def grad(x, on):
      r = resid(x, on)
      cnt[on] += 1
      return np.einsum('bij,bi->bj', a, r)

    relu = lambda v: np.maximum(v, 0)
    x = np.zeros((B, m), dt)
    y = np.zeros((B, m), dt)
    t = np.ones(B, dt)
    ss = np.ones(B, dt)
    err = np.full(B, np.inf, dt)
    active = np.ones(B, bool)
    one = dt.type(1.0)
    for it in range(maxiter):
      if it > 0:
        active = active & (err > tol + self._margin(np.maximum(err, tol)))
      if not active.any():
        break
      ry = resid(y, active)  # value_and_grad at y: one residual, one A^T r
      fy = np.sum(0.5 * ry ** 2, axis=-1)
      cnt[active] += 1
      gy = np.einsum('bij,bi->bj', a, ry)
      cur = ss.copy()
      nx = relu(y + (-cur)[:, None] * gy)
      ls_on = active.copy()
      for _ in range(maxls):
        dx = nx - y
        fn = fun(nx, ls_on)
        dv = np.sum(dx * gy, -1)
        sq = np.sum(dx * dx, -1)
        scale = np.abs(cur * fn) + np.abs(cur * fy) + cur * np.sum(np.abs(dx * gy), -1) + 0.5 * sq
        # a trial point equal to y (sq = 0) is accepted in any precision
        cond = (cur * (fn - fy) > cur * dv + 0.5 * sq + self._margin(scale)) & (sq > 0)
        ls_on = ls_on & cond
        if not ls_on.any():
          break
        cur = np.where(ls_on, cur * dt.type(0.5), cur)
        nx = np.where(ls_on[:, None], relu(y + (-cur)[:, None] * gy), nx)
      nss = np.where(cur <= 1e-6, one, cur / dt.type(0.5))
      nt = dt.type(0.5) * (1 + np.sqrt(1 + 4 * t ** 2))
      ny = nx + ((t - 1) / nt)[:, None] * (nx - x)
      gx = grad(nx, active)
      e = np.sqrt(np.sum((relu(nx + (-one) * gx) - nx) ** 2, -1))
      on = active[:, None]
      x = np.where(on, nx, x)
      y = np.where(on, ny, y)
      t = np.where(active, nt, t)
      ss = np.where(active, nss, ss)
      err = np.where(active, e, err)
    self.last_pg = {'maxiter': active & (err > tol) & (maxiter > 0) & (m > 0), 'err': err}
    return x, cnt

  def constraint_force(self, s: State):
    """constraint.py:194-240."""
    sys = self.sys
    B, dt, nv = s.q.shape[0], self.dt_, self.st.nv
    if s.con_jac.shape[1] == 0:
      self.last_pg = {'maxiter': np.zeros(B, bool), 'err': np.zeros(B, dt)}
      return np.zeros((B, nv), dt), np.zeros(B, np.int64)
    jt = np.swapaxes(s.con_jac, -1, -2)
    if self.order == 'right':  # J (Minv J^T), J (Minv qf_smooth)
      a = s.con_jac @ (s.mass_mx_inv @ jt)
      b = np.einsum('bij,bj->bi', s.con_jac, np.einsum('bij,bj->bi', s.mass_mx_inv, s.qf_smooth)) - s.con_aref
    else:
      jm = self._mm(s.con_jac, s.mass_mx_inv)
      a = self._mm(jm, jt)
      b = self._mv(jm, s.qf_smooth) - s.con_aref
    a = a + np.einsum('bi,ij->bij', s.con_diag, np.eye(a.shape[-1], dtype=dt))
    a, b = self._nudge(a, symmetric=True), self._nudge(b)
    xs, cnt = self.pg_solve(a, b, sys.solver_iterations, sys.solver_maxls)
    return np.einsum('bij,bi->bj', s.con_jac, xs), cnt

  # -------------------------------------------------------------------------
  # actuator.to_tau: brax/actuator.py:23-57
  # -------------------------------------------------------------------------
  def to_tau(self, act, q, qd):
    c, B, dt = self.c, q.shape[0], self.dt_
    nu = self.sys.act_size()
    tau = np.zeros((B, self.st.nv), dt)
    if nu == 0 or act is None:
      return tau
    qa, qda = q[:, self.sys.actuator.q_id], qd[:, self.sys.actuator.qd_id]
    act = np.clip(act, c['a_cr'][:, 0], c['a_cr'][:, 1])
    bias = c['a_gear'] * (qa * c['a_bq'] + qda * c['a_bqd'])
    force = c['a_gain'] * act + bias
    force = np.clip(force, c['a_fr'][:, 0], c['a_fr'][:, 1])
    force = force * c['a_gear']
    for k, d in enumerate(self.sys.actuator.qd_id):
      tau[:, d] = tau[:, d] + force[:, k]
    return tau

  # -------------------------------------------------------------------------
  # dynamics.inverse / _passive / forward: brax/generalized/dynamics.py:137-236
  # -------------------------------------------------------------------------
  def inverse(self, s: State):
    st, c = self.st, self.c
    B, dt = s.q.shape[0], self.dt_
    cdd_a = np.zeros((B, st.nl, 3), dt)
    cdd_v = np.zeros((B, st.nl, 3), dt)
    for lvl in st.levels:  # :153-165
      for i in lvl:
        p = st.parents[i]
        if p < 0:
          a_ = np.zeros((B, 3), dt)
          v_ = np.broadcast_to(-c['gravity'], (B, 3)).copy()
        else:
          a_, v_ = cdd_a[:, p].copy(), cdd_v[:, p].copy()
        for d in range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[st.types[i]]):
          a_ = a_ + s.cdofd_ang[:, d] * s.qd[:, d, None]
          v_ = v_ + s.cdofd_vel[:, d] * s.qd[:, d, None]
        cdd_a[:, i], cdd_v[:, i] = a_, v_
    # cfrc_flat = cinr*cdd + cd x (cinr*cd): :168-171
    fa, fv = inertia_mul(s.cinr_i, s.cinr_pos, s.cinr_mass, cdd_a, cdd_v)
    ga, gv = inertia_mul(s.cinr_i, s.cinr_pos, s.cinr_mass, s.cd_ang, s.cd_vel)
    xa, xv = force_cross(s.cd_ang, s.cd_vel, ga, gv)
    fa, fv = fa + xa, fv + xv
    for lvl in reversed(st.levels):  # :174-179
      for i in lvl:
        if not st.children[i]:
          continue
        sa = np.zeros((B, 3), dt)
        sv = np.zeros((B, 3), dt)
        for ch in st.children[i]:
          sa, sv = sa + fa[:, ch], sv + fv[:, ch]
        fa[:, i], fv[:, i] = fa[:, i] + sa, fv[:, i] + sv
    dl = st.dof_link
    return dot(s.cdof_vel, fv[:, dl]) + dot(s.cdof_ang, fa[:, dl])  # :182

  def passive(self, s: State):
    st, c = self.st, self.c
    frc = np.zeros_like(s.qd)
    for i, t in enumerate(st.types):  # :190-195
      if t == 'f':
        continue
      for k in range(int(t)):
        d = st.dadr[i] + k
        frc[:, d] = -s.q[:, st.qadr[i] + k] * c['stiffness'][d]
    frc = frc - c['damping'] * s.qd
    if self.sys.enable_fluid:  # :198-211
      fa, fv, xi_p = self.fluid_force(s)
      for i in range(st.nl):
        ja, jv = self.point_jacobian(s, xi_p[:, i], i)
        frc = frc + (dot(jv, fv[:, None, i]) + dot(ja, fa[:, None, i]))
    return frc

  def fluid_force(self, s: State):
    """fluid.force, brax/fluid.py:53-82: (force ang, force vel) per link in
    world orientation, and the links' com positions x_i.pos."""
    c, dt = self.c, self.dt_
    xi_p, xi_r = tf_do_tf(s.x_pos, s.x_rot, c['li_pos'], c['li_rot'])  # :64
    off = xi_p - s.root_com  # :66
    rt = quat_inv(xi_r)  # :67, Transform.do(Motion), base.py:573-578
    wa = rotate(s.cd_ang, rt)
    wv = rotate(s.cd_vel - cross(off, s.cd_ang), rt)
    diag = np.diagonal(c['li_i'], axis1=-2, axis2=-1)  # :71-76
    sign = np.ones((3, 3), dt) - 2 * np.eye(3, dtype=dt)
    box = np.sum(diag[:, None, :] * sign, axis=-1)
    box = dt.type(6.0) * np.maximum(box, dt.type(1e-12))
    box = np.sqrt(box / c['li_mass'][:, None])
    pi = dt.type(np.pi)
    diam = np.mean(box, axis=-1)  # _box_viscosity, :24-33
    fa = (-pi * diam ** 3 * c['viscosity'])[:, None] * wa
    fv = (dt.type(-3.0) * pi * diam * c['viscosity'])[:, None] * wv
    b0, b1, b2 = box[:, 0], box[:, 1], box[:, 2]  # _box_density, :36-50
    bv = np.stack([b1 * b2, b0 * b2, b0 * b1], axis=-1)
    fv = fv + dt.type(-0.5) * c['density'] * bv * np.abs(wv) * wv
    ba = np.stack([b0 * (b1 ** 4 + b2 ** 4), b1 * (b0 ** 4 + b2 ** 4), b2 * (b0 ** 4 + b1 ** 4)], axis=-1)
    fa = fa + dt.type(-1.0) * c['density'] * ba * np.abs(wa) * wa / dt.type(64.0)
    return rotate(fa, xi_r), rotate(fv, xi_r), xi_p  # :80, Transform.do(Force) with pos 0

  def forward(self, s: State, tau):
    return self._nudge(self.passive(s) - self.inverse(s) + tau)

  # -------------------------------------------------------------------------
  # integrator.integrate: brax/generalized/integrator.py:26-84
  # -------------------------------------------------------------------------
  def integrate(self, s: State) -> State:
    st, c = self.st, self.c
    dt_, h = self.dt_, self.c['dt']
    if self.sys.matrix_inv_iterations == 0:
      mx = s.mass_mx + np.diag(c['damping']) * h
      minv = self.spd_inverse(mx)
    else:
      minv = s.mass_mx_inv
    qdd = self._mv(minv, s.qf_smooth + s.qf_constraint)
    qd = s.qd + qdd * h
    q = s.q.copy()
    for i, t in enumerate(st.types):
      qa, da = st.qadr[i], st.dadr[i]
      if t == 'f':
        rot, ang = s.q[:, qa + 3:qa + 7], qd[:, da + 3:da + 6]
        an = np.sqrt(np.sum(ang * ang, -1)) + 1e-8
        axis = ang / an[:, None]
        angle = h * an
        qrot = quat_rot_axis(axis, angle)
        rot = quat_mul(rot, qrot)
        rot = rot / np.sqrt(np.sum(rot * rot, -1))[:, None]
        pos = s.q[:, qa:qa + 3] + qd[:, da:da + 3] * h
        q[:, qa:qa + 3], q[:, qa + 3:qa + 7] = pos, rot
      else:
        n = int(t)
        q[:, qa:qa + n] = s.q[:, qa:qa + n] + qd[:, da:da + n] * h
    return s.replace(q=q, qd=qd, qdd=qdd)

  # -------------------------------------------------------------------------
  # pipeline.init / pipeline.step: brax/generalized/pipeline.py:32-94
  # -------------------------------------------------------------------------
  def init(self, q, qd) -> State:
    q = np.asarray(q, self.dt_)
    qd = np.asarray(qd, self.dt_)
    xp, xr, xa, xv = self.kinematics(q, qd)
    B, nv = q.shape[0], self.st.nv
    z = np.zeros((B, nv), self.dt_)
    s = State(q=q, qd=qd, x_pos=xp, x_rot=xr, xd_ang=xa, xd_vel=xv,
              qf_smooth=z, qf_constraint=z.copy(), qdd=z.copy(),
              mass_mx_inv=np.zeros((B, nv, nv), self.dt_))
    s = self.transform_com(s)
    s = self.matrix_inv(s, 0)
    s = self.jacobian(s)
    return s

  def restore(self, q, qd, minv) -> State:
    """The full State the reference holds for (q, qd, mass_mx_inv): every
    other field is the position-level function of (q, qd) computed at the end
    of the previous step (pipeline.py:86-92)."""
    s = self.init(q, qd)
    if minv is not None:
      s = s.replace(mass_mx_inv=np.asarray(minv, self.dt_))
    return s

  def step(self, s: State, act) -> State:
    act = None if act is None else np.asarray(act, self.dt_)
    tau = self.to_tau(act, s.q, s.qd)
    s = s.replace(qf_smooth=self.forward(s, tau))
    qfc, cnt = self.constraint_force(s)
    s = s.replace(qf_constraint=qfc, pg_matvecs=cnt, pg_maxiter=self.last_pg['maxiter'],
                  pg_err=self.last_pg['err'])
    s = self.integrate(s)
    xp, xr, xa, xv = self.kinematics(s.q, s.qd)
    s = s.replace(x_pos=xp, x_rot=xr, xd_ang=xa, xd_vel=xv)
    s = self.transform_com(s)
    s = self.matrix_inv(s, self.sys.matrix_inv_iterations)
    s = self.jacobian(s)
    return s

  def env_step(self, s: State, act, n_frames: int) -> State:
    """PipelineEnv.pipeline_step: n_frames steps with one action (envs/base.py:128-137)."""
    for _ in range(n_frames):
      s = self.step(s, act)
    return s


# mujoco.mjx primitive collision helpers (restated; unpinned) ---------------


def _plane_sphere(n, plane_pos, sphere_pos, radius):
  dist = dot(sphere_pos - plane_pos, n) - radius
  pos = sphere_pos - n * (radius + 0.5 * dist)[..., None]
  return dist, pos


def _sphere_sphere(p1, r1, p2, r2):
  n, d = _norm_with_norm(p2 - p1)
  n = np.where((d == 0.0)[..., None], np.array([1.0, 0.0, 0.0], dtype=p1.dtype), n)
  dist = d - (r1 + r2)
  pos = p1 + n * (r1 + 0.5 * dist)[..., None]
  return dist, pos, n


# mujoco.mjx plane-box: the box as a convex polytope (its 8 vertices in
# itertools.product((-1, 1), repeat=3) order, x slowest) against the plane
# (mujoco-mjx _src/collision_convex.py: the plane-convex routine and its
# 4-point manifold choice).  A vertex is a candidate when it lies below the
# plane or within a 1 mm skin above it; of the candidates the manifold takes
# a (the first), b (furthest from a), c (furthest from the line ab in the
# plane) and d (furthest from the edges ac / bc); a point chosen twice keeps
# only its first slot, the others get dist 1 (inactive).
_BOX_VERTS = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], np.float64)


def _box_manifold(vert, mask, n, margin=None):
  """Indices (B, 4) of the manifold points of `vert` (B, 8, 3) among the
  candidates `mask` (B, 8), n (B, 3) the plane normal in the box frame.
  `margin` (the oracle's rounding envelope) shifts every score of the b, c and
  d choices by up to a few ulps: a box's symmetric vertices often score
  exactly alike, and which of them another operation order ranks first is a
  matter of rounding."""
  big = np.asarray(1e6, vert.dtype)
  dm = np.where(mask, 0, -big).astype(vert.dtype)
  jit = (lambda x: x) if margin is None else (lambda x: x + margin(np.abs(x)))
  ar = np.arange(vert.shape[0])
  a_i = np.argmax(dm, axis=1)
  a = vert[ar, a_i]
  b_i = np.argmax(jit(np.sum((a[:, None] - vert) ** 2, -1)) + dm, axis=1)
  b = vert[ar, b_i]
  ab = cross(n, a - b)
  ap = a[:, None] - vert
  c_i = np.argmax(jit(np.abs(np.sum(ap * ab[:, None], -1))) + dm, axis=1)
  c = vert[ar, c_i]
  ac, bc = cross(n, a - c), cross(n, b - c)
  bp = b[:, None] - vert
  d_bp = jit(np.abs(np.sum(bp * bc[:, None], -1))) + dm
  d_ap = jit(np.abs(np.sum(ap * ac[:, None], -1))) + dm
  d_i = np.argmax(np.concatenate([d_bp, d_ap], axis=1), axis=1) % vert.shape[1]
  return np.stack([a_i, b_i, c_i, d_i], axis=1)


def _plane_box(plane_pos, plane_mat, box_pos, box_mat, size, sub, margin=None):
  """Contact `sub` (0..3) of a plane and a box: dist, pos, frame."""
  dt = box_pos.dtype
  vert = (_BOX_VERTS.astype(dt) * size.astype(dt))[None]            # (1, 8, 3) box frame
  rel = np.einsum('bji,bj->bi', box_mat, plane_pos - box_pos)       # box_mat^T (plane - box)
  n_l = np.einsum('bji,bj->bi', box_mat, plane_mat[..., :, 2])
  support = np.sum((rel[:, None] - vert) * n_l[:, None], -1)        # (B, 8): depth below the plane
  B = box_pos.shape[0]
  idx = _box_manifold(np.broadcast_to(vert, (B, 8, 3)), support > -1e-3, n_l, margin)
  i = idx[:, sub]
  unique = np.all(idx[:, :sub] != i[:, None], axis=1) if sub > 0 else np.ones(B, bool)
  ar = np.arange(B)
  dist = np.where(unique, -support[ar, i], np.asarray(1, dt)).astype(dt)
  n = plane_mat[..., :, 2]
  pos = box_pos + np.einsum('bij,bj->bi', box_mat, vert[0][i]) - n * (0.5 * dist)[:, None]
  return dist, pos, make_frame(n)


def _closest_segment_point(a, b, pt):
  ab = b - a
  t = dot(pt - a, ab) / (dot(ab, ab) + 1e-6)
  return a + np.clip(t, 0.0, 1.0)[..., None] * ab


def _closest_segment_point_and_dist(a, b, pt):
  p = _closest_segment_point(a, b, pt)
  return p, dot(pt - p, pt - p)


def _closest_segment_to_segment_points(a0, a1, b0, b1, margin=None):
  dir_a, len_a = _norm_with_norm(a1 - a0)
  dir_b, len_b = _norm_with_norm(b1 - b0)
  half_a, half_b = len_a * 0.5, len_b * 0.5
  a_mid = a0 + dir_a * half_a[..., None]
  b_mid = b0 + dir_b * half_b[..., None]
  trans = a_mid - b_mid
  dd = dot(dir_a, dir_b)
  dat = dot(dir_a, trans)
  dbt = dot(dir_b, trans)
  denom = 1 - dd * dd
  ta0 = (-dat + dd * dbt) / (denom + 1e-6)
  tb0 = dbt + ta0 * dd
  ta = np.clip(ta0, -half_a, half_a)
  tb = np.clip(tb0, -half_b, half_b)
  best_a = a_mid + dir_a * ta[..., None]
  best_b = b_mid + dir_b * tb[..., None]
  new_a, d1 = _closest_segment_point_and_dist(a0, a1, best_b)
  new_b, d2 = _closest_segment_point_and_dist(b0, b1, best_a)
  # `margin` (the oracle's rounding envelope): the decision's two sides shifted
  sel = (d1 < d2 + (0 if margin is None else margin(np.maximum(d1, d2))))[..., None]
  return np.where(sel, new_a, best_a), np.where(sel, best_b, new_b)
