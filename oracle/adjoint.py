"""Reverse-mode derivative (VJP) of the pipeline step, restated in numpy.

TEST INFRASTRUCTURE ONLY (the checker for the CUDA adjoint).

The reference differentiates the step with ``jax.grad`` through every stage
of brax/generalized/pipeline.py:64-94, including the unrolled jaxopt
iterations (``implicit_diff=False``, brax/generalized/constraint.py:229-238).
This module restates that derivative by hand, for the step with the exact
mass-matrix inverse (Minv = M(q)^-1, the fixed point Newton-Schulz converges
to; a converged iterate's dependence on its warm start vanishes), so the step
is the map (q, qd, act) -> (q', qd').  Discrete decisions (active-contact
mask, clip ranges, line-search step sizes, projection active sets, iteration
counts) are piecewise constant, as under ``jax.grad``.

Differentiable envelope: hinge / slide / free joints, plane-sphere and
plane-capsule contacts against a world plane, joint limits, actuators.
"""

from __future__ import annotations

import numpy as np

from brax_gb300 import system as S
from oracle.pipeline import (Oracle, cross, dot, quat_mul, quat_rot_axis, quat_to_3x3, rotate,
                             normalize, tf_do_tf, inertia_mul, force_cross, motion_cross,
                             _norm_with_norm, _plane_sphere, safe_norm)


# ---------------------------------------------------------------------------
# Newton-Schulz inverse with its tape, and its reverse
# ---------------------------------------------------------------------------


def ns_forward(a, x0, num_iter):
  """brax/math.py:278-305 on a batch (a, x0 [B, n, n]): the reset to
  0.5 a^T / tr(a a^T) when |I - a x0| > 1, then num_iter updates
  x <- x (I + r), r <- I - a x, each kept only if its residual norm is below
  the previous one (r is carried either way).  Returns (x, tape)."""
  B, n = a.shape[0], a.shape[-1]
  eye = np.eye(n)
  r0 = eye - a @ x0
  reset = safe_norm(r0, 2) > 1
  s = np.trace(a @ np.swapaxes(a, -1, -2), axis1=-2, axis2=-1)
  alt = 0.5 * np.swapaxes(a, -1, -2) / s[:, None, None]
  x = np.where(reset[:, None, None], alt, x0)
  r, err = r0, np.ones(B)
  xs, rs, cands, accs = [], [], [], []
  for _ in range(num_iter):
    xn = x @ (eye + r)
    rn = eye - a @ xn
    en = safe_norm(rn, 2)
    acc = en < err
    xs.append(x)
    rs.append(r)
    cands.append(xn)
    accs.append(acc)
    x = np.where(acc[:, None, None], xn, x)
    r, err = rn, en
  return x, dict(a=a, x0=x0, reset=reset, s=s, xs=xs, rs=rs, cands=cands, accs=accs)


def ns_vjp(tape, xbar):
  """Reverse of ns_forward: the cotangent of its result -> (a_bar, x0_bar).
  The reset and acceptance decisions are piecewise constant (jnp.where in the
  reference)."""
  a = tape['a']
  at = np.swapaxes(a, -1, -2)
  n = a.shape[-1]
  eye = np.eye(n)
  abar = np.zeros_like(a)
  rbar = np.zeros_like(a)
  xbar = xbar.copy()
  for k in range(len(tape['xs']) - 1, -1, -1):
    acc = tape['accs'][k][:, None, None]
    xnbar = np.where(acc, xbar, 0.0)
    xkbar = np.where(acc, 0.0, xbar)
    xn = tape['cands'][k]
    # r_{k+1} = I - a xn_k
    xnbar = xnbar - at @ rbar
    abar -= rbar @ np.swapaxes(xn, -1, -2)
    # xn_k = x_k (I + r_k)
    xk, rk = tape['xs'][k], tape['rs'][k]
    xkbar = xkbar + xnbar @ np.swapaxes(eye + rk, -1, -2)
    rbar = np.swapaxes(xk, -1, -2) @ xnbar
    xbar = xkbar
  # r0 = I - a x0 (of the input, whether or not it was reset)
  x0 = tape['x0']
  x0bar = -at @ rbar
  abar -= rbar @ np.swapaxes(x0, -1, -2)
  # x after the reset: 0.5 a^T / s (s = tr(a a^T)) or x0
  reset = tape['reset'][:, None, None]
  s = tape['s'][:, None, None]
  g = xbar
  alt_bar = 0.5 * np.swapaxes(g, -1, -2) / s - (np.sum(at * g, axis=(-2, -1))[:, None, None] / s ** 2) * a
  abar += np.where(reset, alt_bar, 0.0)
  x0bar += np.where(reset, 0.0, g)
  return abar, x0bar

# ---------------------------------------------------------------------------
# primitive reverses
# ---------------------------------------------------------------------------


def conj(q):
  return q * np.array([1.0, -1.0, -1.0, -1.0])


def rotate_vjp(v, q, rb):
  """r = rotate(v, q) (brax/math.py:25-40) -> (v_bar, q_bar)."""
  s, u = q[..., 0:1], q[..., 1:]
  ru = dot(rb, u)[..., None]
  vb = 2 * ru * u + (s * s - dot(u, u)[..., None]) * rb + 2 * s * cross(rb, u)
  ub = 2 * ru * v + 2 * dot(u, v)[..., None] * rb - 2 * dot(rb, v)[..., None] * u + 2 * s * cross(v, rb)
  sb = 2 * s[..., 0] * dot(rb, v) + 2 * dot(rb, cross(u, v))
  return vb, np.concatenate([sb[..., None], ub], axis=-1)


def qmul_vjp(a, b, cb):
  """c = quat_mul(a, b) -> (a_bar, b_bar)."""
  return quat_mul(cb, conj(b)), quat_mul(conj(a), cb)


def tf_do_vjp(ap, ar, bp, br, opb, orb):
  """(op, or) = Transform.do -> (ap_b, ar_b, bp_b, br_b)."""
  bpb, arb1 = rotate_vjp(bp, ar, opb)
  arb2, brb = qmul_vjp(ar, br, orb)
  return opb, arb1 + arb2, bpb, brb


def normalize_vjp(x, yb):
  """y = x / |x| (x nonzero) -> x_bar."""
  n = np.sqrt(np.sum(x * x, -1, keepdims=True))
  y = x / n
  return (yb - y * np.sum(y * yb, -1, keepdims=True)) / n


def cross_vjp(a, b, cb):
  return cross(b, cb), cross(cb, a)


def quat_to_3x3_vjp(q, Rb):
  """R = quat_to_3x3(q) (brax/math.py:151-165) -> q_bar."""
  w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
  d = w * w + x * x + y * y + z * z
  s = 2 / d
  R = lambda a, b: Rb[..., a, b]
  gw = -z * R(0, 1) + y * R(0, 2) + z * R(1, 0) - x * R(1, 2) - y * R(2, 0) + x * R(2, 1)
  gx = (y * R(0, 1) + z * R(0, 2) + y * R(1, 0) - 2 * x * R(1, 1) - w * R(1, 2) + z * R(2, 0)
        + w * R(2, 1) - 2 * x * R(2, 2))
  gy = (-2 * y * R(0, 0) + x * R(0, 1) + w * R(0, 2) + x * R(1, 0) + z * R(1, 2) - w * R(2, 0)
        + z * R(2, 1) - 2 * y * R(2, 2))
  gz = (-2 * z * R(0, 0) - w * R(0, 1) + x * R(0, 2) + w * R(1, 0) - 2 * z * R(1, 1) + y * R(1, 2)
        + x * R(2, 0) + y * R(2, 1))
  P = np.stack([
      np.stack([-(y * y + z * z), x * y - w * z, x * z + w * y], -1),
      np.stack([x * y + w * z, -(x * x + z * z), y * z - w * x], -1),
      np.stack([x * z - w * y, y * z + w * x, -(x * x + y * y)], -1)], -2)
  sp = np.sum(Rb * P, axis=(-2, -1))
  g = np.stack([gw, gx, gy, gz], -1) * s[..., None]
  return g - (2 * s / d * sp)[..., None] * q


def inertia_mul_vjp(i, tpos, mass, m_ang, m_vel, fab, fvb):
  """(fa, fv) = Inertia.mul (brax/base.py:297-302) -> (i_b, tpos_b, ang_b, vel_b)."""
  ib = fab[..., :, None] * m_ang[..., None, :]
  mab = np.einsum('...ji,...j->...i', i, fab)
  pb1, mvb = cross_vjp(tpos, m_vel, fab)
  mvb = mvb + mass[..., None] * fvb
  pb2, mab2 = cross_vjp(tpos, m_ang, -fvb)
  return ib, pb1 + pb2, mab + mab2, mvb


def motion_cross_vjp(sa, sv, oa, ov, rab, rvb):
  """(ra, rv) = (sa x oa, sa x ov + sv x oa)."""
  sab, oab = cross_vjp(sa, oa, rab)
  sab2, ovb = cross_vjp(sa, ov, rvb)
  svb, oab2 = cross_vjp(sv, oa, rvb)
  return sab + sab2, svb, oab + oab2, ovb


def force_cross_vjp(sa, sv, fa, fv, rab, rvb):
  """(ra, rv) = (sa x fa + sv x fv, sa x fv)."""
  sab, fab = cross_vjp(sa, fa, rab)
  svb, fvb = cross_vjp(sv, fv, rab)
  sab2, fvb2 = cross_vjp(sa, fv, rvb)
  return sab + sab2, svb, fab, fvb + fvb2


def quat_rot_axis_vjp_angle(axis, angle, qb):
  """q = quat_rot_axis(axis, angle) with a constant axis -> angle_bar."""
  s, c = np.sin(angle / 2), np.cos(angle / 2)
  return qb[..., 0] * (-0.5 * s) + dot(qb[..., 1:], axis) * (0.5 * c)


def clip_grad(x, lo, hi):
  """d jnp.clip(x, lo, hi) / dx (brax/actuator.py:44,52): jnp.clip is
  maximum(lo, x) then minimum(hi, .), and jax differentiates maximum /
  minimum with ties split evenly: 1 inside, 1/2 on a bound, 0 beyond."""
  m = np.maximum(lo, x)
  dm = np.where(x > lo, 1.0, np.where(x == lo, 0.5, 0.0))
  dh = np.where(m < hi, 1.0, np.where(m == hi, 0.5, 0.0))
  return dm * dh


def imp_parts(params, pos, vel):
  """_imp_aref (constraint.py:29-65) plus d imp / d pos, b and k."""
  timeconst, dampratio, dmin, dmax, width, mid, power = [params[..., k] for k in range(7)]
  x = np.abs(pos) / width
  ia = (1.0 / np.power(mid, power - 1)) * np.power(x, power)
  ib = 1 - (1.0 / np.power(1 - mid, power - 1)) * np.power(1 - x, power)
  dia = (1.0 / np.power(mid, power - 1)) * power * np.power(x, power - 1)
  dib = (1.0 / np.power(1 - mid, power - 1)) * power * np.power(1 - x, power - 1)
  y = np.where(x < mid, ia, ib)
  dy = np.where(x < mid, dia, dib)
  imp0 = dmin + y * (dmax - dmin)
  imp = np.clip(imp0, dmin, dmax)
  dimp = np.where((imp0 > dmin) & (imp0 < dmax), dy * (dmax - dmin), 0.0)
  imp = np.where(x > 1.0, dmax, imp)
  dimp = np.where(x > 1.0, 0.0, dimp) * np.sign(pos) / width
  b = 2 / (dmax * timeconst)
  k = 1 / (dmax * dmax * timeconst * timeconst * dampratio * dampratio)
  b = np.where(dampratio <= 0, -dampratio / dmax, b)
  k = np.where(timeconst <= 0, -timeconst / (dmax * dmax), k)
  return imp, dimp, b, k


def _ddiag_dimp(imp):
  """d/dimp of (1 - imp) / (imp + 1e-8)."""
  return -1 / (imp + 1e-8) - (1 - imp) / (imp + 1e-8) ** 2


# ---------------------------------------------------------------------------
# the step: forward with a tape, then its reverse
# ---------------------------------------------------------------------------


class StepAdjoint:
  """Forward with tape + reverse of brax/generalized/pipeline.py:64-94.

  With ``newton_schulz=True`` (and a model with matrix_inv_iterations > 0)
  the step's mass_mx_inv is the reference's Newton-Schulz update of the
  carried inverse (brax/generalized/mass.py:99-101): ``forward(q, qd, act,
  minv_prev)`` takes the previous pipeline step's inverse (None: the exact
  inverse, as pipeline.init computes it), ``T['s'].mass_mx_inv`` is the
  inverse this step carries on, and ``vjp(T, qb, qdb, minvb_out)`` takes
  that inverse's cotangent from the next step and leaves the cotangent of
  ``minv_prev`` in ``self.minvb_prev``."""

  def __init__(self, sys: S.System, newton_schulz: bool = False):
    self.sys = sys
    self.ns_iters = sys.matrix_inv_iterations if newton_schulz else 0
    self.minvb_prev = None
    self.o = Oracle(sys, np.float64, exact_inverse=True)
    self.st = self.o.st
    self.c = self.o.c
    for k in sys.contacts.kind:
      if k not in (S.CON_PLANE_SPHERE, S.CON_PLANE_CAPSULE):
        raise NotImplementedError('gradients support plane-sphere and plane-capsule contacts')
    for la in sys.contacts.link_a:
      if la >= 0:
        raise NotImplementedError('gradients support contacts against world planes only')
    self.anc = []
    for d in range(self.st.nv):
      a_, j = set(), self.st.dof_link[d]
      while j >= 0:
        a_.add(j)
        j = self.st.parents[j]
      self.anc.append(a_)

  # ------------------------------------------------------------------ FK tape
  def _fk(self, q):
    st, c = self.st, self.c
    B = q.shape[0]
    jp = np.zeros((B, st.nl, 3))
    jr = np.zeros((B, st.nl, 4))
    per = {}
    for i, t in enumerate(st.types):
      qa = st.qadr[i]
      if t == 'f':
        jp[:, i], jr[:, i] = q[:, qa:qa + 3], q[:, qa + 3:qa + 7]
        continue
      acc_p = acc_r = None
      pieces = []
      for k in range(int(t)):
        d = st.dadr[i] + k
        raw = quat_rot_axis(np.broadcast_to(c['m_ang'][d], (B, 3)), q[:, qa + k])
        rk = normalize(raw)
        pk = c['m_vel'][d] * q[:, qa + k, None]
        pieces.append(dict(raw=raw, rk=rk, pk=pk, acc_p=acc_p, acc_r=acc_r))
        if k == 0:
          acc_p, acc_r = pk, rk
        else:
          acc_p, acc_r = tf_do_tf(acc_p, acc_r, pk, rk)
      per[i] = pieces
      jp[:, i], jr[:, i] = acc_p, acc_r
    jpos = np.broadcast_to(c['lj_pos'], jp.shape)
    jp2 = jp + jpos - rotate(jpos, jr)
    jp3, jr3 = tf_do_tf(c['lt_pos'], c['lt_rot'], jp2, jr)
    xp = np.zeros_like(jp3)
    xraw = np.zeros_like(jr3)
    for lvl in st.levels:
      for i in lvl:
        p = st.parents[i]
        if p < 0:
          xp[:, i], xraw[:, i] = jp3[:, i], jr3[:, i]
        else:
          xp[:, i], xraw[:, i] = tf_do_tf(xp[:, p], xraw[:, p], jp3[:, i], jr3[:, i])
    return dict(jp=jp, jr=jr, per=per, jp2=jp2, jp3=jp3, jr3=jr3, xp=xp, xraw=xraw,
                xr=normalize(xraw))

  # -------------------------------------------------------------- forward
  def forward(self, q, qd, act, minv_prev=None):
    """One pipeline step from (q, qd) (and, in Newton-Schulz mode, the
    carried inverse); returns (q', qd', tape)."""
    o, st, c, sys = self.o, self.st, self.c, self.sys
    B = q.shape[0]
    T = dict(q=q, qd=qd, act=act)
    T['fk'] = fk = self._fk(q)
    s = o.init(q, qd)  # the position terms, exactly as the oracle computes them
    if self.ns_iters > 0 and minv_prev is not None:
      minv, T['ns'] = ns_forward(s.mass_mx, np.asarray(minv_prev, np.float64), self.ns_iters)
      s = s.replace(mass_mx_inv=minv)
    assert np.allclose(s.x_pos, fk['xp']) and np.allclose(s.x_rot, fk['xr'])
    T['s'] = s
    # com-stage intermediates the reverse needs
    xi_p, xi_r = tf_do_tf(s.x_pos, s.x_rot, c['li_pos'], c['li_rot'])
    jj_p = np.zeros((B, st.nl, 3))
    jj_r = np.zeros((B, st.nl, 4))
    a_pr = []
    for i, t in enumerate(st.types):
      pi = i if t == 'f' else st.parents[i]
      if pi >= 0:
        pp, pr = s.x_pos[:, pi], s.x_rot[:, pi]
      else:
        pp, pr = np.zeros((B, 3)), np.broadcast_to(np.array([1.0, 0, 0, 0]), (B, 4))
      ap, ar = tf_do_tf(pp, pr, c['lt_pos'][i], c['lt_rot'][i])
      jj_p[:, i] = ap + rotate(np.broadcast_to(c['lj_pos'][i], (B, 3)), ar)
      jj_r[:, i] = ar
      a_pr.append((pi, pp, pr, ap, ar))
    T.update(xi_p=xi_p, xi_r=xi_r, jj_p=jj_p, jj_r=jj_r, a_pr=a_pr)
    # cdof before the jj rotation (stacked joints)
    cang0 = np.zeros((B, st.nv, 3))
    cvel0 = np.zeros((B, st.nv, 3))
    stack = {}
    for i, t in enumerate(st.types):
      qa, da = st.qadr[i], st.dadr[i]
      if t == 'f':
        cang0[:, da:da + 6] = c['m_ang'][da:da + 6]
        cvel0[:, da:da + 6] = c['m_vel'][da:da + 6]
        continue
      ap_, ar_ = np.zeros((B, 3)), np.broadcast_to(np.array([1.0, 0, 0, 0]), (B, 4)).copy()
      recs = []
      for k in range(int(t)):
        d = da + k
        ang, vel = c['m_ang'][d], c['m_vel'][d]
        a_ = rotate(np.broadcast_to(ang, (B, 3)), ar_)
        cang0[:, d] = a_
        cvel0[:, d] = rotate(np.broadcast_to(vel, (B, 3)), ar_) + cross(ap_, a_)
        raw = quat_rot_axis(np.broadcast_to(ang, (B, 3)), q[:, qa + k])
        rk = normalize(raw)
        pk = vel * q[:, qa + k, None]
        recs.append(dict(ap=ap_, ar=ar_, raw=raw, rk=rk, pk=pk))
        ap_, ar_ = tf_do_tf(ap_, ar_, pk, rk)
      stack[i] = recs
    T.update(cang0=cang0, cvel0=cvel0, stack=stack)
    # contacts
    T['contacts'] = self._contacts(s.x_pos, s.x_rot)
    # accelerations
    tau = o.to_tau(act, q, qd)
    qfs = o.forward(s, tau)
    s = s.replace(qf_smooth=qfs)
    jac, diag, aref, minv = s.con_jac, s.con_diag, s.con_aref, s.mass_mx_inv
    m = jac.shape[1]
    if m:
      jm = jac @ minv
      a = jm @ np.swapaxes(jac, -1, -2) + np.einsum('bi,ij->bij', diag, np.eye(m))
      b = np.einsum('bij,bj->bi', jm, qfs) - aref
      xs, pg = self._pg_tape(a, b)
      qfc = np.einsum('bij,bi->bj', jac, xs)
      T.update(a=a, b=b, xs=xs, pg=pg, pg_gap=self.last_gap, proj_gap=self.last_proj_gap)
    else:
      qfc = np.zeros_like(qfs)
      T.update(pg_gap=np.full(B, np.inf), proj_gap=np.full(B, np.inf))
    s = s.replace(qf_constraint=qfc)
    s2 = o.integrate(s)
    T.update(qfs=qfs, qfc=qfc, s_int=s2)
    return s2.q, s2.qd, T

  def _contacts(self, xp, xr):
    c, cs = self.c, self.sys.contacts
    out = []
    for k in range(cs.n):
      g1, g2, lb, sub = cs.geom1[k], cs.geom2[k], int(cs.link_b[k]), int(cs.sub[k])
      B = xp.shape[0]
      n = np.broadcast_to(quat_to_3x3(c['geom_quat'][g1])[:, 2], (B, 3))
      p1 = c['geom_pos'][g1]
      gpos, gquat = c['geom_pos'][g2], c['geom_quat'][g2]
      gq = quat_mul(xr[:, lb], np.broadcast_to(gquat, (B, 4)))
      p2 = xp[:, lb] + rotate(np.broadcast_to(gpos, (B, 3)), xr[:, lb])
      R2 = quat_to_3x3(gq)
      r = c['geom_size'][g2, 0]
      rec = dict(kind=cs.kind[k], lb=lb, sub=sub, n=n, p1=p1, gq=gq, gpos=gpos, gquat=gquat, r=r)
      if cs.kind[k] == S.CON_PLANE_CAPSULE:
        axis = R2[:, :, 2]
        h = c['geom_size'][g2, 1]
        center = p2 + axis * h if sub == 0 else p2 - axis * h
        w = axis - n * dot(n, axis)[:, None]
        rec.update(axis=axis, h=h, w=w)
      else:
        center = p2
      dist, pos = _plane_sphere(n, p1, center, r)
      rec.update(center=center, dist=dist, pos=pos)
      out.append(rec)
    return out

  def _pg_tape(self, a, b):
    """Oracle.pg_solve's iteration, recording what the reverse needs.

    With self.force = (iterations, step sizes) set (one env), the solve takes
    exactly those iterations and accepted step sizes instead of its own
    stopping and line-search decisions: the branch another implementation
    took (a GPU tape), so that its reverse can be compared on the same
    branch."""
    sys = self.sys
    force = getattr(self, 'force', None)
    B, m = b.shape
    relu = lambda v: np.maximum(v, 0)
    mv = lambda x: np.einsum('bij,bj->bi', a, x)
    mvt = lambda r: np.einsum('bij,bi->bj', a, r)
    x = np.zeros((B, m))
    y = np.zeros((B, m))
    t = np.ones(B)
    ss = np.ones(B)
    err = np.full(B, np.inf)
    active = np.ones(B, bool)
    tape = []
    # the closest call of any decision of the solve, relative to the compared
    # values' size: below ~1e-6 the same decision in FP32 is a tie
    gap = np.full(B, np.inf)
    # the closest call of the projection: a component of y - step grad that
    # cancels to within this fraction of its terms is a tie of its sign
    pgap = np.full(B, np.inf)
    for it in range(sys.solver_iterations):
      if force is not None:
        if it >= force[0]:
          break
      else:
        if it > 0:
          active = active & (err > 1e-3)
        if not active.any():
          break
      ry = mv(y) + b
      fy = np.sum(0.5 * ry ** 2, -1)
      gy = mvt(ry)
      cur = ss.copy() if force is None else np.full(B, float(force[1][it]))
      nx = relu(y + (-cur)[:, None] * gy)
      on = active.copy() if force is None else np.zeros(B, bool)
      for _ in range(sys.solver_maxls if force is None else 0):
        dx = nx - y
        r2 = mv(nx) + b
        f2 = np.sum(0.5 * r2 ** 2, -1)
        lhs, rhs = cur * (f2 - fy), cur * np.sum(dx * gy, -1) + 0.5 * np.sum(dx * dx, -1)
        scale = np.abs(cur * f2) + np.abs(cur * fy) + cur * np.sum(np.abs(dx * gy), -1) + 0.5 * np.sum(dx * dx, -1)
        # a trial point equal to y (|dx| = 0) is accepted in any precision
        sqd = np.sum(dx * dx, -1)
        gap = np.where(on & (sqd > 0), np.minimum(gap, np.abs(lhs - rhs) / np.maximum(scale, 1e-300)), gap)
        cond = lhs > rhs
        on = on & cond
        if not on.any():
          break
        cur = np.where(on, cur * 0.5, cur)
        nx = np.where(on[:, None], relu(y + (-cur)[:, None] * gy), nx)
      nss = np.where(cur <= 1e-6, 1.0, cur / 0.5)
      nt = 0.5 * (1 + np.sqrt(1 + 4 * t ** 2))
      beta = (t - 1) / nt
      ny = nx + beta[:, None] * (nx - x)
      gx = mvt(mv(nx) + b)
      e = np.sqrt(np.sum((relu(nx - gx) - nx) ** 2, -1))
      z = y - cur[:, None] * gy
      zs = np.abs(y) + cur[:, None] * np.abs(gy)
      pz = np.where(zs > 0, np.abs(z) / np.maximum(zs, 1e-300), np.inf).min(-1) if m else np.full(B, np.inf)
      pgap = np.where(active, np.minimum(pgap, pz), pgap)
      tape.append(dict(active=active.copy(), y=y.copy(), ry=ry, step=cur.copy(), beta=beta,
                       zpos=(z > 0)))
      gap = np.where(active, np.minimum(gap, np.abs(e - 1e-3) / 1e-3), gap)
      on2 = active[:, None]
      x = np.where(on2, nx, x)
      y = np.where(on2, ny, y)
      t = np.where(active, nt, t)
      ss = np.where(active, nss, ss)
      err = np.where(active, e, err)
    self.last_gap = gap
    self.last_proj_gap = pgap
    return x, tape

  # -------------------------------------------------------------- reverse
  def vjp(self, T, qb_out, qdb_out, minvb_out=None):
    """(q'_bar, qd'_bar) -> (q_bar, qd_bar, act_bar); minvb_out: the
    cotangent of the inverse this step carries on (Newton-Schulz mode)."""
    st, c, sys = self.st, self.c, self.sys
    s = T['s']
    q, qd = T['q'], T['qd']
    B, nv = q.shape[0], st.nv
    h = c['dt']
    qb = np.zeros_like(q)
    qdb = np.zeros_like(qd)
    s2 = T['s_int']
    # ---- integrator (integrator.py:46-84) ----
    qdnb = qdb_out.copy()
    for i, t in enumerate(st.types):
      qa, da = st.qadr[i], st.dadr[i]
      if t == 'f':
        qb[:, qa:qa + 3] += qb_out[:, qa:qa + 3]
        qdnb[:, da:da + 3] += h * qb_out[:, qa:qa + 3]
        rot0, ang = q[:, qa + 3:qa + 7], s2.qd[:, da + 3:da + 6]
        n = np.sqrt(np.sum(ang * ang, -1))
        an = n + 1e-8
        qrot = quat_rot_axis(ang / an[:, None], h * an)
        prod = quat_mul(rot0, qrot)
        prodb = normalize_vjp(prod, qb_out[:, qa + 3:qa + 7])
        rotb, qrotb = qmul_vjp(rot0, qrot, prodb)
        qb[:, qa + 3:qa + 7] += rotb
        sn, cs_ = np.sin(h * an / 2), np.cos(h * an / 2)
        f = sn / an
        dfdan = (cs_ * h / 2 * an - sn) / an ** 2
        unit = ang / np.maximum(n, 1e-30)[:, None]
        qvb = qrotb[:, 1:]
        angb = ((qrotb[:, 0] * (-sn / 2 * h))[:, None] * unit + f[:, None] * qvb
                + (dot(ang, qvb) * dfdan)[:, None] * unit)
        qdnb[:, da + 3:da + 6] += angb
      else:
        k = int(t)
        qb[:, qa:qa + k] += qb_out[:, qa:qa + k]
        qdnb[:, da:da + k] += h * qb_out[:, qa:qa + k]
    qdb += qdnb
    qddb = h * qdnb
    # ---- qdd = Minv (qfs + qfc) ----
    minv = s.mass_mx_inv
    v = T['qfs'] + T['qfc']
    minvb = np.einsum('bi,bj->bij', qddb, v)
    vb = np.einsum('bji,bj->bi', minv, qddb)
    qfsb = vb.copy()
    qfcb = vb.copy()
    jac = s.con_jac
    m = jac.shape[1]
    jacb = np.zeros_like(jac)
    diagb = np.zeros((B, m))
    arefb = np.zeros((B, m))
    if m:
      jacb += np.einsum('bi,bj->bij', T['xs'], qfcb)  # qfc = J^T x
      xb = np.einsum('bij,bj->bi', jac, qfcb)
      ab, bb = self._pg_vjp(T, xb)
      jacb += np.einsum('bij,bjk,bkl->bil', ab, jac, np.swapaxes(minv, -1, -2))
      jacb += np.einsum('bji,bjk,bkl->bil', ab, jac, minv)
      minvb += np.einsum('bki,bkl,blj->bij', jac, ab, jac)
      diagb += np.einsum('bii->bi', ab)
      u = np.einsum('bij,bj->bi', minv, T['qfs'])  # b = J Minv qfs - aref
      jacb += np.einsum('bi,bj->bij', bb, u)
      tb = np.einsum('bij,bi->bj', jac, bb)
      minvb += np.einsum('bi,bj->bij', tb, T['qfs'])
      qfsb += np.einsum('bji,bj->bi', minv, tb)
      arefb -= bb
    # ---- qf_smooth = passive - bias + tau (dynamics.py:187-236, actuator.py) ----
    for i, t in enumerate(st.types):
      if t == 'f':
        continue
      for k in range(int(t)):
        d = st.dadr[i] + k
        qb[:, st.qadr[i] + k] += -c['stiffness'][d] * qfsb[:, d]
    qdb += -c['damping'] * qfsb
    actb = self._actuator_vjp(T, qfsb, qb, qdb)
    P = {k: np.zeros_like(getattr(s, k)) for k in
         ('cinr_i', 'cinr_pos', 'cd_ang', 'cd_vel', 'cdof_ang', 'cdof_vel', 'cdofd_ang',
          'cdofd_vel', 'root_com', 'x_pos', 'x_rot')}
    self._rne_vjp(s, -qfsb, P, qdb)
    # ---- the inverse (exact, or the Newton-Schulz update of the carried one), CRBA ----
    if minvb_out is not None:
      minvb = minvb + minvb_out
    if 'ns' in T:
      mb, self.minvb_prev = ns_vjp(T['ns'], minvb)
    else:
      mb = -np.swapaxes(minv, -1, -2) @ minvb @ np.swapaxes(minv, -1, -2)
      self.minvb_prev = None
    self._crba_vjp(s, mb, P)
    # ---- constraint rows ----
    if m:
      self._rows_vjp(T, jacb, diagb, arefb, P, qb, qdb)
    # ---- transform_com, kinematics ----
    self._com_vjp(T, P, qb, qdb)
    self._fk_vjp(T, P, qb)
    return qb, qdb, actb

  def _pg_vjp(self, T, xb):
    a = T['a']
    mv = lambda x: np.einsum('bij,bj->bi', a, x)
    mvt = lambda r: np.einsum('bij,bi->bj', a, r)
    ab = np.zeros_like(a)
    bb = np.zeros_like(T['b'])
    xbar, ybar = xb.copy(), np.zeros_like(xb)
    for rec in reversed(T['pg']):
      on = rec['active'][:, None]
      beta = rec['beta'][:, None]
      nxb = xbar + (1 + beta) * ybar
      xprevb = -beta * ybar
      zb = nxb * rec['zpos']
      gb = -rec['step'][:, None] * zb
      # g = A^T r, r = A y + b
      ab_k = np.einsum('bi,bj->bij', rec['ry'], gb)
      rb = mv(gb)
      ab_k += np.einsum('bi,bj->bij', rb, rec['y'])
      yb = zb + mvt(rb)
      ab += np.where(on[:, :, None], ab_k, 0.0)
      bb += np.where(on, rb, 0.0)
      xbar = np.where(on, xprevb, xbar)
      ybar = np.where(on, yb, ybar)
    return ab, bb

  def _actuator_vjp(self, T, taub, qb, qdb):
    c, sys = self.c, self.sys
    act, q, qd = T['act'], T['q'], T['qd']
    nu = sys.act_size()
    actb = np.zeros((q.shape[0], nu))
    if nu and act is not None:
      qid, qdid = sys.actuator.q_id, sys.actuator.qd_id
      inu = clip_grad(act, c['a_cr'][:, 0], c['a_cr'][:, 1])
      u = np.clip(act, c['a_cr'][:, 0], c['a_cr'][:, 1])
      f0 = c['a_gain'] * u + c['a_gear'] * (q[:, qid] * c['a_bq'] + qd[:, qdid] * c['a_bqd'])
      inf = clip_grad(f0, c['a_fr'][:, 0], c['a_fr'][:, 1])
      fb = taub[:, qdid] * c['a_gear'] * inf
      actb = fb * c['a_gain'] * inu
      for k in range(nu):
        qb[:, qid[k]] += fb[:, k] * c['a_gear'][k] * c['a_bq'][k]
        qdb[:, qdid[k]] += fb[:, k] * c['a_gear'][k] * c['a_bqd'][k]
    return actb

  def _rne_vjp(self, s, biasb, P, qdb):
    st, c = self.st, self.c
    B = s.q.shape[0]
    cdd_a = np.zeros((B, st.nl, 3))
    cdd_v = np.zeros((B, st.nl, 3))
    for lvl in st.levels:
      for i in lvl:
        p = st.parents[i]
        a_ = cdd_a[:, p].copy() if p >= 0 else np.zeros((B, 3))
        v_ = cdd_v[:, p].copy() if p >= 0 else np.broadcast_to(-c['gravity'], (B, 3)).copy()
        for d in range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[st.types[i]]):
          a_ = a_ + s.cdofd_ang[:, d] * s.qd[:, d, None]
          v_ = v_ + s.cdofd_vel[:, d] * s.qd[:, d, None]
        cdd_a[:, i], cdd_v[:, i] = a_, v_
    ga, gv = inertia_mul(s.cinr_i, s.cinr_pos, s.cinr_mass, s.cd_ang, s.cd_vel)
    fa, fv = inertia_mul(s.cinr_i, s.cinr_pos, s.cinr_mass, cdd_a, cdd_v)
    xa, xv = force_cross(s.cd_ang, s.cd_vel, ga, gv)
    cfa, cfv = fa + xa, fv + xv
    for lvl in reversed(st.levels):
      for i in lvl:
        for ch in st.children[i]:
          cfa[:, i] = cfa[:, i] + cfa[:, ch]
          cfv[:, i] = cfv[:, i] + cfv[:, ch]
    dl = st.dof_link
    P['cdof_vel'] += biasb[:, :, None] * cfv[:, dl]
    P['cdof_ang'] += biasb[:, :, None] * cfa[:, dl]
    cfab = np.zeros_like(cfa)
    cfvb = np.zeros_like(cfv)
    for d in range(st.nv):
      cfvb[:, dl[d]] += biasb[:, d, None] * s.cdof_vel[:, d]
      cfab[:, dl[d]] += biasb[:, d, None] * s.cdof_ang[:, d]
    for lvl in st.levels:  # reverse of the leaf-to-root sum
      for i in lvl:
        for ch in st.children[i]:
          cfab[:, ch] += cfab[:, i]
          cfvb[:, ch] += cfvb[:, i]
    ib, pb, cddab, cddvb = inertia_mul_vjp(s.cinr_i, s.cinr_pos, s.cinr_mass, cdd_a, cdd_v, cfab, cfvb)
    P['cinr_i'] += ib
    P['cinr_pos'] += pb
    sab, svb, gab, gvb = force_cross_vjp(s.cd_ang, s.cd_vel, ga, gv, cfab, cfvb)
    ib2, pb2, cdab2, cdvb2 = inertia_mul_vjp(s.cinr_i, s.cinr_pos, s.cinr_mass, s.cd_ang, s.cd_vel,
                                             gab, gvb)
    P['cinr_i'] += ib2
    P['cinr_pos'] += pb2
    P['cd_ang'] += sab + cdab2
    P['cd_vel'] += svb + cdvb2
    for lvl in reversed(st.levels):  # cdd = cdd[parent] + sum(cdofd qd)
      for i in lvl:
        for d in range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[st.types[i]]):
          P['cdofd_ang'][:, d] += cddab[:, i] * s.qd[:, d, None]
          P['cdofd_vel'][:, d] += cddvb[:, i] * s.qd[:, d, None]
          qdb[:, d] += dot(s.cdofd_ang[:, d], cddab[:, i]) + dot(s.cdofd_vel[:, d], cddvb[:, i])
        p = st.parents[i]
        if p >= 0:
          cddab[:, p] += cddab[:, i]
          cddvb[:, p] += cddvb[:, i]

  def _crba_vjp(self, s, mb, P):
    st = self.st
    crb_i, crb_p, crb_m = s.cinr_i.copy(), s.cinr_pos.copy(), s.cinr_mass.copy()
    for lvl in reversed(st.levels):
      for i in lvl:
        for ch in st.children[i]:
          crb_i[:, i] += crb_i[:, ch]
          crb_p[:, i] += crb_p[:, ch]
          crb_m[:, i] += crb_m[:, ch]
    dl = st.dof_link
    fa, fv = inertia_mul(crb_i[:, dl], crb_p[:, dl], crb_m[:, dl], s.cdof_ang, s.cdof_vel)
    vb = mb + np.swapaxes(mb, -1, -2)
    idx = np.arange(st.nv)
    vb[:, idx, idx] = mb[:, idx, idx]
    fab = np.zeros_like(fa)
    fvb = np.zeros_like(fv)
    for r in range(st.nv):
      for cc in range(r + 1):
        if dl[cc] not in self.anc[r]:
          continue
        w = vb[:, r, cc][:, None]
        P['cdof_vel'][:, cc] += w * fv[:, r]
        P['cdof_ang'][:, cc] += w * fa[:, r]
        fvb[:, r] += w * s.cdof_vel[:, cc]
        fab[:, r] += w * s.cdof_ang[:, cc]
    ib, pb, mab, mvb = inertia_mul_vjp(crb_i[:, dl], crb_p[:, dl], crb_m[:, dl], s.cdof_ang,
                                       s.cdof_vel, fab, fvb)
    P['cdof_ang'] += mab
    P['cdof_vel'] += mvb
    crbib = np.zeros_like(crb_i)
    crbpb = np.zeros_like(crb_p)
    for d in range(st.nv):
      crbib[:, dl[d]] += ib[:, d]
      crbpb[:, dl[d]] += pb[:, d]
    for lvl in st.levels:
      for i in lvl:
        for ch in st.children[i]:
          crbib[:, ch] += crbib[:, i]
          crbpb[:, ch] += crbpb[:, i]
    P['cinr_i'] += crbib
    P['cinr_pos'] += crbpb

  def _rows_vjp(self, T, jacb, diagb, arefb, P, qb, qdb):
    st, c, sys = self.st, self.c, self.sys
    s = T['s']
    q, qd = T['q'], T['qd']
    ncon = sys.contacts.n
    if sys.dof.limit is not None:  # constraint.py:101-132
      q_idx, qd_idx = sys.q_idx('123'), sys.qd_idx('123')
      pmin = q[:, q_idx] - c['lo'][qd_idx]
      pmax = c['hi'][qd_idx] - q[:, q_idx]
      pos = np.minimum(np.minimum(pmin, pmax), 0)
      side = ((pmin < pmax) * 2 - 1) * (pos < 0)
      imp, dimp, bco, kco = imp_parts(c['solp'][qd_idx], pos, side * qd[:, qd_idx])
      act = (pos < 0)
      ab = arefb[:, 4 * ncon:] * act
      db = diagb[:, 4 * ncon:] * act
      qdb[:, qd_idx] += -bco * ab * side
      impb = -kco * pos * ab + db * c['d_invw'][qd_idx] * _ddiag_dimp(imp)
      posb = -kco * imp * ab + impb * dimp
      gq = posb * (((pmin <= pmax) & act) * 1.0 - ((pmax < pmin) & act) * 1.0)
      for k, qi in enumerate(q_idx):
        qb[:, qi] += gq[:, k]
    for k, rec in enumerate(T['contacts']):  # constraint.py:135-176
      actv = rec['dist'] < 0
      if not actv.any():
        continue
      lb = rec['lb']
      mu = c['c_fric'][k, 0]
      rows = s.con_jac[:, 4 * k:4 * k + 4]
      vel = np.einsum('brv,bv->br', rows, qd)
      p4 = np.repeat(rec['dist'][:, None], 4, 1)
      params = np.concatenate([c['c_solref'][k], c['c_solimp'][k]])
      imp, dimp, bco, kco = imp_parts(params, p4, vel)
      ab = arefb[:, 4 * k:4 * k + 4] * actv[:, None]
      db = diagb[:, 4 * k:4 * k + 4] * actv[:, None]
      jb = jacb[:, 4 * k:4 * k + 4] * actv[:, None, None]
      velb = -bco * ab
      jb = jb + velb[:, :, None] * qd[:, None, :]
      qdb += np.einsum('br,brv->bv', velb, rows)
      tw = c['l_invw'][lb]
      impb = -kco * p4 * ab + db * (tw + mu * mu * tw) * 2 * mu * mu * _ddiag_dimp(imp)
      distb = np.sum(-kco * imp * ab + impb * dimp, -1)
      # rows = diff . v_q with v_q = -t * (-+mu) + n
      _, _, frame = self.o.contacts(s.x_pos, s.x_rot)
      n, t1, t2 = frame[:, k, 0], frame[:, k, 1], frame[:, k, 2]
      vs = [(-t1) * (-mu) + n, (-t1) * mu + n, (-t2) * (-mu) + n, (-t2) * mu + n]
      _, diff = self.o.point_jacobian(s, rec['pos'], lb)  # link_a is the world
      diffb = np.zeros_like(diff)
      vbs = []
      for qq in range(4):
        diffb += jb[:, qq, :, None] * vs[qq][:, None, :]
        vbs.append(np.einsum('bv,bvj->bj', jb[:, qq], diff))
      t1b = mu * vbs[0] - mu * vbs[1]
      t2b = mu * vbs[2] - mu * vbs[3]
      ancl = self._anc_links(lb)
      mask = np.array([1.0 if st.dof_link[d] in ancl else 0.0 for d in range(st.nv)])
      jbm = diffb * mask[None, :, None]
      off = rec['pos'] - s.root_com[:, lb]
      P['cdof_vel'] += jbm
      offb = -np.sum(cross(s.cdof_ang, jbm), axis=1)   # y = v - off x a
      P['cdof_ang'] += -cross(jbm, off[:, None, :])
      P['root_com'][:, lb] -= offb
      self._contact_geom_vjp(rec, t1b * actv[:, None], t2b * actv[:, None], distb * actv,
                             offb * actv[:, None], P)

  def _anc_links(self, link):
    a_, j = set(), link
    while j >= 0:
      a_.add(j)
      j = self.st.parents[j]
    return a_

  def _contact_geom_vjp(self, rec, t1b, t2b, distb, posb, P):
    n = rec['n']
    lb = rec['lb']
    B = distb.shape[0]
    centerb = posb.copy()                       # pos = center - n (r + 0.5 dist)
    distb = distb - 0.5 * dot(posb, n)
    centerb = centerb + distb[:, None] * n      # dist = (center - p1) . n - r
    p2b = centerb.copy()
    R2b = np.zeros((B, 3, 3))
    if rec['kind'] == S.CON_PLANE_CAPSULE:
      sgn = 1.0 if rec['sub'] == 0 else -1.0
      axisb = sgn * rec['h'] * centerb
      _, bn = _norm_with_norm(rec['w'])
      bb = t1b + cross(t2b, n)                  # t1 = b, t2 = n x b
      wb = np.where((bn >= 0.5)[:, None], normalize_vjp(rec['w'], bb), 0.0)
      axisb = axisb + wb - n * dot(n, wb)[:, None]
      R2b[:, :, 2] = axisb
    xr = self._xr
    gqb = quat_to_3x3_vjp(rec['gq'], R2b)
    xrb, _ = qmul_vjp(xr[:, lb], np.broadcast_to(rec['gquat'], (B, 4)), gqb)
    _, xrb2 = rotate_vjp(np.broadcast_to(rec['gpos'], (B, 3)), xr[:, lb], p2b)
    P['x_pos'][:, lb] += p2b
    P['x_rot'][:, lb] += xrb + xrb2

  def _com_vjp(self, T, P, qb, qdb):
    st, c = self.st, self.c
    s = T['s']
    B = s.q.shape[0]
    qd = T['qd']
    dl = st.dof_link
    cdab, cdvb = P['cd_ang'], P['cd_vel']
    cang, cvel = s.cdof_ang, s.cdof_vel
    # cdofd (dynamics.py:106-130)
    for i, t in enumerate(st.types):
      da = st.dadr[i]
      if t == 'f':
        sa = cang[:, da] * qd[:, da, None] + cang[:, da + 1] * qd[:, da + 1, None] + cang[:, da + 2] * qd[:, da + 2, None]
        sv = cvel[:, da] * qd[:, da, None] + cvel[:, da + 1] * qd[:, da + 1, None] + cvel[:, da + 2] * qd[:, da + 2, None]
        sab = np.zeros((B, 3))
        svb = np.zeros((B, 3))
        for k in range(3, 6):
          d = da + k
          a1, v1, oab, ovb = motion_cross_vjp(sa, sv, cang[:, d], cvel[:, d], P['cdofd_ang'][:, d],
                                              P['cdofd_vel'][:, d])
          sab, svb = sab + a1, svb + v1
          P['cdof_ang'][:, d] += oab
          P['cdof_vel'][:, d] += ovb
        for k in range(3):
          d = da + k
          P['cdof_ang'][:, d] += qd[:, d, None] * sab
          P['cdof_vel'][:, d] += qd[:, d, None] * svb
          qdb[:, d] += dot(cang[:, d], sab) + dot(cvel[:, d], svb)
        continue
      p = st.parents[i]
      sas, svs = [], []
      sa = s.cd_ang[:, p] if p >= 0 else np.zeros((B, 3))
      sv = s.cd_vel[:, p] if p >= 0 else np.zeros((B, 3))
      for k in range(int(t)):
        d = da + k
        sas.append(sa)
        svs.append(sv)
        sa, sv = sa + cang[:, d] * qd[:, d, None], sv + cvel[:, d] * qd[:, d, None]
      sab = np.zeros((B, 3))
      svb = np.zeros((B, 3))
      for k in reversed(range(int(t))):
        d = da + k
        # s_{k+1} = s_k + cdof_k qd_k : the carried adjoint applies to cdof_k, qd_k
        P['cdof_ang'][:, d] += qd[:, d, None] * sab
        P['cdof_vel'][:, d] += qd[:, d, None] * svb
        qdb[:, d] += dot(cang[:, d], sab) + dot(cvel[:, d], svb)
        a1, v1, oab, ovb = motion_cross_vjp(sas[k], svs[k], cang[:, d], cvel[:, d], P['cdofd_ang'][:, d],
                                            P['cdofd_vel'][:, d])
        sab, svb = sab + a1, svb + v1
        P['cdof_ang'][:, d] += oab
        P['cdof_vel'][:, d] += ovb
      if p >= 0:
        cdab[:, p] += sab
        cdvb[:, p] += svb
    # cd (dynamics.py:93-103): leaf-to-root reverse of the root-to-leaf sum
    for lvl in reversed(st.levels):
      for i in lvl:
        for d in range(st.dadr[i], st.dadr[i] + S.QD_WIDTHS[st.types[i]]):
          P['cdof_ang'][:, d] += qd[:, d, None] * cdab[:, i]
          P['cdof_vel'][:, d] += qd[:, d, None] * cdvb[:, i]
          qdb[:, d] += dot(cang[:, d], cdab[:, i]) + dot(cvel[:, d], cdvb[:, i])
        p = st.parents[i]
        if p >= 0:
          cdab[:, p] += cdab[:, i]
          cdvb[:, p] += cdvb[:, i]
    # cdof = off.do(rotate(cdof0, jj_r)) (dynamics.py:85-89)
    rc, jj_p, jj_r = s.root_com, T['jj_p'], T['jj_r']
    rcb = P['root_com']
    jjpb = np.zeros_like(jj_p)
    jjrb = np.zeros_like(jj_r)
    cang0b = np.zeros_like(cang)
    cvel0b = P['cdof_vel'].copy()
    for d in range(st.nv):
      l = dl[d]
      off2 = rc[:, l] - jj_p[:, l]
      yb = P['cdof_vel'][:, d]
      offb = -cross(cang[:, d], yb)
      angb = P['cdof_ang'][:, d] - cross(yb, off2)
      rcb[:, l] += offb
      jjpb[:, l] -= offb
      a0b, jrb = rotate_vjp(T['cang0'][:, d], jj_r[:, l], angb)
      cang0b[:, d] = a0b
      jjrb[:, l] += jrb
    # stacked joints (dynamics.py:55-83)
    for i, recs in T['stack'].items():
      qa, da = st.qadr[i], st.dadr[i]
      apb = np.zeros((B, 3))
      arb = np.zeros((B, 4))
      for k in reversed(range(len(recs))):
        r = recs[k]
        d = da + k
        # (ap, ar) <- (ap, ar).do(pk, rk) for the next dof
        if k + 1 < len(recs):
          pass
        # accumulated transform adjoint flows from later dofs (handled below)
      # process in reverse with explicit recurrence
      apb = np.zeros((B, 3))
      arb = np.zeros((B, 4))
      for k in reversed(range(len(recs))):
        r = recs[k]
        d = da + k
        ang, vel = c['m_ang'][d], c['m_vel'][d]
        # the transform produced after dof k feeds dof k+1 (apb, arb hold its adjoint)
        if k + 1 < len(recs) or True:
          ap0b, ar0b, pkb, rkb = tf_do_vjp(r['ap'], r['ar'], r['pk'], r['rk'], apb, arb)
          rawb = normalize_vjp(r['raw'], rkb)
          qb[:, qa + k] += quat_rot_axis_vjp_angle(np.broadcast_to(ang, (B, 3)), q_k := T['q'][:, qa + k], rawb)
          qb[:, qa + k] += dot(pkb, np.broadcast_to(vel, (B, 3)))
          apb, arb = ap0b, ar0b
        # cdof0_k = (rotate(ang, ar), rotate(vel, ar) + ap x a_)
        a_ = T['cang0'][:, d]
        vb_ = cvel0b[:, d]
        apb2, ab2 = cross_vjp(r['ap'], a_, vb_)
        _, arb2 = rotate_vjp(np.broadcast_to(vel, (B, 3)), r['ar'], vb_)
        abt = cang0b[:, d] + ab2
        _, arb3 = rotate_vjp(np.broadcast_to(ang, (B, 3)), r['ar'], abt)
        apb = apb + apb2
        arb = arb + arb2 + arb3
    # jj = parent.do(link.transform).do(link.joint)
    xpb, xrb = P['x_pos'], P['x_rot']
    for i in range(st.nl):
      pi, pp, pr, ap, ar = T['a_pr'][i]
      ab_p = jjpb[:, i]
      _, arb1 = rotate_vjp(np.broadcast_to(c['lj_pos'][i], (B, 3)), ar, ab_p)
      arb = jjrb[:, i] + arb1
      ppb, prb, _, _ = tf_do_vjp(pp, pr, c['lt_pos'][i], c['lt_rot'][i], ab_p, arb)
      if pi >= 0:
        xpb[:, pi] += ppb
        xrb[:, pi] += prb
    # cinr (dynamics.py:44, base.py:589-595)
    xi_p, xi_r = T['xi_p'], T['xi_r']
    xipb = np.zeros_like(xi_p)
    xirb = np.zeros_like(xi_r)
    I0 = c['li_i']
    m = c['li_mass']
    for i in range(st.nl):
      Cb = P['cinr_i'][:, i]
      R = quat_to_3x3(xi_r[:, i])
      Rb = (Cb + np.swapaxes(Cb, -1, -2)) @ R @ I0[i]
      xirb[:, i] += quat_to_3x3_vjp(xi_r[:, i], Rb)
      o = xi_p[:, i] - rc[:, i]
      trC = np.trace(Cb, axis1=-2, axis2=-1)
      ob = m[i] * (2 * trC[:, None] * o - np.einsum('bij,bj->bi', Cb + np.swapaxes(Cb, -1, -2), o))
      ob = ob + m[i] * P['cinr_pos'][:, i]
      xipb[:, i] += ob
      rcb[:, i] -= ob
    # root_com (dynamics.py:38-43)
    for r in set(st.roots):
      mem = [i for i in range(st.nl) if st.roots[i] == r]
      mt = sum(m[i] for i in mem)
      tot = sum(rcb[:, i] for i in mem)
      for j in mem:
        xipb[:, j] += m[j] / mt * tot
    # x_i = x.do(inertia.transform)
    for i in range(st.nl):
      xpb_, xrb_, _, _ = tf_do_vjp(s.x_pos[:, i], s.x_rot[:, i], c['li_pos'][i], c['li_rot'][i],
                                   xipb[:, i], xirb[:, i])
      xpb[:, i] += xpb_
      xrb[:, i] += xrb_

  def _fk_vjp(self, T, P, qb):
    st, c = self.st, self.c
    fk = T['fk']
    q = T['q']
    B = q.shape[0]
    xpb = P['x_pos'].copy()
    xrawb = normalize_vjp(fk['xraw'], P['x_rot'])
    jp3b = np.zeros_like(fk['jp3'])
    jr3b = np.zeros_like(fk['jr3'])
    for lvl in reversed(st.levels):
      for i in lvl:
        p = st.parents[i]
        if p < 0:
          jp3b[:, i] += xpb[:, i]
          jr3b[:, i] += xrawb[:, i]
        else:
          ppb, prb, bpb, brb = tf_do_vjp(fk['xp'][:, p], fk['xraw'][:, p], fk['jp3'][:, i],
                                         fk['jr3'][:, i], xpb[:, i], xrawb[:, i])
          xpb[:, p] += ppb
          xrawb[:, p] += prb
          jp3b[:, i] += bpb
          jr3b[:, i] += brb
    # (jp3, jr3) = link.transform.do((jp2, jr))
    jp2b, _ = rotate_vjp(fk['jp2'], np.broadcast_to(c['lt_rot'], fk['jr'].shape), jp3b)
    _, jrb = qmul_vjp(np.broadcast_to(c['lt_rot'], fk['jr'].shape), fk['jr'], jr3b)
    # jp2 = jp + jpos - rotate(jpos, jr)
    jpos = np.broadcast_to(c['lj_pos'], fk['jp'].shape)
    _, jrb2 = rotate_vjp(jpos, fk['jr'], -jp2b)
    jrb = jrb + jrb2
    jpb = jp2b
    for i, t in enumerate(st.types):
      qa = st.qadr[i]
      if t == 'f':
        qb[:, qa:qa + 3] += jpb[:, i]
        qb[:, qa + 3:qa + 7] += jrb[:, i]
        continue
      pieces = fk['per'][i]
      accpb, accrb = jpb[:, i], jrb[:, i]
      for k in reversed(range(len(pieces))):
        pc = pieces[k]
        d = st.dadr[i] + k
        if k == 0:
          pkb, rkb = accpb, accrb
        else:
          app, arr, pkb, rkb = tf_do_vjp(pc['acc_p'], pc['acc_r'], pc['pk'], pc['rk'], accpb, accrb)
          accpb, accrb = app, arr
        rawb = normalize_vjp(pc['raw'], rkb)
        qb[:, qa + k] += quat_rot_axis_vjp_angle(np.broadcast_to(c['m_ang'][d], (B, 3)), q[:, qa + k], rawb)
        qb[:, qa + k] += dot(pkb, np.broadcast_to(c['m_vel'][d], (B, 3)))

  # -------------------------------------------------------------- drivers
  def step_vjp(self, q, qd, act, qb_out, qdb_out):
    qn, qdn, T = self.forward(q, qd, act)
    self._xr = T['s'].x_rot
    return self.vjp(T, qb_out, qdb_out)
