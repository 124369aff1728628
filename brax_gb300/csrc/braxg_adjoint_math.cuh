// Reverse-mode derivatives of the primitives in braxg_math.cuh (each matches
// jax.grad of the corresponding brax/math.py or brax/base.py function).
#pragma once
#include "braxg_math.cuh"

__device__ __forceinline__ q4 qconj(q4 q) { return q4{q.w, -q.x, -q.y, -q.z}; }
__device__ __forceinline__ q4 qadd(q4 a, q4 b) { return q4{a.w + b.w, a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ q4 qscale(q4 a, float s) { return q4{a.w * s, a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float qdot(q4 a, q4 b) { return a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ void add3(float* p, f3 v) {
  p[0] += v.x;
  p[1] += v.y;
  p[2] += v.z;
}
__device__ __forceinline__ void add4(float* p, q4 v) {
  p[0] += v.w;
  p[1] += v.x;
  p[2] += v.y;
  p[3] += v.z;
}

// r = rotate(v, q): (v_bar, q_bar) from r_bar
__device__ __forceinline__ void rotate_vjp(f3 v, q4 q, f3 rb, f3& vb, q4& qb) {
  f3 u = mk3(q.x, q.y, q.z);
  float s = q.w;
  float ru = dot3(rb, u);
  vb = (2.f * ru) * u + (s * s - dot3(u, u)) * rb + (2.f * s) * cross3(rb, u);
  f3 ub = (2.f * ru) * v + (2.f * dot3(u, v)) * rb - (2.f * dot3(rb, v)) * u + (2.f * s) * cross3(v, rb);
  float sb = 2.f * s * dot3(rb, v) + 2.f * dot3(rb, cross3(u, v));
  qb = q4{sb, ub.x, ub.y, ub.z};
}

// c = qmul(a, b)
__device__ __forceinline__ void qmul_vjp(q4 a, q4 b, q4 cb, q4& ab, q4& bb) {
  ab = qmul(cb, qconj(b));
  bb = qmul(qconj(a), cb);
}

// (op, or) = tf_do(ap, ar, bp, br)
__device__ __forceinline__ void tf_do_vjp(f3 ar_unused_pos, q4 ar, f3 bp, q4 br, f3 opb, q4 orb, f3& apb, q4& arb,
                                          f3& bpb, q4& brb) {
  (void)ar_unused_pos;
  q4 arb1, arb2;
  rotate_vjp(bp, ar, opb, bpb, arb1);
  qmul_vjp(ar, br, orb, arb2, brb);
  apb = opb;
  arb = qadd(arb1, arb2);
}

// y = x / |x| (x nonzero)
__device__ __forceinline__ q4 normalize4_vjp(q4 x, q4 yb) {
  float n = sqrtf(qdot(x, x));
  q4 y = qscale(x, 1.f / n);
  float p = qdot(y, yb);
  return q4{(yb.w - y.w * p) / n, (yb.x - y.x * p) / n, (yb.y - y.y * p) / n, (yb.z - y.z * p) / n};
}
__device__ __forceinline__ f3 normalize3_vjp(f3 x, f3 yb) {
  float n = sqrtf(dot3(x, x));
  f3 y = x * (1.f / n);
  float p = dot3(y, yb);
  return mk3((yb.x - y.x * p) / n, (yb.y - y.y * p) / n, (yb.z - y.z * p) / n);
}

// c = a x b
__device__ __forceinline__ void cross_vjp(f3 a, f3 b, f3 cb, f3& ab, f3& bb) {
  ab = cross3(b, cb);
  bb = cross3(cb, a);
}

// R = quat_to_3x3(q) (row-major R) -> q_bar
__device__ __forceinline__ q4 quat_to_3x3_vjp(q4 q, const float* Rb) {
  float w = q.w, x = q.x, y = q.y, z = q.z;
  float d = w * w + x * x + y * y + z * z;
  float s = 2.f / d;
  float gw = -z * Rb[1] + y * Rb[2] + z * Rb[3] - x * Rb[5] - y * Rb[6] + x * Rb[7];
  float gx = y * Rb[1] + z * Rb[2] + y * Rb[3] - 2.f * x * Rb[4] - w * Rb[5] + z * Rb[6] + w * Rb[7] - 2.f * x * Rb[8];
  float gy = -2.f * y * Rb[0] + x * Rb[1] + w * Rb[2] + x * Rb[3] + z * Rb[5] - w * Rb[6] + z * Rb[7] - 2.f * y * Rb[8];
  float gz = -2.f * z * Rb[0] - w * Rb[1] + x * Rb[2] + w * Rb[3] - 2.f * z * Rb[4] + y * Rb[5] + x * Rb[6] + y * Rb[7];
  float sp = Rb[0] * (-(y * y + z * z)) + Rb[1] * (x * y - w * z) + Rb[2] * (x * z + w * y) +
             Rb[3] * (x * y + w * z) + Rb[4] * (-(x * x + z * z)) + Rb[5] * (y * z - w * x) +
             Rb[6] * (x * z - w * y) + Rb[7] * (y * z + w * x) + Rb[8] * (-(x * x + y * y));
  float c = 2.f * s / d * sp;
  return q4{gw * s - c * w, gx * s - c * x, gy * s - c * y, gz * s - c * z};
}

// (fa, fv) = inertia_mul(I, p, m, ma, mv) -> I_bar (added), p_bar, ma_bar, mv_bar
__device__ __forceinline__ void inertia_mul_vjp(const float* I, f3 p, float m, f3 ma, f3 mv, f3 fab, f3 fvb,
                                                float* Ib, f3& pb, f3& mab, f3& mvb) {
  if (Ib != nullptr) {
    Ib[0] += fab.x * ma.x;
    Ib[1] += fab.x * ma.y;
    Ib[2] += fab.x * ma.z;
    Ib[3] += fab.y * ma.x;
    Ib[4] += fab.y * ma.y;
    Ib[5] += fab.y * ma.z;
    Ib[6] += fab.z * ma.x;
    Ib[7] += fab.z * ma.y;
    Ib[8] += fab.z * ma.z;
  }
  mab = mk3(I[0] * fab.x + I[3] * fab.y + I[6] * fab.z, I[1] * fab.x + I[4] * fab.y + I[7] * fab.z,
            I[2] * fab.x + I[5] * fab.y + I[8] * fab.z);
  f3 pb1, mvb1, pb2, mab2;
  cross_vjp(p, mv, fab, pb1, mvb1);
  cross_vjp(p, ma, -fvb, pb2, mab2);
  pb = pb1 + pb2;
  mab = mab + mab2;
  mvb = mvb1 + m * fvb;
}

// (ra, rv) = motion_cross(sa, sv, oa, ov)
__device__ __forceinline__ void motion_cross_vjp(f3 sa, f3 sv, f3 oa, f3 ov, f3 rab, f3 rvb, f3& sab, f3& svb,
                                                 f3& oab, f3& ovb) {
  f3 s1, o1, s2, o3;
  cross_vjp(sa, oa, rab, s1, o1);
  cross_vjp(sa, ov, rvb, s2, ovb);
  cross_vjp(sv, oa, rvb, svb, o3);
  sab = s1 + s2;
  oab = o1 + o3;
}

// (ra, rv) = force_cross(sa, sv, fa, fv)
__device__ __forceinline__ void force_cross_vjp(f3 sa, f3 sv, f3 fa, f3 fv, f3 rab, f3 rvb, f3& sab, f3& svb,
                                                f3& fab, f3& fvb) {
  f3 s1, s2, f2;
  cross_vjp(sa, fa, rab, s1, fab);
  cross_vjp(sv, fv, rab, svb, fvb);
  cross_vjp(sa, fv, rvb, s2, f2);
  sab = s1 + s2;
  fvb = fvb + f2;
}

// q = quat_rot_axis(axis, angle), axis constant -> angle_bar
__device__ __forceinline__ float quat_rot_axis_vjp_angle(f3 axis, float angle, q4 qb) {
  float s, c;
  sincos_ool(angle * 0.5f, &s, &c);
  return qb.w * (-0.5f * s) + (qb.x * axis.x + qb.y * axis.y + qb.z * axis.z) * (0.5f * c);
}

// _imp_aref (constraint.py:29-65): imp, d imp / d pos, b, k
__device__ __forceinline__ void imp_parts(const float* p, float pos, float& imp, float& dimp, float& b, float& k) {
  float timeconst = p[0], dampratio = p[1], dmin = p[2], dmax = p[3], width = p[4], mid = p[5], power = p[6];
  float x = fabsf(pos) / width;
  float ia = (1.f / pow_fast(mid, power - 1.f)) * pow_fast(x, power);
  float ib = 1.f - (1.f / pow_fast(1.f - mid, power - 1.f)) * pow_fast(1.f - x, power);
  float dia = (1.f / pow_fast(mid, power - 1.f)) * power * pow_fast(x, power - 1.f);
  float dib = (1.f / pow_fast(1.f - mid, power - 1.f)) * power * pow_fast(1.f - x, power - 1.f);
  float y = x < mid ? ia : ib;
  float dy = x < mid ? dia : dib;
  float imp0 = dmin + y * (dmax - dmin);
  imp = fminf(fmaxf(imp0, dmin), dmax);
  dimp = (imp0 > dmin && imp0 < dmax) ? dy * (dmax - dmin) : 0.f;
  if (x > 1.f) {
    imp = dmax;
    dimp = 0.f;
  }
  float sg = pos > 0.f ? 1.f : (pos < 0.f ? -1.f : 0.f);
  dimp = dimp * sg / width;
  b = 2.f / (dmax * timeconst);
  k = 1.f / (dmax * dmax * timeconst * timeconst * dampratio * dampratio);
  b = dampratio <= 0.f ? -dampratio / dmax : b;
  k = timeconst <= 0.f ? -timeconst / (dmax * dmax) : k;
}

// d jnp.clip(x, lo, hi) / dx: jnp.clip is maximum(lo, x) then minimum(hi, .),
// and jax differentiates maximum / minimum with ties split evenly (1 inside,
// 1/2 on a bound, 0 beyond; brax/actuator.py:44,52 clip the controls and forces)
__device__ __forceinline__ float clip_grad(float x, float lo, float hi) {
  const float m = fmaxf(lo, x);
  const float dm = x > lo ? 1.f : (x == lo ? 0.5f : 0.f);
  const float dh = m < hi ? 1.f : (m == hi ? 0.5f : 0.f);
  return dm * dh;
}

__device__ __forceinline__ float ddiag_dimp(float imp) {
  return -1.f / (imp + 1e-8f) - (1.f - imp) / ((imp + 1e-8f) * (imp + 1e-8f));
}
