// Derivatives of the contact primitives between two moving geoms
// (mujoco.mjx sphere-sphere, sphere-capsule and capsule-capsule, as
// stage_contacts restates them): forward mode with dual numbers over the 12
// world-space inputs of a contact -- the geoms' centres p1, p2 and unit axes
// u1, u2 (a capsule's segment runs p - u h .. p + u h) -- through the same
// branches the values take (clamps and the closer of the two candidate
// pairs piecewise constant, as jax.grad treats them); the reverse of the
// constraint rows contracts that 13 x 12 Jacobian of (dist, pos, n, t1, t2)
// with their cotangents.
#pragma once
#include "braxg_adjoint_math.cuh"

namespace braxg {

constexpr int kContactIn = 12;  // p1, u1, p2, u2
// tangents carried per pass: the 12 inputs take kContactIn / kDualLanes
// passes (few registers per pass)
constexpr int kDualLanes = 2;

struct Dn {
  float v;
  float g[kDualLanes];
};
struct D3 {
  Dn x, y, z;
};

__device__ __forceinline__ Dn dn_const(float c) {
  Dn r;
  r.v = c;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = 0.f;
  return r;
}
// input i of the 12, seeded when it is one of this pass's tangents [base, base + kDualLanes)
__device__ __forceinline__ Dn dn_var(float c, int i, int base) {
  Dn r = dn_const(c);
#pragma unroll
  for (int k = 0; k < kDualLanes; ++k)
    if (i == base + k) r.g[k] = 1.f;
  return r;
}
__device__ __forceinline__ Dn operator+(const Dn& a, const Dn& b) {
  Dn r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = a.g[i] + b.g[i];
  return r;
}
__device__ __forceinline__ Dn operator-(const Dn& a, const Dn& b) {
  Dn r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = a.g[i] - b.g[i];
  return r;
}
__device__ __forceinline__ Dn operator-(const Dn& a) {
  Dn r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = -a.g[i];
  return r;
}
__device__ __forceinline__ Dn operator*(const Dn& a, const Dn& b) {
  Dn r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = a.g[i] * b.v + a.v * b.g[i];
  return r;
}
__device__ __forceinline__ Dn operator*(const Dn& a, float s) {
  Dn r;
  r.v = a.v * s;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = a.g[i] * s;
  return r;
}
__device__ __forceinline__ Dn operator+(const Dn& a, float s) {
  Dn r = a;
  r.v = a.v + s;
  return r;
}
__device__ __forceinline__ Dn operator/(const Dn& a, const Dn& b) {
  Dn r;
  r.v = a.v / b.v;
  const float ib = 1.f / b.v;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = (a.g[i] - r.v * b.g[i]) * ib;
  return r;
}
__device__ __forceinline__ Dn dn_sqrt(const Dn& a) {
  Dn r;
  r.v = sqrtf(a.v);
  const float h = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
  for (int i = 0; i < kDualLanes; ++i) r.g[i] = a.g[i] * h;
  return r;
}
// clamp to [lo, hi]: the bound (constant) where the value is clamped
__device__ __forceinline__ Dn dn_clamp(const Dn& a, float lo, float hi) {
  return a.v < lo ? dn_const(lo) : (a.v > hi ? dn_const(hi) : a);
}
__device__ __forceinline__ Dn dn_clamp(const Dn& a, const Dn& lo, const Dn& hi) {  // fminf(fmaxf(a, lo), hi)
  const Dn m = a.v < lo.v ? lo : a;
  return m.v > hi.v ? hi : m;
}

__device__ __forceinline__ D3 d3_var(f3 v, int i0, int base) {
  return D3{dn_var(v.x, i0, base), dn_var(v.y, i0 + 1, base), dn_var(v.z, i0 + 2, base)};
}
__device__ __forceinline__ D3 d3_const(f3 v) { return D3{dn_const(v.x), dn_const(v.y), dn_const(v.z)}; }
__device__ __forceinline__ D3 operator+(const D3& a, const D3& b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(const D3& a, const D3& b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(const D3& a, const Dn& s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 operator*(const D3& a, float s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ Dn d3_dot(const D3& a, const D3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 d3_cross(const D3& a, const D3& b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 d3_val(const D3& a) { return mk3(a.x.v, a.y.v, a.z.v); }

// mjx math.normalize_with_norm
__device__ __forceinline__ D3 d3_normalize_with_norm(const D3& v, Dn& n) {
  n = dn_sqrt(d3_dot(v, v));
  const Dn d = n + (n.v == 0.f ? 1e-6f : 0.f);
  return D3{v.x / d, v.y / d, v.z / d};
}
// brax/math.py normalize (braxg normalize3)
__device__ __forceinline__ D3 d3_normalize(const D3& v) {
  const bool z = fabsf(v.x.v) <= 1e-8f && fabsf(v.y.v) <= 1e-8f && fabsf(v.z.v) <= 1e-8f;
  if (z) return v * (1.f / 1e-6f);  // the reference's zero-vector branch: v / 1e-6
  const Dn n = dn_sqrt(d3_dot(v, v));
  return D3{v.x / n, v.y / n, v.z / n};
}

__device__ __forceinline__ D3 d3_closest_segment_point(const D3& a, const D3& b, const D3& pt) {
  const D3 ab = b - a;
  const Dn t = d3_dot(pt - a, ab) / (d3_dot(ab, ab) + 1e-6f);
  return a + ab * dn_clamp(t, 0.f, 1.f);
}

__device__ __forceinline__ void d3_closest_seg_seg(const D3& a0, const D3& a1, const D3& b0, const D3& b1, D3& ba,
                                                   D3& bb) {
  Dn la, lb;
  const D3 da = d3_normalize_with_norm(a1 - a0, la);
  const D3 db = d3_normalize_with_norm(b1 - b0, lb);
  const Dn ha = la * 0.5f, hb = lb * 0.5f;
  const D3 am = a0 + da * ha, bm = b0 + db * hb;
  const D3 tr = am - bm;
  const Dn dd = d3_dot(da, db), dat = d3_dot(da, tr), dbt = d3_dot(db, tr);
  const Dn denom = dn_const(1.f) - dd * dd;
  const Dn ta0 = (-dat + dd * dbt) / (denom + 1e-6f);
  const Dn tb0 = dbt + ta0 * dd;
  const Dn ta = dn_clamp(ta0, -ha, ha), tb = dn_clamp(tb0, -hb, hb);
  const D3 besta = am + da * ta, bestb = bm + db * tb;
  const D3 na = d3_closest_segment_point(a0, a1, bestb);
  const D3 nb = d3_closest_segment_point(b0, b1, besta);
  const Dn d1 = d3_dot(bestb - na, bestb - na), d2 = d3_dot(besta - nb, besta - nb);
  if (d1.v < d2.v) {
    ba = na;
    bb = bestb;
  } else {
    ba = besta;
    bb = nb;
  }
}

// sphere_sphere + make_frame: dist, pos and the frame rows n, t1, t2
__device__ __forceinline__ void d3_sphere_sphere_frame(const D3& p1, float r1, const D3& p2, float r2, Dn& dist,
                                                       D3& pos, D3& n, D3& t1, D3& t2) {
  Dn d;
  n = d3_normalize_with_norm(p2 - p1, d);
  if (d.v == 0.f) n = d3_const(mk3(1.f, 0.f, 0.f));
  dist = d + (-(r1 + r2));
  pos = p1 + n * (dist * 0.5f + r1);
  // make_frame(n): n is normalised again there, then the second row is the
  // axis e (y, or z when |n.y| >= 0.5) made orthogonal to it
  const D3 a = d3_normalize(n);
  const f3 e = (-0.5f < a.y.v && a.y.v < 0.5f) ? mk3(0.f, 1.f, 0.f) : mk3(0.f, 0.f, 1.f);
  const D3 b = d3_const(e) - a * d3_dot(a, d3_const(e));
  const bool any = (a.x.v != 0.f) || (a.y.v != 0.f) || (a.z.v != 0.f);
  n = a;
  t1 = any ? d3_normalize(b) : d3_const(mk3(0.f, 0.f, 0.f));
  t2 = d3_cross(a, t1);
}

// The reverse of the contact of a two-geom slot (kind: BXM_CON_SPHERE_SPHERE,
// BXM_CON_SPHERE_CAPSULE, BXM_CON_CAPSULE_CAPSULE): from the cotangents `cot`
// of (dist, pos (3), n (3), t1 (3), t2 (3)), those of the inputs p1, u1, p2,
// u2 into `inb` (12).
static __device__ __noinline__ void two_geom_contact_vjp(int kind, f3 p1v, f3 u1v, float r1, float h1, f3 p2v, f3 u2v,
                                                         float r2, float h2, const float* cot, float* inb) {
  for (int base = 0; base < kContactIn; base += kDualLanes) {
    const D3 p1 = d3_var(p1v, 0, base), u1 = d3_var(u1v, 3, base), p2 = d3_var(p2v, 6, base),
             u2 = d3_var(u2v, 9, base);
    D3 a = p1, b = p2;
    if (kind == BXM_CON_SPHERE_CAPSULE) {
      const D3 s2 = u2 * h2;
      b = d3_closest_segment_point(p2 - s2, p2 + s2, p1);
    } else if (kind == BXM_CON_CAPSULE_CAPSULE) {
      const D3 s1 = u1 * h1, s2 = u2 * h2;
      d3_closest_seg_seg(p1 - s1, p1 + s1, p2 - s2, p2 + s2, a, b);
    }
    Dn dist;
    D3 pos, n, t1, t2;
    d3_sphere_sphere_frame(a, r1, b, r2, dist, pos, n, t1, t2);
#pragma unroll
    for (int k = 0; k < kDualLanes; ++k) {
      const float g[13] = {dist.g[k], pos.x.g[k], pos.y.g[k], pos.z.g[k], n.x.g[k], n.y.g[k], n.z.g[k],
                           t1.x.g[k], t1.y.g[k], t1.z.g[k], t2.x.g[k], t2.y.g[k], t2.z.g[k]};
      float acc = 0.f;
      for (int o = 0; o < 13; ++o) acc += cot[o] * g[o];
      inb[base + k] = acc;
    }
  }
}

// The contact of a two-geom slot (values, as stage_contacts computes them):
// dist, pos and the frame rows n, t1, t2.  Out of line: the constraint-row
// reverse calls it only for such slots.
static __device__ __noinline__ void two_geom_contact(int kind, f3 p1, f3 u1, float r1, float h1, f3 p2, f3 u2,
                                                     float r2, float h2, float* out) {
  f3 ca = p1, cb = p2, n, pos;
  float dist;
  if (kind == BXM_CON_SPHERE_CAPSULE) {
    cb = closest_segment_point(p2 - u2 * h2, p2 + u2 * h2, p1);
  } else if (kind == BXM_CON_CAPSULE_CAPSULE) {
    closest_seg_seg(p1 - u1 * h1, p1 + u1 * h1, p2 - u2 * h2, p2 + u2 * h2, ca, cb);
  }
  sphere_sphere(ca, r1, cb, r2, dist, pos, n);
  out[0] = dist;
  st3(out + 1, pos);
  make_frame(n, out + 4);  // rows n, t1, t2
}

// The manifold vertex of a plane-box slot (box frame; -1: the slot repeats
// an earlier vertex and is inactive).  Out of line, as two_geom_contact.
static __device__ __noinline__ int plane_box_vertex(f3 p1, f3 n, f3 p2, const float* R2, f3 h, int sub) {
  float dd;
  f3 pp;
  int v = -1;
  plane_box(p1, n, p2, R2, h, sub, dd, pp, &v);
  return v;
}

}  // namespace braxg
