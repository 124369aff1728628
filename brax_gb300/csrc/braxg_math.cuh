// Small-vector, quaternion and spatial-algebra helpers for the step kernel.
// Formulas follow brax/math.py and brax/base.py term for term so that the
// FP32 results track the reference's FP32 arithmetic.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

struct f3 {
  float x, y, z;
};
struct q4 {
  float w, x, y, z;
};

constexpr float kPi = 3.14159265358979323846f;

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 ld3(const float* p) { return mk3(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(float* p, f3 v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}
__device__ __forceinline__ q4 ld4(const float* p) { return q4{p[0], p[1], p[2], p[3]}; }
__device__ __forceinline__ void st4(float* p, q4 q) {
  p[0] = q.w;
  p[1] = q.x;
  p[2] = q.y;
  p[3] = q.z;
}
__device__ __forceinline__ q4 qident() { return q4{1.f, 0.f, 0.f, 0.f}; }

// brax/math.py:25-40
__device__ __forceinline__ f3 rotate(f3 v, q4 q) {
  f3 u = mk3(q.x, q.y, q.z);
  float s = q.w;
  f3 r = (2.f * dot3(u, v)) * u + (s * s - dot3(u, u)) * v;
  return r + (2.f * s) * cross3(u, v);
}

// brax/math.py:86-101
__device__ __forceinline__ q4 qmul(q4 u, q4 v) {
  return q4{u.w * v.w - u.x * v.x - u.y * v.y - u.z * v.z,
            u.w * v.x + u.x * v.w + u.y * v.z - u.z * v.y,
            u.w * v.y - u.x * v.z + u.y * v.w + u.z * v.x,
            u.w * v.z + u.x * v.y - u.y * v.x + u.z * v.w};
}

// One out-of-line copy of the precise sine/cosine (keeps the kernel's code
// footprint small: every call site would otherwise carry its own expansion).
static __device__ __noinline__ void sincos_ool(float x, float* s, float* c) { sincosf(x, s, c); }
static __device__ __noinline__ float pow_ool(float x, float y) { return powf(x, y); }
// x^y with the exact shortcuts y == 1 and y == 2 (powf is correctly rounded
// there, and so are x and x*x, so the results are identical).
__device__ __forceinline__ float pow_fast(float x, float y) {
  return y == 2.f ? x * x : (y == 1.f ? x : pow_ool(x, y));
}

// brax/math.py:134-148
__device__ __forceinline__ q4 quat_rot_axis(f3 axis, float angle) {
  float s, c;
  sincos_ool(angle * 0.5f, &s, &c);
  return q4{c, axis.x * s, axis.y * s, axis.z * s};
}

// brax/math.py:308-345: normalize with safe_norm (allclose(x, 0) -> norm 0)
__device__ __forceinline__ q4 qnormalize(q4 q) {
  bool z = fabsf(q.w) <= 1e-8f && fabsf(q.x) <= 1e-8f && fabsf(q.y) <= 1e-8f && fabsf(q.z) <= 1e-8f;
  float add = z ? 1.f : 0.f;
  float n = sqrtf((q.w + add) * (q.w + add) + (q.x + add) * (q.x + add) + (q.y + add) * (q.y + add) +
                  (q.z + add) * (q.z + add)) *
            (1.f - add);
  float d = n + (n == 0.f ? 1e-6f : 0.f);
  return q4{q.w / d, q.x / d, q.y / d, q.z / d};
}
__device__ __forceinline__ f3 normalize3(f3 v) {
  bool z = fabsf(v.x) <= 1e-8f && fabsf(v.y) <= 1e-8f && fabsf(v.z) <= 1e-8f;
  float add = z ? 1.f : 0.f;
  float n = sqrtf((v.x + add) * (v.x + add) + (v.y + add) * (v.y + add) + (v.z + add) * (v.z + add)) *
            (1.f - add);
  float d = n + (n == 0.f ? 1e-6f : 0.f);
  return mk3(v.x / d, v.y / d, v.z / d);
}

// brax/math.py:151-165; R row-major
__device__ __forceinline__ void quat_to_3x3(q4 q, float* R) {
  float d = q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z;
  float s = 2.f / d;
  float xs = q.x * s, ys = q.y * s, zs = q.z * s;
  float wx = q.w * xs, wy = q.w * ys, wz = q.w * zs;
  float xx = q.x * xs, xy = q.x * ys, xz = q.x * zs;
  float yy = q.y * ys, yz = q.y * zs, zz = q.z * zs;
  R[0] = 1.f - (yy + zz);
  R[1] = xy - wz;
  R[2] = xz + wy;
  R[3] = xy + wz;
  R[4] = 1.f - (xx + zz);
  R[5] = yz - wx;
  R[6] = xz - wy;
  R[7] = yz + wx;
  R[8] = 1.f - (xx + yy);
}

// Transform.do(Transform), brax/base.py:566-570
__device__ __forceinline__ void tf_do(f3 ap, q4 ar, f3 bp, q4 br, f3& op, q4& orr) {
  op = ap + rotate(bp, ar);
  orr = qmul(ar, br);
}

// Motion.cross(Motion), brax/base.py:604-608: returns (ang, vel)
__device__ __forceinline__ void motion_cross(f3 sa, f3 sv, f3 oa, f3 ov, f3& ra, f3& rv) {
  ra = cross3(sa, oa);
  rv = cross3(sa, ov) + cross3(sv, oa);
}

// Motion x Force, brax/base.py:611-614: returns (ang, vel)
__device__ __forceinline__ void force_cross(f3 sa, f3 sv, f3 fa, f3 fv, f3& ra, f3& rv) {
  ra = cross3(sa, fa) + cross3(sv, fv);
  rv = cross3(sa, fv);
}

// Inertia.mul, brax/base.py:297-302; I row-major 3x3, p = transform.pos
__device__ __forceinline__ void inertia_mul(const float* I, f3 p, float m, f3 ma, f3 mv, f3& fa, f3& fv) {
  f3 ia = mk3(I[0] * ma.x + I[1] * ma.y + I[2] * ma.z, I[3] * ma.x + I[4] * ma.y + I[5] * ma.z,
              I[6] * ma.x + I[7] * ma.y + I[8] * ma.z);
  fa = ia + cross3(p, mv);
  fv = m * mv - cross3(p, ma);
}

// mujoco.mjx math.normalize_with_norm
__device__ __forceinline__ f3 normalize_with_norm(f3 v, float& n) {
  n = sqrtf(dot3(v, v));
  float d = n + (n == 0.f ? 1e-6f : 0.f);
  return mk3(v.x / d, v.y / d, v.z / d);
}

// brax/math.py:247-254 / mjx math.orthogonals + make_frame: rows n, b, c
__device__ __forceinline__ void make_frame(f3 a, float* F) {
  a = normalize3(a);
  f3 b = (-0.5f < a.y && a.y < 0.5f) ? mk3(0.f, 1.f, 0.f) : mk3(0.f, 0.f, 1.f);
  b = b - a * dot3(a, b);
  bool any = (a.x != 0.f) || (a.y != 0.f) || (a.z != 0.f);
  b = normalize3(b) * (any ? 1.f : 0.f);
  f3 c = cross3(a, b);
  st3(F, a);
  st3(F + 3, b);
  st3(F + 6, c);
}
