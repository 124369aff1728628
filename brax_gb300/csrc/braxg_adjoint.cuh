// Reverse pass of one pipeline step (brax/generalized/pipeline.py:64-94) with
// the exact mass-matrix inverse: given the adjoints of the step's outputs
// (q', qd') it accumulates the adjoints of its inputs (q, qd, act).  Each
// reverse stage mirrors the forward stage it differentiates; discrete choices
// (contact mask, clip ranges, line-search step sizes, projection active sets,
// iteration counts) are held fixed, as jax.grad does.  Parent-link
// accumulations go through per-link slots and child-list gathers, so lanes
// never write the same word.
#pragma once
#include "braxg_adjoint_math.cuh"
#include "braxg_step.cuh"
#include "braxg_adjoint_contact.cuh"

namespace braxg {

struct AdjLayout {
  int q0, qd0, qb, qdb, qbo, qdbo, actb, qddb, qfsb, qfcb, vb, u, tb;
  int Minvb, Mb, Minvbc, Jb, diagb, arefb, bb, xb, Ab, tape;
  int xpb, xrb, cib, cpb, cdb, rcb, cdofb, cdofdb;
  int tmp, tmp_words;
  int ns;  // Newton-Schulz mode: the inverse reverse's working set (ns_rev_smem_words), else -1
  int total;
};

// `ns_words`: words of the Newton-Schulz reverse's shared working set (0
// in exact-inverse mode).
__host__ __device__ inline AdjLayout make_adj_layout(int nl, int nq, int nv, int nu, int ncon, int nlim,
                                                     int pg_iters, int ns_words = 0) {
  AdjLayout A;
  const int m = 4 * ncon + nlim;
  // rows of the explicit solve's A cotangent; the row cotangents cover all m
  // rows (the implicit solve's rows beyond kMaxExplicitRows too)
  const int na = m < kMaxExplicitRows ? m : kMaxExplicitRows;
  const int ldm = nv | 1, ldj = nv | 1, la = (na | 1);
  int o = 0;
  auto take = [&](int words) {
    int at = o;
    o += al4(words);
    return at;
  };
  A.q0 = take(nq);
  A.qd0 = take(nv);
  A.qb = take(nq);
  A.qdb = take(nv);
  A.qbo = take(nq);
  A.qdbo = take(nv);
  A.actb = take(nu);
  A.qddb = take(nv);
  A.qfsb = take(nv);
  A.qfcb = take(nv);
  A.vb = take(nv);
  A.u = take(nv);
  A.tb = take(nv);
  A.Minvb = take(nv * ldm);
  A.Mb = take(nv * ldm);
  A.Minvbc = take(nv * ldm);  // Newton-Schulz mode: the carried inverse's cotangent, frame to frame
  A.Jb = take(m * ldj);
  A.diagb = take(m);
  A.arefb = take(m);
  A.bb = take(m);
  A.xb = take(m);
  A.Ab = take(na * la);
  A.tape = take(tape_words(m, pg_iters));
  A.xpb = take(3 * nl);
  A.xrb = take(4 * nl);
  A.cib = take(9 * nl);
  A.cpb = take(3 * nl);
  A.cdb = take(6 * nl);
  A.rcb = take(6 * nl);
  A.cdofb = take(6 * nv);
  A.cdofdb = take(6 * nv);
  // scratch shared by the reverse stages (each uses it only while it runs)
  int t = 25 * nl + 12 * nv;                               // CRBA: crb, F, F_bar, crb_bar
  t = t > 28 * nl ? t : 28 * nl;                           // FK: tree recompute + gathers
  t = t > 24 * nl ? t : 24 * nl;                           // RNE: cdd, cfrc and their adjoints
  t = t > 20 * nl ? t : 20 * nl;                           // com: per-link gathers
  t = t > nv * ldm ? t : nv * ldm;                         // inverse: Minv_bar Minv
  const int kA = (kMaxExplicitRows + 3) & ~3;
  const int lae = explicit_lda(na);
  t = t > na * lae + na * ldm + 4 * kA ? t : na * lae + na * ldm + 4 * kA;  // constraint: A, W, vectors
  if (m > kMaxExplicitRows) {  // implicit solve: Ab J, Ab^T J, 4 row vectors, 6 dof vectors
    const int ti = 2 * m * ldm + 4 * al4(m) + 6 * al4(nv);
    t = t > ti ? t : ti;
  }
  t += 16;
  A.tmp_words = al4(t);
  A.tmp = take(A.tmp_words);
  A.ns = ns_words > 0 ? take(ns_words) : -1;
  A.total = al4(o);
  return A;
}

struct AWs {
  float* b;
  const AdjLayout* A;
  __device__ __forceinline__ float* at(int off) const { return b + off; }
};

// ---------------------------------------------------------------------------
// integrator reverse (integrator.py:46-84).  Workspace q/qd hold (q', qd'),
// a.q0 the step's input q.  Produces qb, qdb (partial) and qddb.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_integrate(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const AdjLayout& A = *a.A;
  const float h = md.dt;
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  float* qb = a.at(A.qb);
  float* qdb = a.at(A.qdb);
  const float* qbo = a.at(A.qbo);
  const float* qdbo = a.at(A.qdbo);
  float* qdnb = a.at(A.vb);  // adjoint of qd' (temporary)
  const float* q0 = a.at(A.q0);
  const float* qdn = w.at(w.L->qd);
  for (int l = tm.lane; l < md.nl; l += T) {
    int typ = ltype[l], qa = qadr[l], da = dadr[l];
    if (typ == 0) {
      for (int k = 0; k < 3; ++k) {
        qb[qa + k] += qbo[qa + k];
        qdnb[da + k] = qdbo[da + k] + h * qbo[qa + k];
      }
      q4 rot0 = ld4(q0 + qa + 3);
      f3 ang = ld3(qdn + da + 3);
      float n = sqrtf(dot3(ang, ang));
      float an = n + 1e-8f;
      f3 axis = mk3(ang.x / an, ang.y / an, ang.z / an);
      q4 qrot = quat_rot_axis(axis, h * an);
      q4 prod = qmul(rot0, qrot);
      q4 prodb = normalize4_vjp(prod, ld4(qbo + qa + 3));
      q4 rotb, qrotb;
      qmul_vjp(rot0, qrot, prodb, rotb, qrotb);
      add4(qb + qa + 3, rotb);
      float sn, cs;
      sincos_ool(h * an * 0.5f, &sn, &cs);
      float f = sn / an;
      float dfdan = (cs * h * 0.5f * an - sn) / (an * an);
      float inv_n = n > 0.f ? 1.f / n : 0.f;
      f3 unit = ang * inv_n;
      f3 qvb = mk3(qrotb.x, qrotb.y, qrotb.z);
      f3 angb = unit * (qrotb.w * (-sn * 0.5f * h)) + qvb * f + unit * (dot3(ang, qvb) * dfdan);
      for (int k = 0; k < 3; ++k) qdnb[da + 3 + k] = qdbo[da + 3 + k] + (&angb.x)[k];
    } else {
      for (int k = 0; k < typ; ++k) {
        qb[qa + k] += qbo[qa + k];
        qdnb[da + k] = qdbo[da + k] + h * qbo[qa + k];
      }
    }
  }
  tm.sync();
  float* qddb = a.at(A.qddb);
  for (int d = tm.lane; d < md.nv; d += T) {
    qdb[d] += qdnb[d];
    qddb[d] = h * qdnb[d];
  }
  tm.sync();
}

// qdd = Minv (qfs + qfc)
template <int T>
__device__ __noinline__ void rev_qdd(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nv = md.nv, ld = L.ldm;
  const float* Minv = w.at(L.Minv);
  const float* qfs = w.at(L.qfs);
  const float* qfc = w.at(L.qfc);
  const float* qddb = a.at(A.qddb);
  float* Minvb = a.at(A.Minvb);
  for (int j = tm.lane; j < nv; j += T) {
    const float vj = qfs[j] + qfc[j];
    float s = 0.f;
    for (int i = 0; i < nv; ++i) {
      Minvb[i * ld + j] = qddb[i] * vj;  // first write of Minv_bar in the step
      s = fmaf(Minv[i * ld + j], qddb[i], s);
    }
    a.at(A.qfsb)[j] = s;
    a.at(A.qfcb)[j] = s;
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// constraint.force reverse on the implicit path (more than kMaxExplicitRows
// active rows), where the forward applied A = J Minv J^T + diag without
// forming it.  The unrolled iterations are reversed with the same implicit
// matvecs; the cotangent of A, sum_k (r_k g_k^T + rb_k y_k^T), is never
// formed: its products P = Ab J and Q = Ab^T J (nrow x nv) are accumulated
// from J^T of the iteration vectors, and then
//   Jb += (P + Q) Minv,   Minvb += J^T P,   diagb = diag(Ab),
// the same contractions the explicit path takes through Ab.  b = J (Minv qfs)
// - aref and qfc = J^T x* are reversed as there.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_constraint_implicit(const int* mw, Ws w, AWs a, int iters, int nrow, bool sym) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nv = md.nv, ldj = L.ldj, ld = L.ldm, m = md.m;
  const int kT = tape_stride(nrow);
  const float* tape = a.at(A.tape);
  const float* Minv = w.at(L.Minv);
  const float* rdiag = w.at(L.rdiag);
  const float* qfs = w.at(L.qfs);
  const float* qfcb = a.at(A.qfcb);
  float* Jb = a.at(A.Jb);
  float* bb = a.at(A.bb);
  float* xbar = a.at(A.xb);
  float* diagb = a.at(A.diagb);
  float* Pm = a.at(A.tmp);          // Ab J      [nrow, ld]
  float* Qm = Pm + m * ld;          // Ab^T J    [nrow, ld]
  float* ybar = Qm + m * ld;
  float* vv = ybar + al4(m);
  float* gb = vv + al4(m);
  float* rb = gb + al4(m);
  float* jg = rb + al4(m);          // J^T gb
  float* jr = jg + al4(nv);         // J^T rb
  float* jy = jr + al4(nv);         // J^T y
  float* jry = jy + al4(nv);        // J^T ry
  float* t2 = jry + al4(nv);        // Minv J^T v
  // A v for the implicit A: out = J (Minv (J^T v)) + diag v, keeping J^T v in
  // jtv; `trans`: A^T v (Minv^T in the middle; the same unless the carried
  // Newton-Schulz inverse is not symmetric)
  auto matvec = [&](const float* v, float* out, float* jtv, bool trans = false) {
    for (int d = tm.lane; d < nv; d += T) {
      float s = 0.f;
      for (int r = 0; r < nrow; ++r) s = fmaf(w.jrow(r)[d], v[r], s);
      jtv[d] = s;
    }
    tm.sync();
    const int si = trans ? 1 : ld, sk = trans ? ld : 1;
    for (int d = tm.lane; d < nv; d += T) {
      float s = 0.f;
      for (int k = 0; k < nv; ++k) s = fmaf(Minv[d * si + k * sk], jtv[k], s);
      t2[d] = s;
    }
    tm.sync();
    for (int r = tm.lane; r < nrow; r += T) {
      const float* jrow = w.jrow(r);
      float s = 0.f;
      for (int k = 0; k < nv; ++k) s = fmaf(jrow[k], t2[k], s);
      out[r] = s + rdiag[r] * v[r];
    }
    tm.sync();
  };
  auto jt = [&](const float* v, float* out) {  // out = J^T v
    for (int d = tm.lane; d < nv; d += T) {
      float s = 0.f;
      for (int r = 0; r < nrow; ++r) s = fmaf(w.jrow(r)[d], v[r], s);
      out[d] = s;
    }
  };
  // qfc = J^T x*: Jb = x* qfcb^T, xbar = J qfcb
  const float* xs = tape + 4;
  for (int e = tm.lane; e < nrow * nv; e += T) {
    const int i = e / nv, d = e - i * nv;
    Jb[i * ldj + d] = xs[i] * qfcb[d];
    Pm[i * ld + d] = 0.f;
    Qm[i * ld + d] = 0.f;
  }
  for (int i = tm.lane; i < nrow; i += T) {
    const float* jrow = w.jrow(i);
    float s = 0.f;
    for (int d = 0; d < nv; ++d) s = fmaf(jrow[d], qfcb[d], s);
    xbar[i] = s;
    bb[i] = 0.f;
    diagb[i] = 0.f;
    ybar[i] = 0.f;
  }
  tm.sync();
  for (int k = iters - 1; k >= 0; --k) {
    const float* rec = tape + tape_head_words(nrow) + k * tape_iter_words(nrow);
    const float step = rec[0], beta = rec[1];
    const float* y = rec + 4;
    const float* ry = rec + 4 + kT;
    const float* zpos = rec + 4 + 2 * kT;
    for (int i = tm.lane; i < nrow; i += T) {
      const float nxb = xbar[i] + (1.f + beta) * ybar[i];
      const float zb = nxb * zpos[i];
      vv[i] = zb;
      gb[i] = -step * zb;
      xbar[i] = -beta * ybar[i];
    }
    tm.sync();
    matvec(gb, rb, jg);  // rb = A gb (g = A^T r, r = A y + b), jg = J^T gb
    jt(y, jy);
    jt(ry, jry);
    for (int i = tm.lane; i < nrow; i += T) {
      bb[i] += rb[i];
      diagb[i] += ry[i] * gb[i] + rb[i] * y[i];
    }
    tm.sync();
    matvec(rb, ybar, jr, !sym);  // A^T rb, jr = J^T rb
    for (int i = tm.lane; i < nrow; i += T) ybar[i] += vv[i];  // ybar = zb + A^T rb
    // Ab += ry gb^T + rb y^T:  P += ry (J^T gb)^T + rb (J^T y)^T,  Q += gb (J^T ry)^T + y (J^T rb)^T
    for (int e = tm.lane; e < nrow * nv; e += T) {
      const int i = e / nv, d = e - i * nv;
      Pm[i * ld + d] += ry[i] * jg[d] + rb[i] * jy[d];
      Qm[i * ld + d] += gb[i] * jry[d] + y[i] * jr[d];
    }
    tm.sync();
  }
  // A = (J Minv) J^T + diag: Jb += P Minv^T + Q Minv, (P + Q) Minv when Minv is symmetric
  for (int e = tm.lane; e < nrow * nv; e += T) {
    const int i = e / nv, d = e - i * nv;
    float s = 0.f;
    if (sym) {
      for (int k = 0; k < nv; ++k) s = fmaf(Pm[i * ld + k] + Qm[i * ld + k], Minv[k * ld + d], s);
    } else {
      for (int k = 0; k < nv; ++k) s = fmaf(Pm[i * ld + k], Minv[d * ld + k], fmaf(Qm[i * ld + k], Minv[k * ld + d], s));
    }
    Jb[i * ldj + d] += s;
  }
  // Minvb += J^T Ab J = J^T P
  float* Minvb = a.at(A.Minvb);
  for (int e = tm.lane; e < nv * nv; e += T) {
    const int i2 = e / nv, j = e - i2 * nv;
    float s = 0.f;
    for (int r = 0; r < nrow; ++r) s = fmaf(w.jrow(r)[i2], Pm[r * ld + j], s);
    Minvb[i2 * ld + j] += s;
  }
  tm.sync();
  // b = J (Minv qfs) - aref
  float* u = a.at(A.u);
  float* tb = a.at(A.tb);
  for (int d = tm.lane; d < nv; d += T) {
    float s = 0.f, t = 0.f;
    for (int k = 0; k < nv; ++k) s = fmaf(Minv[d * ld + k], qfs[k], s);
    for (int i = 0; i < nrow; ++i) t = fmaf(w.jrow(i)[d], bb[i], t);
    u[d] = s;
    tb[d] = t;
  }
  tm.sync();
  float* arefb = a.at(A.arefb);
  float* qfsb = a.at(A.qfsb);
  for (int d = tm.lane; d < nv; d += T) {
    for (int i = 0; i < nrow; ++i) Jb[i * ldj + d] += bb[i] * u[d];
    float s = 0.f;
    for (int k = 0; k < nv; ++k) {
      Minvb[k * ld + d] += tb[k] * qfs[d];
      s = fmaf(Minv[k * ld + d], tb[k], s);
    }
    qfsb[d] += s;
  }
  for (int i = tm.lane; i < nrow; i += T) arefb[i] = -bb[i];
  tm.sync();
}

// ---------------------------------------------------------------------------
// constraint.force reverse: qfc = J^T x*, the unrolled projected gradient
// (jaxopt ProximalGradient, constraint.py:229-238), A = (J Minv) J^T + diag,
// b = (J Minv) qfs - aref.  Produces Jb, diagb, arefb for the active rows and
// adds to Minvb, qfsb.  Returns false when the forward solve ran the implicit
// path (more than kMaxExplicitRows active rows), which has no tape.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ bool rev_constraint(const int* mw, Ws w, AWs a, bool sym = true) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nv = md.nv, ldj = L.ldj, ld = L.ldm;
  const float* tape = a.at(A.tape);
  const int iters = (int)tape[0];
  const int nrow = (int)tape[1];
  if (iters < 0 || nrow > md.m) return false;
  if (nrow == 0) return true;
  if (nrow > kMaxExplicitRows) {
    rev_constraint_implicit<T>(mw, w, a, iters, nrow, sym);
    return true;
  }
  const int lab = nrow | 1;  // Ab rows
  const int la = explicit_lda(nrow), n4 = al4(nrow) / 4;  // Am rows (16-byte matvecs, as the forward)
  constexpr int kA = (kMaxExplicitRows + 3) & ~3;
  const int kT = tape_stride(nrow);  // the tape's row vectors
  const float* J = w.at(L.J);
  const float* Minv = w.at(L.Minv);
  const float* rdiag = w.at(L.rdiag);
  const float* qfs = w.at(L.qfs);
  const float* qfcb = a.at(A.qfcb);
  float* Jb = a.at(A.Jb);
  float* Ab = a.at(A.Ab);
  float* bb = a.at(A.bb);
  float* xbar = a.at(A.xb);
  float* Am = a.at(A.tmp);
  float* W = Am + nrow * la;
  float* ybar = W + al4(nrow * ld);  // 16-byte aligned: gb and rb are float4 matvec inputs
  float* vv = ybar + kA;   // scratch vectors of length nrow
  float* gb = vv + kA;
  float* rb = gb + kA;
  // W = J Minv (lanes over its entries), then A = W J^T + diag as the forward
  // formed it: the lower triangle mirrored, zero padding columns
  for (int e = tm.lane; e < nrow * nv; e += T) {
    const int i = e / nv, k = e - i * nv;
    float s0 = 0.f, s1 = 0.f;
    int d = 0;
    for (; d + 1 < nv; d += 2) {
      s0 = fmaf(J[i * ldj + d], Minv[d * ld + k], s0);
      s1 = fmaf(J[i * ldj + d + 1], Minv[(d + 1) * ld + k], s1);
    }
    if (d < nv) s0 = fmaf(J[i * ldj + d], Minv[d * ld + k], s0);
    W[i * ld + k] = s0 + s1;
  }
  for (int e = tm.lane; e < 4 * kA; e += T) ybar[e] = 0.f;  // ybar, vv, gb, rb with their padding
  for (int e = tm.lane; e < nrow * lab; e += T) Ab[e] = 0.f;
  tm.sync();
  if (!sym) {  // every entry, as the forward formed A with a non-symmetric Newton-Schulz inverse
    for (int e = tm.lane; e < nrow * nrow; e += T) {
      const int i = e / nrow, c = e - i * nrow;
      float s0 = 0.f, s1 = 0.f;
      int k = 0;
      for (; k + 1 < nv; k += 2) {
        s0 = fmaf(W[i * ld + k], J[c * ldj + k], s0);
        s1 = fmaf(W[i * ld + k + 1], J[c * ldj + k + 1], s1);
      }
      if (k < nv) s0 = fmaf(W[i * ld + k], J[c * ldj + k], s0);
      Am[i * la + c] = (s0 + s1) + (i == c ? rdiag[i] : 0.f);
    }
    for (int e = tm.lane; e < nrow * (4 * n4 - nrow); e += T) {
      const int r = e / (4 * n4 - nrow);
      Am[r * la + nrow + (e - r * (4 * n4 - nrow))] = 0.f;
    }
  } else {
    int i = 0, c = tm.lane;
    while (c > i) {
      c -= i + 1;
      ++i;
    }
    for (; i < nrow;) {
      float s0 = 0.f, s1 = 0.f;
      int k = 0;
      for (; k + 1 < nv; k += 2) {
        s0 = fmaf(W[i * ld + k], J[c * ldj + k], s0);
        s1 = fmaf(W[i * ld + k + 1], J[c * ldj + k + 1], s1);
      }
      if (k < nv) s0 = fmaf(W[i * ld + k], J[c * ldj + k], s0);
      const float v = (s0 + s1) + (i == c ? rdiag[i] : 0.f);
      Am[i * la + c] = v;
      Am[c * la + i] = v;
      c += T;
      while (c > i) {
        c -= i + 1;
        ++i;
      }
    }
    for (int e = tm.lane; e < nrow * (4 * n4 - nrow); e += T) {
      const int r = e / (4 * n4 - nrow);
      Am[r * la + nrow + (e - r * (4 * n4 - nrow))] = 0.f;
    }
  }
  // qfc = J^T x*: Jb = x* qfcb^T, xbar = J qfcb
  const float* xs = tape + 4;
  for (int e = tm.lane; e < nrow * nv; e += T) {
    const int i = e / nv, d = e - i * nv;
    Jb[i * ldj + d] = xs[i] * qfcb[d];
  }
  for (int i = tm.lane; i < nrow; i += T) {
    float s = 0.f;
    for (int d = 0; d < nv; ++d) s = fmaf(J[i * ldj + d], qfcb[d], s);
    xbar[i] = s;
    bb[i] = 0.f;
  }
  tm.sync();
  // A v for v with zero padding (A is symmetric: also A^T v)
  auto matvec = [&](const float* v, int i) {
    const float4* a4 = reinterpret_cast<const float4*>(Am + i * la);
    const float4* v4 = reinterpret_cast<const float4*>(v);
    float s0 = 0.f, s1 = 0.f;
    for (int c = 0; c < n4; ++c) {
      const float4 x = a4[c], u = v4[c];
      s0 = fmaf(x.x, u.x, s0);
      s1 = fmaf(x.y, u.y, s1);
      s0 = fmaf(x.z, u.z, s0);
      s1 = fmaf(x.w, u.w, s1);
    }
    return s0 + s1;
  };
  for (int k = iters - 1; k >= 0; --k) {
    const float* rec = tape + tape_head_words(nrow) + k * tape_iter_words(nrow);
    const float step = rec[0], beta = rec[1];
    const float* y = rec + 4;
    const float* ry = rec + 4 + kT;
    const float* zpos = rec + 4 + 2 * kT;
    for (int i = tm.lane; i < nrow; i += T) {
      float nxb = xbar[i] + (1.f + beta) * ybar[i];
      float zb = nxb * zpos[i];
      vv[i] = zb;
      gb[i] = -step * zb;
      xbar[i] = -beta * ybar[i];
    }
    tm.sync();
    for (int i = tm.lane; i < nrow; i += T) {  // rb = A gb
      const float s = matvec(gb, i);
      rb[i] = s;
      bb[i] += s;
    }
    tm.sync();
    for (int c = tm.lane; c < nrow; c += T)  // Ab += ry gb^T + rb y^T
      for (int i = 0; i < nrow; ++i) Ab[i * lab + c] += ry[i] * gb[c] + rb[i] * y[c];
    if (sym) {
      for (int i = tm.lane; i < nrow; i += T) ybar[i] = vv[i] + matvec(rb, i);  // ybar = zb + A^T rb
    } else {
      for (int i = tm.lane; i < nrow; i += T) {  // ybar = zb + A^T rb by columns
        float s0 = 0.f, s1 = 0.f;
        int r = 0;
        for (; r + 1 < nrow; r += 2) {
          s0 = fmaf(Am[r * la + i], rb[r], s0);
          s1 = fmaf(Am[(r + 1) * la + i], rb[r + 1], s1);
        }
        if (r < nrow) s0 = fmaf(Am[r * la + i], rb[r], s0);
        ybar[i] = vv[i] + (s0 + s1);
      }
    }
    tm.sync();
  }
  // A = (J Minv) J^T + diag: Jb += Ab (J Minv^T) + Ab^T (J Minv), i.e.
  // (Ab + Ab^T) W when Minv is symmetric; lanes over Jb's entries
  float* diagb = a.at(A.diagb);
  for (int e = tm.lane; e < nrow * nv; e += T) {
    const int i = e / nv, d = e - i * nv;
    float s = 0.f;
    if (sym) {
      for (int c = 0; c < nrow; ++c) s = fmaf(Ab[i * lab + c] + Ab[c * lab + i], W[c * ld + d], s);
    } else {
      for (int c = 0; c < nrow; ++c) s = fmaf(Ab[c * lab + i], W[c * ld + d], s);
    }
    Jb[i * ldj + d] += s;
  }
  for (int i = tm.lane; i < nrow; i += T) diagb[i] = Ab[i * lab + i];
  tm.sync();
  if (!sym) {  // W <- J Minv^T, then Jb += Ab W
    for (int e = tm.lane; e < nrow * nv; e += T) {
      const int i = e / nv, k = e - i * nv;
      float s = 0.f;
      for (int d = 0; d < nv; ++d) s = fmaf(J[i * ldj + d], Minv[k * ld + d], s);
      W[i * ld + k] = s;
    }
    tm.sync();
    for (int e = tm.lane; e < nrow * nv; e += T) {
      const int i = e / nv, d = e - i * nv;
      float s = 0.f;
      for (int c = 0; c < nrow; ++c) s = fmaf(Ab[i * lab + c], W[c * ld + d], s);
      Jb[i * ldj + d] += s;
    }
    tm.sync();
  }
  // Minvb += J^T Ab J via Z = Ab J (reuses W's rows as Z)
  float* Z = W;
  for (int e = tm.lane; e < nrow * nv; e += T) {
    const int i = e / nv, d = e - i * nv;
    float s = 0.f;
    for (int c = 0; c < nrow; ++c) s = fmaf(Ab[i * lab + c], J[c * ldj + d], s);
    Z[i * ld + d] = s;
  }
  tm.sync();
  float* Minvb = a.at(A.Minvb);
  for (int e = tm.lane; e < nv * nv; e += T) {
    const int i2 = e / nv, j = e - i2 * nv;
    float s = 0.f;
    for (int r = 0; r < nrow; ++r) s = fmaf(J[r * ldj + i2], Z[r * ld + j], s);
    Minvb[i2 * ld + j] += s;
  }
  tm.sync();
  // b = J (Minv qfs) - aref
  float* u = a.at(A.u);
  float* tb = a.at(A.tb);
  for (int d = tm.lane; d < nv; d += T) {
    float s = 0.f, t2 = 0.f;
    for (int k = 0; k < nv; ++k) s = fmaf(Minv[d * ld + k], qfs[k], s);
    for (int i = 0; i < nrow; ++i) t2 = fmaf(J[i * ldj + d], bb[i], t2);
    u[d] = s;
    tb[d] = t2;
  }
  tm.sync();
  float* arefb = a.at(A.arefb);
  float* qfsb = a.at(A.qfsb);
  for (int d = tm.lane; d < nv; d += T) {
    for (int i = 0; i < nrow; ++i) Jb[i * ldj + d] += bb[i] * u[d];
    float s = 0.f;
    for (int k = 0; k < nv; ++k) {
      Minvb[k * ld + d] += tb[k] * qfs[d];
      s = fmaf(Minv[k * ld + d], tb[k], s);
    }
    qfsb[d] += s;
  }
  for (int i = tm.lane; i < nrow; i += T) arefb[i] = -bb[i];
  tm.sync();
  return true;
}

// ---------------------------------------------------------------------------
// qf_smooth reverse: passive, actuator (actuator.py:23-57), RNE
// (dynamics.py:137-184) with bias_bar = -qfs_bar.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_smooth(const int* mw, Ws w, AWs a, bool has_act) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nl = md.nl, nv = md.nv;
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const int* dlink = md.I(BXM_O_DOF_LINK);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* cstart = md.I(BXM_O_CHILD_START);
  const int* cidx = md.I(BXM_O_CHILD_IDX);
  const float* q = a.at(A.q0);
  const float* qd = a.at(A.qd0);
  const float* qfsb = a.at(A.qfsb);
  float* qb = a.at(A.qb);
  float* qdb = a.at(A.qdb);
  // passive (dynamics.py:187-196)
  for (int d = tm.lane; d < nv; d += T) {
    int l = dlink[d];
    if (ltype[l] != 0) qb[qadr[l] + (d - dadr[l])] += -md.F(BXM_O_D_STIFF)[d] * qfsb[d];
    qdb[d] += -md.F(BXM_O_D_DAMP)[d] * qfsb[d];
  }
  tm.sync();
  // fluid forces (dynamics.py:198-211, fluid.py:53-82): each link's drag
  // recomputed as the forward forms it (the inertia-box drag of its com
  // point's velocity in the inertia frame, rotated back to world), then
  // qf_smooth += sum_k J_k(x_i.pos) . f_k reversed into cdof, the drag's
  // inputs (cd, the com offset from the tree's com), and x
  if (md.fluid) {
    const float* xp = w.at(L.xp);
    const float* xr = w.at(L.xr);
    const float* rc = w.at(L.rc);
    const float* cd = w.at(L.cd);
    const float* cdof = w.at(L.cdof);
    const float* lip = md.F(BXM_O_LI_POS);
    const float* lir = md.F(BXM_O_LI_ROT);
    const float* box = md.F(BXM_O_LI_BOX);
    float* cdofb = a.at(A.cdofb);
    float* cdb = a.at(A.cdb);
    float* rcb = a.at(A.rcb);
    float* xpb = a.at(A.xpb);
    float* xrb = a.at(A.xrb);
    float* fw = a.at(A.tmp);  // per link: world force ang, vel, then the com offset
    // the drag of link l from its com velocity in the inertia frame (wa, wv),
    // and d f / d w per component (the drag is componentwise)
    auto drag = [&](int l, f3 wa, f3 wv, f3& fa, f3& fv, f3& dfa, f3& dfv) {
      const f3 b = ld3(box + 3 * l);
      const float diam = (b.x + b.y + b.z) / 3.f;
      const float ang_scale = -kPi * (diam * diam * diam) * md.visc;
      const float vel_scale = -3.f * kPi * diam * md.visc;
      const float dv = -0.5f * md.dens, da = -1.f * md.dens;
      const f3 ev = mk3(b.y * b.z, b.x * b.z, b.x * b.y);
      const float b4x = (b.x * b.x) * (b.x * b.x), b4y = (b.y * b.y) * (b.y * b.y), b4z = (b.z * b.z) * (b.z * b.z);
      const f3 ea = mk3(b.x * (b4y + b4z), b.y * (b4x + b4z), b.z * (b4x + b4y));
      fa = ang_scale * wa + mk3(da * ea.x * fabsf(wa.x) * wa.x / 64.f, da * ea.y * fabsf(wa.y) * wa.y / 64.f,
                                da * ea.z * fabsf(wa.z) * wa.z / 64.f);
      fv = vel_scale * wv + mk3(dv * ev.x * fabsf(wv.x) * wv.x, dv * ev.y * fabsf(wv.y) * wv.y,
                                dv * ev.z * fabsf(wv.z) * wv.z);
      dfa = mk3(ang_scale + da * ea.x * 2.f * fabsf(wa.x) / 64.f, ang_scale + da * ea.y * 2.f * fabsf(wa.y) / 64.f,
                ang_scale + da * ea.z * 2.f * fabsf(wa.z) / 64.f);
      dfv = mk3(vel_scale + dv * ev.x * 2.f * fabsf(wv.x), vel_scale + dv * ev.y * 2.f * fabsf(wv.y),
                vel_scale + dv * ev.z * 2.f * fabsf(wv.z));
    };
    for (int l = tm.lane; l < nl; l += T) {
      f3 ip;
      q4 ir;
      tf_do(ld3(xp + 3 * l), ld4(xr + 4 * l), ld3(lip + 3 * l), ld4(lir + 4 * l), ip, ir);
      const f3 off = ip - ld3(rc + 3 * l);
      const q4 rt = q4{ir.w, -ir.x, -ir.y, -ir.z};
      const f3 ca = ld3(cd + 6 * l), cv = ld3(cd + 6 * l + 3);
      f3 fa, fv, dfa, dfv;
      drag(l, rotate(ca, rt), rotate(cv - cross3(off, ca), rt), fa, fv, dfa, dfv);
      st3(fw + 9 * l, rotate(fa, ir));
      st3(fw + 9 * l + 3, rotate(fv, ir));
      st3(fw + 9 * l + 6, off);
    }
    tm.sync();
    // term (cv_d - off_k x ca_d) . Fv_k + ca_d . Fa_k for every link k that dof d moves
    for (int d = tm.lane; d < nv; d += T) {
      f3 sv = mk3(0.f, 0.f, 0.f), sa = sv;
      for (int k = 0; k < nl; ++k) {
        if (!((md.anc(k) >> d) & 1ull)) continue;
        const f3 Fa = ld3(fw + 9 * k), Fv = ld3(fw + 9 * k + 3), off = ld3(fw + 9 * k + 6);
        sv = sv + Fv;
        sa = sa + Fa + cross3(off, Fv);
      }
      add3(cdofb + 6 * d + 3, sv * qfsb[d]);
      add3(cdofb + 6 * d, sa * qfsb[d]);
    }
    for (int l = tm.lane; l < nl; l += T) {
      const f3 Fv = ld3(fw + 9 * l + 3), off = ld3(fw + 9 * l + 6);
      f3 Fvb = mk3(0.f, 0.f, 0.f), Fab = Fvb, offb = Fvb;
      for (int d = 0; d < nv; ++d) {
        if (!((md.anc(l) >> d) & 1ull)) continue;
        const float g = qfsb[d];
        const f3 ca = ld3(cdof + 6 * d), cv = ld3(cdof + 6 * d + 3);
        Fvb = Fvb + (cv - cross3(off, ca)) * g;
        Fab = Fab + ca * g;
        offb = offb + cross3(Fv, ca) * g;
      }
      f3 ip;
      q4 ir;
      const f3 xpl = ld3(xp + 3 * l);
      const q4 xrl = ld4(xr + 4 * l);
      tf_do(xpl, xrl, ld3(lip + 3 * l), ld4(lir + 4 * l), ip, ir);
      const q4 rt = q4{ir.w, -ir.x, -ir.y, -ir.z};
      const f3 ca = ld3(cd + 6 * l), cv = ld3(cd + 6 * l + 3);
      const f3 u = cv - cross3(off, ca);
      const f3 wa = rotate(ca, rt), wv = rotate(u, rt);
      f3 fa, fv, dfa, dfv;
      drag(l, wa, wv, fa, fv, dfa, dfv);
      // F = rotate(f, ir)
      f3 fab, fvb;
      q4 irb1, irb2;
      rotate_vjp(fa, ir, Fab, fab, irb1);
      rotate_vjp(fv, ir, Fvb, fvb, irb2);
      const f3 wab = mk3(fab.x * dfa.x, fab.y * dfa.y, fab.z * dfa.z);
      const f3 wvb = mk3(fvb.x * dfv.x, fvb.y * dfv.y, fvb.z * dfv.z);
      // wa = rotate(ca, rt), wv = rotate(cv - off x ca, rt)
      f3 cab, ub;
      q4 rtb1, rtb2;
      rotate_vjp(ca, rt, wab, cab, rtb1);
      rotate_vjp(u, rt, wvb, ub, rtb2);
      add3(cdb + 6 * l, cab + cross3(off, ub));
      add3(cdb + 6 * l + 3, ub);
      offb = offb + cross3(ub, ca);
      // rt = quat_inv(ir); off = ip - root_com
      const q4 rtb = qadd(rtb1, rtb2);
      const q4 irb = qadd(qadd(irb1, irb2), q4{rtb.w, -rtb.x, -rtb.y, -rtb.z});
      add3(rcb + 3 * l, -offb);
      // (ip, ir) = x_l . inertia transform
      f3 apb, bpb;
      q4 arb, brb;
      tf_do_vjp(xpl, xrl, ld3(lip + 3 * l), ld4(lir + 4 * l), offb, irb, apb, arb, bpb, brb);
      add3(xpb + 3 * l, apb);
      add4(xrb + 4 * l, arb);
    }
    tm.sync();
  }
  // actuators (lane 0 scatters: several actuators may share a dof)
  if (has_act && tm.lane == 0) {
    const float* act = w.at(L.act);
    const int* aqid = md.I(BXM_O_ACT_QID);
    const int* aqdid = md.I(BXM_O_ACT_QDID);
    float* actb = a.at(A.actb);
    for (int k = 0; k < md.nu; ++k) {
      const float* cr = md.F(BXM_O_ACT_CR) + 2 * k;
      const float* fr = md.F(BXM_O_ACT_FR) + 2 * k;
      float gear = md.F(BXM_O_ACT_GEAR)[k], gain = md.F(BXM_O_ACT_GAIN)[k];
      float bq = md.F(BXM_O_ACT_BQ)[k], bqd = md.F(BXM_O_ACT_BQD)[k];
      float u = fminf(fmaxf(act[k], cr[0]), cr[1]);
      float f0 = gain * u + gear * (q[aqid[k]] * bq + qd[aqdid[k]] * bqd);
      float fb = qfsb[aqdid[k]] * gear * clip_grad(f0, fr[0], fr[1]);
      actb[k] += fb * gain * clip_grad(act[k], cr[0], cr[1]);
      qb[aqid[k]] += fb * gear * bq;
      qdb[aqdid[k]] += fb * gear * bqd;
    }
  }
  tm.sync();
  // RNE: recompute cdd, g = I cd, cfrc
  float* cdd = a.at(A.tmp);
  float* cf = cdd + 6 * nl;
  float* cfb = cf + 6 * nl;
  float* cddb = cfb + 6 * nl;
  const float* cdofd = w.at(L.cdofd);
  const float* cdof = w.at(L.cdof);
  const float* ci = w.at(L.ci);
  const float* cp = w.at(L.cp);
  const float* cd = w.at(L.cd);
  const float* mass = md.F(BXM_O_LI_MASS);
  for (int lv = 0; lv < md.nlevel; ++lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx], p = parent[l];
      f3 ca = p >= 0 ? ld3(cdd + 6 * p) : mk3(0.f, 0.f, 0.f);
      f3 cv = p >= 0 ? ld3(cdd + 6 * p + 3) : -md.g;
      int nd = ltype[l] == 0 ? 6 : ltype[l];
      for (int k = 0; k < nd; ++k) {
        int d = dadr[l] + k;
        ca = ca + ld3(cdofd + 6 * d) * qd[d];
        cv = cv + ld3(cdofd + 6 * d + 3) * qd[d];
      }
      st3(cdd + 6 * l, ca);
      st3(cdd + 6 * l + 3, cv);
    }
    tm.sync();
  }
  for (int l = tm.lane; l < nl; l += T) {
    f3 fa, fv, ga, gv, xa, xv;
    inertia_mul(ci + 9 * l, ld3(cp + 3 * l), mass[l], ld3(cdd + 6 * l), ld3(cdd + 6 * l + 3), fa, fv);
    inertia_mul(ci + 9 * l, ld3(cp + 3 * l), mass[l], ld3(cd + 6 * l), ld3(cd + 6 * l + 3), ga, gv);
    force_cross(ld3(cd + 6 * l), ld3(cd + 6 * l + 3), ga, gv, xa, xv);
    st3(cf + 6 * l, fa + xa);
    st3(cf + 6 * l + 3, fv + xv);
  }
  tm.sync();
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      f3 sa = mk3(0.f, 0.f, 0.f), sv = mk3(0.f, 0.f, 0.f);
      for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
        sa = sa + ld3(cf + 6 * cidx[c]);
        sv = sv + ld3(cf + 6 * cidx[c] + 3);
      }
      st3(cf + 6 * l, ld3(cf + 6 * l) + sa);
      st3(cf + 6 * l + 3, ld3(cf + 6 * l + 3) + sv);
    }
    tm.sync();
  }
  // bias_d = cdof_d . cfrc[l]
  float* cdofb = a.at(A.cdofb);
  for (int d = tm.lane; d < nv; d += T) {
    float bb = -qfsb[d];
    int l = dlink[d];
    add3(cdofb + 6 * d, ld3(cf + 6 * l) * bb);
    add3(cdofb + 6 * d + 3, ld3(cf + 6 * l + 3) * bb);
  }
  for (int l = tm.lane; l < nl; l += T) {
    f3 sa = mk3(0.f, 0.f, 0.f), sv = mk3(0.f, 0.f, 0.f);
    int nd = ltype[l] == 0 ? 6 : ltype[l];
    for (int k = 0; k < nd; ++k) {
      int d = dadr[l] + k;
      float bb = -qfsb[d];
      sa = sa + ld3(cdof + 6 * d) * bb;
      sv = sv + ld3(cdof + 6 * d + 3) * bb;
    }
    st3(cfb + 6 * l, sa);
    st3(cfb + 6 * l + 3, sv);
  }
  tm.sync();
  for (int lv = 1; lv < md.nlevel; ++lv) {  // reverse of the leaf-to-root sum
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx], p = parent[l];
      st3(cfb + 6 * l, ld3(cfb + 6 * l) + ld3(cfb + 6 * p));
      st3(cfb + 6 * l + 3, ld3(cfb + 6 * l + 3) + ld3(cfb + 6 * p + 3));
    }
    tm.sync();
  }
  float* cib = a.at(A.cib);
  float* cpb = a.at(A.cpb);
  float* cdb = a.at(A.cdb);
  for (int l = tm.lane; l < nl; l += T) {
    f3 fab = ld3(cfb + 6 * l), fvb = ld3(cfb + 6 * l + 3);
    f3 pb, mab, mvb;
    inertia_mul_vjp(ci + 9 * l, ld3(cp + 3 * l), mass[l], ld3(cdd + 6 * l), ld3(cdd + 6 * l + 3), fab, fvb,
                    cib + 9 * l, pb, mab, mvb);
    add3(cpb + 3 * l, pb);
    st3(cddb + 6 * l, mab);
    st3(cddb + 6 * l + 3, mvb);
    f3 cda = ld3(cd + 6 * l), cdv = ld3(cd + 6 * l + 3);
    f3 ga, gv;
    inertia_mul(ci + 9 * l, ld3(cp + 3 * l), mass[l], cda, cdv, ga, gv);
    f3 sab, svb, gab, gvb;
    force_cross_vjp(cda, cdv, ga, gv, fab, fvb, sab, svb, gab, gvb);
    f3 pb2, cab2, cvb2;
    inertia_mul_vjp(ci + 9 * l, ld3(cp + 3 * l), mass[l], cda, cdv, gab, gvb, cib + 9 * l, pb2, cab2, cvb2);
    add3(cpb + 3 * l, pb2);
    add3(cdb + 6 * l, sab + cab2);
    add3(cdb + 6 * l + 3, svb + cvb2);
  }
  tm.sync();
  // cdd reverse: total adjoint = own + children (leaf to root)
  float* cdofdb = a.at(A.cdofdb);
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      f3 sa = ld3(cddb + 6 * l), sv = ld3(cddb + 6 * l + 3);
      for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
        sa = sa + ld3(cddb + 6 * cidx[c]);
        sv = sv + ld3(cddb + 6 * cidx[c] + 3);
      }
      st3(cddb + 6 * l, sa);
      st3(cddb + 6 * l + 3, sv);
      int nd = ltype[l] == 0 ? 6 : ltype[l];
      for (int k = 0; k < nd; ++k) {
        int d = dadr[l] + k;
        add3(cdofdb + 6 * d, sa * qd[d]);
        add3(cdofdb + 6 * d + 3, sv * qd[d]);
        qdb[d] += dot3(ld3(cdofd + 6 * d), sa) + dot3(ld3(cdofd + 6 * d + 3), sv);
      }
    }
    tm.sync();
  }
}

// Minv = M^-1 (exact): Mb = -Minv Minvb Minv  (Minv symmetric)
template <int T, int NVB>
__device__ __noinline__ void rev_inverse(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int n = md.nv, ld = L.ldm;
  float* T1 = a.at(A.tmp);
  matmul<T, NVB>(tm, n, ld, a.at(A.Minvb), w.at(L.Minv), T1, 0);
  float* Mb = a.at(A.Mb);
  matmul<T, NVB>(tm, n, ld, w.at(L.Minv), T1, Mb, 0);
  for (int j = tm.lane; j < n; j += T)
    for (int i = 0; i < n; ++i) Mb[i * ld + j] = -Mb[i * ld + j];
  tm.sync();
}

// n x n product C = alpha A B of row-major NVB x NVB blocks (rows and
// columns from n up to NVB zero), added to C when `acc`; C's entry (i, j)
// goes to C[i * cr + j * cc] (cc = NVB, cr = 1 writes the transpose).
// Register-tiled like matmul: the lanes form an RB x CB grid, each lane owns
// a TR x TC block of C, and A's rows and B's rows are read with 16-byte loads;
// every entry is one chain over k in ascending order (the zero padding adds
// exact zeros past n).
template <int T, int NVB>
__device__ void gemm_rr(const Team<T>& tm, int n, const float* A, const float* B, float* C, int cr, int cc,
                        float alpha, bool acc) {
  using G = MMTile<T, NVB>;
  static_assert(G::tiled && G::TC % 4 == 0, "gemm_rr needs a register tile of 16-byte rows");
  constexpr int lr = NVB;
  const int rb = tm.lane / G::CB, cb = tm.lane - rb * G::CB;
  const int i0 = rb * G::TR, j0 = cb * G::TC;
  if (i0 < n && j0 < n) {
    float s[G::TR][G::TC];
#pragma unroll
    for (int r = 0; r < G::TR; ++r)
#pragma unroll
      for (int c = 0; c < G::TC; ++c) s[r][c] = 0.f;
    for (int k4 = 0; k4 < n; k4 += 4) {
      float4 a4[G::TR];
#pragma unroll
      for (int r = 0; r < G::TR; ++r) a4[r] = *reinterpret_cast<const float4*>(A + (i0 + r) * lr + k4);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        float bv[G::TC];
#pragma unroll
        for (int c4 = 0; c4 < G::TC / 4; ++c4) {
          const float4 v = *reinterpret_cast<const float4*>(B + (k4 + kk) * lr + j0 + 4 * c4);
          bv[4 * c4] = v.x;
          bv[4 * c4 + 1] = v.y;
          bv[4 * c4 + 2] = v.z;
          bv[4 * c4 + 3] = v.w;
        }
#pragma unroll
        for (int r = 0; r < G::TR; ++r) {
          const float av = kk == 0 ? a4[r].x : kk == 1 ? a4[r].y : kk == 2 ? a4[r].z : a4[r].w;
#pragma unroll
          for (int c = 0; c < G::TC; ++c) s[r][c] = fmaf(av, bv[c], s[r][c]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < G::TR; ++r)
#pragma unroll
      for (int c = 0; c < G::TC; ++c) {
        const int i = i0 + r, j = j0 + c;
        if (i < n && j < n) {
          float* o = C + i * cr + j * cc;
          *o = acc ? fmaf(alpha, s[r][c], *o) : alpha * s[r][c];
        }
      }
  }
  tm.sync();
}

// Words of rev_ns's per-env scratch in global memory: the recompute's tape.
__host__ __device__ inline int ns_rev_scratch_words(int n, int nvb, int num_iter) {
  return al4(ns_tape_words(n, nvb, num_iter));
}
// Words of rev_ns's shared working set (the AdjLayout's `ns` region): M
// (n x ld), the carried inverse's transpose (an nvb x nvb block), then the
// recompute's iterate and scratch, whose words the reverse's ten nvb x nvb
// blocks take over once the recompute is done.
__host__ __device__ inline int ns_rev_smem_words(int n, int nvb) {
  const int ld = n | 1;
  const int s1 = nvb <= 16 ? 3 * n * ns_ldb(n) : 2 * n * ld;
  const int upd = al4(n * ld) + al4(s1), rev = 10 * nvb * nvb;
  return al4(n * ld) + nvb * nvb + (upd > rev ? upd : rev);
}

// mass.matrix_inv reverse in Newton-Schulz mode (brax/math.py:278-305, under
// jax.grad): the frame's inverse is the update of the carried one against M.
// From the frame's record (M, then the carried inverse before the update;
// n x ld each, global memory) the update is recomputed with its tape (the
// same calls, so the same decisions bit for bit), then reversed: Minvb (the
// result's cotangent) -> Mb, and the carried inverse's cotangent into
// Minvbc.  The reset and the acceptance decisions are piecewise constant.
// The recompute and the products run in the env's shared `ns` region
// (ns_rev_smem_words); only the tape goes to `scr` (ns_rev_scratch_words of
// global memory).  The reverse keeps every matrix as a zero-padded NVB x NVB
// row-major block, transposes included (M^T, X0^T, and per iteration the
// staged X_k, X_k^T, I + R_k and its transpose), so that each product is a
// gemm_rr of 16-byte rows.
template <int T, int NVB>
__device__ __noinline__ void rev_ns(const int* mw, Ws w, AWs a, const float* rec, float* scr, int num_iter) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  constexpr int lr = NVB, bb = NVB * NVB;
  const int n = md.nv, ld = L.ldm, lb = ns_tape_stride(n, NVB);
  float* Mr = a.at(A.ns);
  float* X0T = Mr + al4(n * ld);
  float* P = X0T + bb;  // the recompute: the iterate, then the update's scratch
  float* S1 = P + al4(n * ld);
  float* MrT = P;  // the reverse, once the recompute is done
  float* Xk = MrT + bb;
  float* XkT = Xk + bb;
  float* RkI = XkT + bb;
  float* RkIT = RkI + bb;
  float* candT = RkIT + bb;
  float* xb = candT + bb;
  float* rbar = xb + bb;
  float* xnb = rbar + bb;
  float* x0b = xnb + bb;
  float* tape = scr;
  const float* Minvb = a.at(A.Minvb);
  float* Mb = a.at(A.Mb);
  for (int e = tm.lane; e < bb; e += T) X0T[e] = 0.f;
  for (int e = tm.lane; e < n * ld; e += T) {
    Mr[e] = rec[e];
    P[e] = rec[n * ld + e];
  }
  tm.sync();
  for (int e = tm.lane; e < n * n; e += T) {  // X0^T, before the update overwrites P
    const int i = e / n, j = e - i * n;
    X0T[j * lr + i] = P[i * ld + j];
  }
  tm.sync();
  ns_update<T, NVB>(tm, n, Mr, ld, P, S1, num_iter, tape);
  {
    float4* z = reinterpret_cast<float4*>(MrT);
    for (int e = tm.lane; e < 10 * bb / 4; e += T) z[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    tm.sync();
  }
  for (int e = tm.lane; e < n * n; e += T) {
    const int i = e / n, j = e - i * n;
    MrT[j * lr + i] = Mr[i * ld + j];
    xb[i * lr + j] = Minvb[i * ld + j];
    Mb[i * ld + j] = 0.f;
  }
  tm.sync();
  for (int k = num_iter - 1; k >= 0; --k) {
    const bool keep = tape[4 + k] != 0.f;
    {  // stage the iteration's iterate X_k and I + R_k (the factor both products use), and their transposes
      const float* src = tape + 4 + al4(num_iter) + 2 * k * n * lb;
      for (int e = tm.lane; e < n * n; e += T) {
        const int i = e / n, j = e - i * n;
        const float x = src[i * lb + j];
        const float r = src[n * lb + i * lb + j] + (i == j ? 1.f : 0.f);
        Xk[i * lr + j] = x;
        XkT[j * lr + i] = x;
        RkI[i * lr + j] = r;
        RkIT[j * lr + i] = r;
      }
      tm.sync();
    }
    gemm_rr<T, NVB>(tm, n, Xk, RkI, candT, 1, lr, 1.f, false);  // the candidate Xk (I + Rk), transposed
    for (int e = tm.lane; e < n * n; e += T) {  // kept: its cotangent is the result's; else the iterate's
      const int i = e / n, j = e - i * n;
      xnb[i * lr + j] = keep ? xb[i * lr + j] : 0.f;
      if (keep) xb[i * lr + j] = 0.f;
    }
    tm.sync();
    // r_{k+1} = I - M cand
    gemm_rr<T, NVB>(tm, n, MrT, rbar, xnb, lr, 1, -1.f, true);
    gemm_rr<T, NVB>(tm, n, rbar, candT, Mb, ld, 1, -1.f, true);
    // cand = Xk (I + Rk)
    gemm_rr<T, NVB>(tm, n, xnb, RkIT, xb, lr, 1, 1.f, true);
    gemm_rr<T, NVB>(tm, n, XkT, xnb, rbar, lr, 1, 1.f, false);
  }
  // r0 = I - M X0 (of the carried inverse, whether or not it was reset)
  gemm_rr<T, NVB>(tm, n, rbar, X0T, Mb, ld, 1, -1.f, true);
  gemm_rr<T, NVB>(tm, n, MrT, rbar, x0b, lr, 1, -1.f, false);
  float* Minvbc = a.at(A.Minvbc);
  if (tape[0] != 0.f) {  // reset: x = 0.5 M^T / s, s = tr(M M^T)
    float s = 0.f, t = 0.f;
    for (int e = tm.lane; e < n * n; e += T) {
      const int i = e / n, j = e - i * n;
      const float v = Mr[i * ld + j];
      s = fmaf(v, v, s);
      t = fmaf(Mr[j * ld + i], xb[i * lr + j], t);
    }
    s = tm.sum(s);
    t = tm.sum(t);
    const float c = t / (s * s);
    for (int e = tm.lane; e < n * n; e += T) {
      const int i = e / n, j = e - i * n;
      Mb[i * ld + j] += 0.5f * xb[j * lr + i] / s - c * Mr[i * ld + j];
      Minvbc[i * ld + j] = x0b[i * lr + j];
    }
  } else {
    for (int e = tm.lane; e < n * n; e += T) {
      const int i = e / n, j = e - i * n;
      Minvbc[i * ld + j] = x0b[i * lr + j] + xb[i * lr + j];
    }
  }
  tm.sync();
}

// mass.matrix reverse (mass.py:27-83)
template <int T>
__device__ __noinline__ void rev_crba(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nl = md.nl, nv = md.nv, ld = L.ldm;
  const int* dlink = md.I(BXM_O_DOF_LINK);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* cstart = md.I(BXM_O_CHILD_START);
  const int* cidx = md.I(BXM_O_CHILD_IDX);
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const float* ci = w.at(L.ci);
  const float* cp = w.at(L.cp);
  const float* mass = md.F(BXM_O_LI_MASS);
  const float* cdof = w.at(L.cdof);
  const float* Mb = a.at(A.Mb);
  float* crbi = a.at(A.tmp);
  float* crbp = crbi + 9 * nl;
  float* crbm = crbp + 3 * nl;
  float* F = crbm + nl;        // 6 nv
  float* Fb = F + 6 * nv;      // 6 nv
  float* crbib = Fb + 6 * nv;  // 9 nl
  float* crbpb = crbib + 9 * nl;
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      float si[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      f3 sp = mk3(0.f, 0.f, 0.f);
      float sm = 0.f;
      for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
        int ch = cidx[c];
        for (int k = 0; k < 9; ++k) si[k] += crbi[9 * ch + k];
        sp = sp + ld3(crbp + 3 * ch);
        sm += crbm[ch];
      }
      for (int k = 0; k < 9; ++k) crbi[9 * l + k] = ci[9 * l + k] + si[k];
      st3(crbp + 3 * l, ld3(cp + 3 * l) + sp);
      crbm[l] = mass[l] + sm;
    }
    tm.sync();
  }
  for (int r = tm.lane; r < nv; r += T) {
    int l = dlink[r];
    f3 fa, fv;
    inertia_mul(crbi + 9 * l, ld3(crbp + 3 * l), crbm[l], ld3(cdof + 6 * r), ld3(cdof + 6 * r + 3), fa, fv);
    st3(F + 6 * r, fa);
    st3(F + 6 * r + 3, fv);
  }
  tm.sync();
  float* cdofb = a.at(A.cdofb);
  // value adjoint vb(r, c) = Mb[r][c] + Mb[c][r] (r > c), Mb[r][r]; c an ancestor dof of r
  for (int c = tm.lane; c < nv; c += T) {  // cdof_c += sum_r vb(r, c) F_r
    f3 sa = mk3(0.f, 0.f, 0.f), sv = mk3(0.f, 0.f, 0.f);
    for (int r = c; r < nv; ++r) {
      if (!((md.anc(dlink[r]) >> c) & 1ull)) continue;
      float vb = (r == c) ? Mb[r * ld + r] : Mb[r * ld + c] + Mb[c * ld + r];
      sa = sa + ld3(F + 6 * r) * vb;
      sv = sv + ld3(F + 6 * r + 3) * vb;
    }
    add3(cdofb + 6 * c, sa);
    add3(cdofb + 6 * c + 3, sv);
  }
  for (int r = tm.lane; r < nv; r += T) {  // F_r bar = sum_c vb(r, c) cdof_c
    f3 sa = mk3(0.f, 0.f, 0.f), sv = mk3(0.f, 0.f, 0.f);
    uint64_t anc = md.anc(dlink[r]);
    for (int c = 0; c <= r; ++c) {
      if (!((anc >> c) & 1ull)) continue;
      float vb = (r == c) ? Mb[r * ld + r] : Mb[r * ld + c] + Mb[c * ld + r];
      sa = sa + ld3(cdof + 6 * c) * vb;
      sv = sv + ld3(cdof + 6 * c + 3) * vb;
    }
    st3(Fb + 6 * r, sa);
    st3(Fb + 6 * r + 3, sv);
  }
  tm.sync();
  // F_r = crb[l(r)] . cdof_r : per link, its own dofs (no races)
  for (int l = tm.lane; l < nl; l += T) {
    float ib[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    f3 pbs = mk3(0.f, 0.f, 0.f);
    int nd = ltype[l] == 0 ? 6 : ltype[l];
    for (int k = 0; k < nd; ++k) {
      int r = dadr[l] + k;
      f3 pb, mab, mvb;
      inertia_mul_vjp(crbi + 9 * l, ld3(crbp + 3 * l), crbm[l], ld3(cdof + 6 * r), ld3(cdof + 6 * r + 3),
                      ld3(Fb + 6 * r), ld3(Fb + 6 * r + 3), ib, pb, mab, mvb);
      pbs = pbs + pb;
      add3(cdofb + 6 * r, mab);
      add3(cdofb + 6 * r + 3, mvb);
    }
    for (int k = 0; k < 9; ++k) crbib[9 * l + k] = ib[k];
    st3(crbpb + 3 * l, pbs);
  }
  tm.sync();
  // crb = cinr + sum(children): total = own + parent's total (root to leaf)
  for (int lv = 1; lv < md.nlevel; ++lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx], p = parent[l];
      for (int k = 0; k < 9; ++k) crbib[9 * l + k] += crbib[9 * p + k];
      st3(crbpb + 3 * l, ld3(crbpb + 3 * l) + ld3(crbpb + 3 * p));
    }
    tm.sync();
  }
  float* cib = a.at(A.cib);
  float* cpb = a.at(A.cpb);
  for (int l = tm.lane; l < nl; l += T) {
    for (int k = 0; k < 9; ++k) cib[9 * l + k] += crbib[9 * l + k];
    add3(cpb + 3 * l, ld3(crbpb + 3 * l));
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// The reverse of one active contact between two moving geoms (a sphere /
// capsule pair: contact.py:28-67 with the mjx primitives, constraint.py:
// 135-176), rows c0..c0+3 of slot kc: its rows hold both links' point
// Jacobians (J_b - J_a at the contact point), reversed into both links' cdof
// and root com; its geometry is differentiated by two_geom_contact_vjp and
// sent back through both geoms' poses.  Out of line: the plane contacts of
// rev_rows do not carry its code.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_contact_pair(const int* mw, Ws w, AWs a, int c0, int kc) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nv = md.nv, ldj = L.ldj;
  const float* qd = a.at(A.qd0);
  const float* Jb = a.at(A.Jb);
  const float* diagb = a.at(A.diagb);
  const float* arefb = a.at(A.arefb);
  float* qdb = a.at(A.qdb);
  const float* rc = w.at(L.rc);
  const float* cdof = w.at(L.cdof);
  const float* xp = w.at(L.xp);
  const float* xr = w.at(L.xr);
  float* cdofb = a.at(A.cdofb);
  float* rcb = a.at(A.rcb);
  float* xpb = a.at(A.xpb);
  float* xrb = a.at(A.xrb);
  const int kind = md.I(BXM_O_CON_KIND)[kc];
  const int la = md.I(BXM_O_CON_LA)[kc], lb = md.I(BXM_O_CON_LB)[kc];
  f3 p1, p2;
  float R1[9], R2[9];
  geom_pose(xp, xr, la, md.F(BXM_O_CON_G1POS) + 3 * kc, md.F(BXM_O_CON_G1QUAT) + 4 * kc, p1, R1);
  geom_pose(xp, xr, lb, md.F(BXM_O_CON_G2POS) + 3 * kc, md.F(BXM_O_CON_G2QUAT) + 4 * kc, p2, R2);
  const float r1 = md.F(BXM_O_CON_G1SIZE)[3 * kc], h1 = md.F(BXM_O_CON_G1SIZE)[3 * kc + 1];
  const float r2 = md.F(BXM_O_CON_G2SIZE)[3 * kc], h2 = md.F(BXM_O_CON_G2SIZE)[3 * kc + 1];
  const f3 u1 = mk3(R1[2], R1[5], R1[8]), u2 = mk3(R2[2], R2[5], R2[8]);
  float c[13];
  two_geom_contact(kind, p1, u1, r1, h1, p2, u2, r2, h2, c);
  const float dist = c[0];
  const f3 pos = ld3(c + 1), n = ld3(c + 4), t1 = ld3(c + 7), t2 = ld3(c + 10);
  const float mu = md.F(BXM_O_CON_FRIC)[kc], tw = md.F(BXM_O_CON_INVW)[kc];
  float imp, dimp, bco, kco;
  imp_parts(md.F(BXM_O_CON_SOLP) + 7 * kc, dist, imp, dimp, bco, kco);
  const f3 vq[4] = {(-t1) * (-mu) + n, (-t1) * mu + n, (-t2) * (-mu) + n, (-t2) * mu + n};
  float velb[4];
  float distb = 0.f;
  for (int qq = 0; qq < 4; ++qq) {
    const float ab = arefb[c0 + qq], db = diagb[c0 + qq];
    velb[qq] = -bco * ab;
    const float impb = -kco * dist * ab + db * (tw + mu * mu * tw) * 2.f * mu * mu * ddiag_dimp(imp);
    distb += -kco * imp * ab + impb * dimp;
  }
  // rows (J_b(pos) - J_a(pos)) . v_q, J_l(pos) = cdof_v - (pos - root_com_l) x cdof_a
  // over the dofs of l's ancestors (none for a world geom)
  const uint64_t mb = md.anc(lb), ma = la >= 0 ? md.anc(la) : 0ull;
  const f3 offb = pos - ld3(rc + 3 * lb);
  const f3 offa = la >= 0 ? pos - ld3(rc + 3 * la) : mk3(0.f, 0.f, 0.f);
  f3 obp = mk3(0.f, 0.f, 0.f), oap = obp, v0b = obp, v1b = obp, v2b = obp, v3b = obp;
  for (int d = tm.lane; d < nv; d += T) {
    float jr[4];
    for (int qq = 0; qq < 4; ++qq) {
      jr[qq] = Jb[(c0 + qq) * ldj + d] + velb[qq] * qd[d];
      qdb[d] += velb[qq] * w.jrow(c0 + qq)[d];
    }
    const bool inb = (mb >> d) & 1ull, ina = (ma >> d) & 1ull;
    if (!inb && !ina) continue;
    const f3 ca = ld3(cdof + 6 * d), cv = ld3(cdof + 6 * d + 3);
    f3 diff = mk3(0.f, 0.f, 0.f);
    if (inb) diff = cv - cross3(offb, ca);
    if (ina) diff = diff - (cv - cross3(offa, ca));
    v0b = v0b + diff * jr[0];
    v1b = v1b + diff * jr[1];
    v2b = v2b + diff * jr[2];
    v3b = v3b + diff * jr[3];
    const f3 diffb = vq[0] * jr[0] + vq[1] * jr[1] + vq[2] * jr[2] + vq[3] * jr[3];
    if (inb) {
      add3(cdofb + 6 * d + 3, diffb);
      add3(cdofb + 6 * d, -cross3(diffb, offb));
      obp = obp - cross3(ca, diffb);
    }
    if (ina) {
      add3(cdofb + 6 * d + 3, -diffb);
      add3(cdofb + 6 * d, cross3(diffb, offa));
      oap = oap + cross3(ca, diffb);
    }
  }
  const f3 offbb = mk3(tm.sum(obp.x), tm.sum(obp.y), tm.sum(obp.z));
  const f3 offab = mk3(tm.sum(oap.x), tm.sum(oap.y), tm.sum(oap.z));
  v0b = mk3(tm.sum(v0b.x), tm.sum(v0b.y), tm.sum(v0b.z));
  v1b = mk3(tm.sum(v1b.x), tm.sum(v1b.y), tm.sum(v1b.z));
  v2b = mk3(tm.sum(v2b.x), tm.sum(v2b.y), tm.sum(v2b.z));
  v3b = mk3(tm.sum(v3b.x), tm.sum(v3b.y), tm.sum(v3b.z));
  if (tm.lane == 0) {
    add3(rcb + 3 * lb, -offbb);
    if (la >= 0) add3(rcb + 3 * la, -offab);
    const f3 t1b = mu * (v0b - v1b), t2b = mu * (v2b - v3b);
    const f3 posb = offbb + offab, nb = v0b + v1b + v2b + v3b;
    const float cot[13] = {distb, posb.x, posb.y, posb.z, nb.x, nb.y, nb.z,
                           t1b.x, t1b.y, t1b.z, t2b.x, t2b.y, t2b.z};
    float inb[kContactIn];
    two_geom_contact_vjp(kind, p1, u1, r1, h1, p2, u2, r2, h2, cot, inb);
    // each geom: p = x_pos + rotate(geom_pos, x_rot), u = third column of
    // quat_to_3x3(x_rot * geom_quat)
    for (int g = 0; g < 2; ++g) {
      const int l = g == 0 ? la : lb;
      if (l < 0) continue;  // a world geom does not move
      const f3 gp = ld3(md.F(g == 0 ? BXM_O_CON_G1POS : BXM_O_CON_G2POS) + 3 * kc);
      const q4 gqr = ld4(md.F(g == 0 ? BXM_O_CON_G1QUAT : BXM_O_CON_G2QUAT) + 4 * kc);
      const q4 xl = ld4(xr + 4 * l);
      const f3 pb = mk3(inb[6 * g], inb[6 * g + 1], inb[6 * g + 2]);
      float Rb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      Rb[2] = inb[6 * g + 3];
      Rb[5] = inb[6 * g + 4];
      Rb[8] = inb[6 * g + 5];
      const q4 gq = qmul(xl, gqr);
      const q4 gqb = quat_to_3x3_vjp(gq, Rb);
      q4 xrb1, gqt, xrb2;
      f3 gpb;
      qmul_vjp(xl, gqr, gqb, xrb1, gqt);
      rotate_vjp(gp, xl, pb, gpb, xrb2);
      add3(xpb + 3 * l, pb);
      add4(xrb + 4 * l, qadd(xrb1, xrb2));
    }
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// constraint rows reverse (constraint.py:68-176): limit rows -> q, qd;
// contact rows -> qd, cdof, root_com, and the contact geometry -> x.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_rows(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nv = md.nv, ldj = L.ldj, ncon = md.ncon;
  const float* tape = a.at(A.tape);
  const int nrow = (int)tape[1];
  if (nrow <= 0) return;
  const int* rmap = reinterpret_cast<const int*>(w.at(L.rmap));
  const float* q = a.at(A.q0);
  const float* qd = a.at(A.qd0);
  const float* Jb = a.at(A.Jb);
  const float* diagb = a.at(A.diagb);
  const float* arefb = a.at(A.arefb);
  float* qb = a.at(A.qb);
  float* qdb = a.at(A.qdb);
  // limit rows: one row per dof, so lanes never collide
  for (int r = tm.lane; r < nrow; r += T) {
    int orig = rmap[r];
    if (orig < 4 * ncon) continue;
    int i = orig - 4 * ncon;
    int d = md.I(BXM_O_LIM_DOF)[i], qi = md.I(BXM_O_LIM_QADR)[i];
    float pmin = q[qi] - md.F(BXM_O_LIM_LO)[i], pmax = md.F(BXM_O_LIM_HI)[i] - q[qi];
    float pos = fminf(fminf(pmin, pmax), 0.f);
    float side = pmin < pmax ? 1.f : -1.f;
    float imp, dimp, b, k;
    imp_parts(md.F(BXM_O_LIM_SOLP) + 7 * i, pos, imp, dimp, b, k);
    float ab = arefb[r], db = diagb[r];
    qdb[d] += -b * ab * side;
    float impb = -k * pos * ab + db * md.F(BXM_O_LIM_INVW)[i] * ddiag_dimp(imp);
    float posb = -k * imp * ab + impb * dimp;
    qb[qi] += posb * (pmin <= pmax ? 1.f : -1.f);
  }
  tm.sync();
  // contact rows, one active contact at a time (rows 4c..4c+3)
  const float* rc = w.at(L.rc);
  const float* cdof = w.at(L.cdof);
  const float* xp = w.at(L.xp);
  const float* xr = w.at(L.xr);
  float* cdofb = a.at(A.cdofb);
  float* rcb = a.at(A.rcb);
  float* xpb = a.at(A.xpb);
  float* xrb = a.at(A.xrb);
  for (int c0 = 0; c0 < nrow; c0 += 4) {
    int orig = rmap[c0];
    if (orig >= 4 * ncon) break;  // contact rows come first
    int kc = orig >> 2;
    int kind = md.I(BXM_O_CON_KIND)[kc], sub = md.I(BXM_O_CON_SUB)[kc];
    if (kind == BXM_CON_SPHERE_SPHERE || kind == BXM_CON_SPHERE_CAPSULE || kind == BXM_CON_CAPSULE_CAPSULE) {
      rev_contact_pair<T>(mw, w, a, c0, kc);  // two moving geoms
      continue;
    }
    int lb = md.I(BXM_O_CON_LB)[kc];
    // recompute the contact (world plane as geom1)
    f3 p1 = ld3(md.F(BXM_O_CON_G1POS) + 3 * kc);
    float R1[9], R2[9];
    quat_to_3x3(ld4(md.F(BXM_O_CON_G1QUAT) + 4 * kc), R1);
    f3 n = mk3(R1[2], R1[5], R1[8]);
    q4 xrl = ld4(xr + 4 * lb);
    f3 gpos = ld3(md.F(BXM_O_CON_G2POS) + 3 * kc);
    q4 gquat = ld4(md.F(BXM_O_CON_G2QUAT) + 4 * kc);
    f3 p2 = ld3(xp + 3 * lb) + rotate(gpos, xrl);
    q4 gq = qmul(xrl, gquat);
    quat_to_3x3(gq, R2);
    float rad = md.F(BXM_O_CON_G2SIZE)[3 * kc], hl = md.F(BXM_O_CON_G2SIZE)[3 * kc + 1];
    f3 axis = mk3(R2[2], R2[5], R2[8]);
    f3 center = p2, wv = mk3(0.f, 0.f, 0.f), t1, t2, bvl = mk3(0.f, 0.f, 0.f);
    float bn = 1.f;
    if (kind == BXM_CON_PLANE_BOX) {  // the slot's manifold vertex, a point of the box (radius 0)
      const f3 hb = ld3(md.F(BXM_O_CON_G2SIZE) + 3 * kc);
      const int bvert = plane_box_vertex(p1, n, p2, R2, hb, sub);
      bvl = box_vertex(bvert < 0 ? 0 : bvert, hb);
      center = p2 + mk3(R2[0] * bvl.x + R2[1] * bvl.y + R2[2] * bvl.z, R2[3] * bvl.x + R2[4] * bvl.y + R2[5] * bvl.z,
                        R2[6] * bvl.x + R2[7] * bvl.y + R2[8] * bvl.z);
      rad = 0.f;
    }
    if (kind == BXM_CON_PLANE_CAPSULE) {
      center = sub == 0 ? p2 + axis * hl : p2 - axis * hl;
      wv = axis - n * dot3(n, axis);
      f3 bvec = normalize_with_norm(wv, bn);
      if (bn < 0.5f) bvec = (-0.5f < n.y && n.y < 0.5f) ? mk3(0.f, 1.f, 0.f) : mk3(0.f, 0.f, 1.f);
      t1 = bvec;
      t2 = cross3(n, bvec);
    } else {
      float F[9];
      make_frame(n, F);
      t1 = ld3(F + 3);
      t2 = ld3(F + 6);
    }
    float dist = dot3(center - p1, n) - rad;
    f3 pos = center - n * (rad + 0.5f * dist);
    float mu = md.F(BXM_O_CON_FRIC)[kc], tw = md.F(BXM_O_CON_INVW)[kc];
    const float* params = md.F(BXM_O_CON_SOLP) + 7 * kc;
    float imp, dimp, bco, kco;
    imp_parts(params, dist, imp, dimp, bco, kco);
    f3 vq[4] = {(-t1) * (-mu) + n, (-t1) * mu + n, (-t2) * (-mu) + n, (-t2) * mu + n};
    float velb[4];
    float distb = 0.f;
    for (int qq = 0; qq < 4; ++qq) {
      float ab = arefb[c0 + qq], db = diagb[c0 + qq];
      velb[qq] = -bco * ab;
      float impb = -kco * dist * ab + db * (tw + mu * mu * tw) * 2.f * mu * mu * ddiag_dimp(imp);
      distb += -kco * imp * ab + impb * dimp;
    }
    f3 offb_part = mk3(0.f, 0.f, 0.f);
    f3 v0b = mk3(0.f, 0.f, 0.f), v1b = v0b, v2b = v0b, v3b = v0b;
    uint64_t mb = md.anc(lb);
    f3 off = pos - ld3(rc + 3 * lb);
    for (int d = tm.lane; d < nv; d += T) {
      float jr[4];
      for (int qq = 0; qq < 4; ++qq) {
        jr[qq] = Jb[(c0 + qq) * ldj + d] + velb[qq] * qd[d];
        qdb[d] += velb[qq] * w.jrow(c0 + qq)[d];
      }
      if (!((mb >> d) & 1ull)) continue;
      f3 ca = ld3(cdof + 6 * d), cv = ld3(cdof + 6 * d + 3);
      f3 diff = cv - cross3(off, ca);
      v0b = v0b + diff * jr[0];
      v1b = v1b + diff * jr[1];
      v2b = v2b + diff * jr[2];
      v3b = v3b + diff * jr[3];
      f3 diffb = vq[0] * jr[0] + vq[1] * jr[1] + vq[2] * jr[2] + vq[3] * jr[3];
      add3(cdofb + 6 * d + 3, diffb);
      add3(cdofb + 6 * d, -cross3(diffb, off));
      offb_part = offb_part - cross3(ca, diffb);
    }
    f3 offb = mk3(tm.sum(offb_part.x), tm.sum(offb_part.y), tm.sum(offb_part.z));
    v0b = mk3(tm.sum(v0b.x), tm.sum(v0b.y), tm.sum(v0b.z));
    v1b = mk3(tm.sum(v1b.x), tm.sum(v1b.y), tm.sum(v1b.z));
    v2b = mk3(tm.sum(v2b.x), tm.sum(v2b.y), tm.sum(v2b.z));
    v3b = mk3(tm.sum(v3b.x), tm.sum(v3b.y), tm.sum(v3b.z));
    if (tm.lane == 0) {
      add3(rcb + 3 * lb, -offb);
      f3 t1b = mu * (v0b - v1b), t2b = mu * (v2b - v3b);
      // pos = center - n (r + 0.5 dist); dist = (center - p1) . n - r
      f3 centerb = offb;
      float db2 = distb - 0.5f * dot3(offb, n);
      centerb = centerb + n * db2;
      f3 p2b = centerb;
      float R2b[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      if (kind == BXM_CON_PLANE_BOX) {  // center = p2 + R2 v: R2b = centerb v^T
        const float cb[3] = {centerb.x, centerb.y, centerb.z}, vv[3] = {bvl.x, bvl.y, bvl.z};
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) R2b[3 * i + j] = cb[i] * vv[j];
      }
      if (kind == BXM_CON_PLANE_CAPSULE) {
        f3 axisb = centerb * (sub == 0 ? hl : -hl);
        if (bn >= 0.5f) {
          f3 bb = t1b + cross3(t2b, n);
          f3 wb = normalize3_vjp(wv, bb);
          axisb = axisb + wb - n * dot3(n, wb);
        }
        R2b[2] = axisb.x;
        R2b[5] = axisb.y;
        R2b[8] = axisb.z;
      }
      q4 gqb = quat_to_3x3_vjp(gq, R2b);
      q4 xrb1, gqt;
      qmul_vjp(xrl, gquat, gqb, xrb1, gqt);
      f3 gpb;
      q4 xrb2;
      rotate_vjp(gpos, xrl, p2b, gpb, xrb2);
      add3(xpb + 3 * lb, p2b);
      add4(xrb + 4 * lb, qadd(xrb1, xrb2));
    }
    tm.sync();
  }
}

// ---------------------------------------------------------------------------
// transform_com reverse (dynamics.py:27-134) -> x_bar (pos, normalized rot),
// q_bar (stacked joints), qd_bar (cd, cdofd).
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_com(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const AdjLayout& A = *a.A;
  const int nl = md.nl;
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* cstart = md.I(BXM_O_CHILD_START);
  const int* cidx = md.I(BXM_O_CHILD_IDX);
  const int* root = md.I(BXM_O_LINK_ROOT);
  const float* mass = md.F(BXM_O_LI_MASS);
  const float* q = a.at(A.q0);
  const float* qd = a.at(A.qd0);
  const float* cdof = w.at(L.cdof);
  const float* cd = w.at(L.cd);
  const float* xp = w.at(L.xp);
  const float* xr = w.at(L.xr);
  const float* rc = w.at(L.rc);
  float* cdofb = a.at(A.cdofb);
  float* cdofdb = a.at(A.cdofdb);
  float* cdb = a.at(A.cdb);
  float* rcb = a.at(A.rcb);
  float* xpb = a.at(A.xpb);
  float* xrb = a.at(A.xrb);
  float* qb = a.at(A.qb);
  float* qdb = a.at(A.qdb);
  float* sdb = a.at(A.tmp);  // per link: adjoint of cd[parent] from cdofd (6)
  float* ppb = sdb + 6 * nl; // per link: adjoint of the parent frame used for cdof (7)
  float* xipb = ppb + 7 * nl;  // 3 nl
  float* xirb = xipb + 3 * nl;  // 4 nl
  // 1. cdofd (dynamics.py:106-130)
  for (int l = tm.lane; l < nl; l += T) {
    int typ = ltype[l], da = dadr[l];
    f3 sab = mk3(0.f, 0.f, 0.f), svb = mk3(0.f, 0.f, 0.f);
    if (typ == 0) {
      f3 sa = ld3(cdof + 6 * da) * qd[da] + ld3(cdof + 6 * (da + 1)) * qd[da + 1];
      sa = sa + ld3(cdof + 6 * (da + 2)) * qd[da + 2];
      f3 sv = ld3(cdof + 6 * da + 3) * qd[da] + ld3(cdof + 6 * (da + 1) + 3) * qd[da + 1];
      sv = sv + ld3(cdof + 6 * (da + 2) + 3) * qd[da + 2];
      for (int k = 3; k < 6; ++k) {
        int d = da + k;
        f3 a1, v1, oab, ovb;
        motion_cross_vjp(sa, sv, ld3(cdof + 6 * d), ld3(cdof + 6 * d + 3), ld3(cdofdb + 6 * d),
                         ld3(cdofdb + 6 * d + 3), a1, v1, oab, ovb);
        sab = sab + a1;
        svb = svb + v1;
        add3(cdofb + 6 * d, oab);
        add3(cdofb + 6 * d + 3, ovb);
      }
      for (int k = 0; k < 3; ++k) {
        int d = da + k;
        add3(cdofb + 6 * d, sab * qd[d]);
        add3(cdofb + 6 * d + 3, svb * qd[d]);
        qdb[d] += dot3(ld3(cdof + 6 * d), sab) + dot3(ld3(cdof + 6 * d + 3), svb);
      }
      st3(sdb + 6 * l, mk3(0.f, 0.f, 0.f));
      st3(sdb + 6 * l + 3, mk3(0.f, 0.f, 0.f));
      continue;
    }
    int p = parent[l];
    f3 s0a = p >= 0 ? ld3(cd + 6 * p) : mk3(0.f, 0.f, 0.f);
    f3 s0v = p >= 0 ? ld3(cd + 6 * p + 3) : mk3(0.f, 0.f, 0.f);
    f3 sas[3], svs[3];
    f3 sa = s0a, sv = s0v;
    for (int k = 0; k < typ; ++k) {
      int d = da + k;
      sas[k] = sa;
      svs[k] = sv;
      sa = sa + ld3(cdof + 6 * d) * qd[d];
      sv = sv + ld3(cdof + 6 * d + 3) * qd[d];
    }
    for (int k = typ - 1; k >= 0; --k) {
      int d = da + k;
      add3(cdofb + 6 * d, sab * qd[d]);
      add3(cdofb + 6 * d + 3, svb * qd[d]);
      qdb[d] += dot3(ld3(cdof + 6 * d), sab) + dot3(ld3(cdof + 6 * d + 3), svb);
      f3 a1, v1, oab, ovb;
      motion_cross_vjp(sas[k], svs[k], ld3(cdof + 6 * d), ld3(cdof + 6 * d + 3), ld3(cdofdb + 6 * d),
                       ld3(cdofdb + 6 * d + 3), a1, v1, oab, ovb);
      sab = sab + a1;
      svb = svb + v1;
      add3(cdofb + 6 * d, oab);
      add3(cdofb + 6 * d + 3, ovb);
    }
    st3(sdb + 6 * l, sab);
    st3(sdb + 6 * l + 3, svb);
  }
  tm.sync();
  for (int l = tm.lane; l < nl; l += T) {  // gather the children's cd[parent] adjoints
    for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
      add3(cdb + 6 * l, ld3(sdb + 6 * cidx[c]));
      add3(cdb + 6 * l + 3, ld3(sdb + 6 * cidx[c] + 3));
    }
  }
  tm.sync();
  // 2. cd = cd[parent] + sum(cdof qd): totals leaf to root, then own dofs
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      f3 sa = ld3(cdb + 6 * l), sv = ld3(cdb + 6 * l + 3);
      for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
        sa = sa + ld3(cdb + 6 * cidx[c]);
        sv = sv + ld3(cdb + 6 * cidx[c] + 3);
      }
      st3(cdb + 6 * l, sa);
      st3(cdb + 6 * l + 3, sv);
      int nd = ltype[l] == 0 ? 6 : ltype[l];
      for (int k = 0; k < nd; ++k) {
        int d = dadr[l] + k;
        add3(cdofb + 6 * d, sa * qd[d]);
        add3(cdofb + 6 * d + 3, sv * qd[d]);
        qdb[d] += dot3(ld3(cdof + 6 * d), sa) + dot3(ld3(cdof + 6 * d + 3), sv);
      }
    }
    tm.sync();
  }
  // 3-4. cdof = off.do(rotate(cdof0, jj_r)) and the stacked joints; jj from the parent frame
  for (int l = tm.lane; l < nl; l += T) {
    int typ = ltype[l], da = dadr[l], qa = qadr[l];
    int pi = typ == 0 ? l : parent[l];
    f3 pp = pi >= 0 ? ld3(xp + 3 * pi) : mk3(0.f, 0.f, 0.f);
    q4 pr = pi >= 0 ? ld4(xr + 4 * pi) : qident();
    f3 ltp = ld3(md.F(BXM_O_LT_POS) + 3 * l), ljp = ld3(md.F(BXM_O_LJ_POS) + 3 * l);
    q4 ltr = ld4(md.F(BXM_O_LT_ROT) + 4 * l);
    f3 ap;
    q4 ar;
    tf_do(pp, pr, ltp, ltr, ap, ar);
    f3 jjp = ap + rotate(ljp, ar);
    q4 jjr = ar;
    f3 off2 = ld3(rc + 3 * l) - jjp;
    f3 jjpb = mk3(0.f, 0.f, 0.f);
    q4 jjrb = q4{0.f, 0.f, 0.f, 0.f};
    f3 rcbl = mk3(0.f, 0.f, 0.f);
    int nd = typ == 0 ? 6 : typ;
    // stacked-joint accumulation state (forward order), reversed below
    f3 acc_p[4];
    q4 acc_r[4];
    acc_p[0] = mk3(0.f, 0.f, 0.f);
    acc_r[0] = qident();
    if (typ != 0)
      for (int k = 0; k < typ; ++k) {
        int d = da + k;
        float qk = q[qa + k];
        q4 rk = qnormalize(quat_rot_axis(ld3(md.F(BXM_O_D_ANG) + 3 * d), qk));
        f3 pk = ld3(md.F(BXM_O_D_VEL) + 3 * d) * qk;
        tf_do(acc_p[k], acc_r[k], pk, rk, acc_p[k + 1], acc_r[k + 1]);
      }
    f3 cang0b[6], cvel0b[6];
    for (int k = 0; k < nd; ++k) {
      int d = da + k;
      f3 ang0 = ld3(md.F(BXM_O_D_ANG) + 3 * d), vel0 = ld3(md.F(BXM_O_D_VEL) + 3 * d);
      f3 ca0 = typ == 0 ? ang0 : rotate(ang0, acc_r[k]);
      f3 ca = rotate(ca0, jjr);
      f3 yb = ld3(cdofb + 6 * d + 3);
      f3 offb = -cross3(ca, yb);
      f3 angb = ld3(cdofb + 6 * d) - cross3(yb, off2);
      rcbl = rcbl + offb;
      jjpb = jjpb - offb;
      f3 a0b;
      q4 jrb;
      rotate_vjp(ca0, jjr, angb, a0b, jrb);
      jjrb = qadd(jjrb, jrb);
      cang0b[k] = a0b;
      cvel0b[k] = yb;
    }
    add3(rcb + 3 * l, rcbl);
    if (typ != 0) {  // cdof0_k = (rotate(ang_k, ar_k), rotate(vel_k, ar_k) + ap_k x a_k)
      f3 apb = mk3(0.f, 0.f, 0.f);
      q4 arb = q4{0.f, 0.f, 0.f, 0.f};
      for (int k = typ - 1; k >= 0; --k) {
        int d = da + k;
        f3 ang0 = ld3(md.F(BXM_O_D_ANG) + 3 * d), vel0 = ld3(md.F(BXM_O_D_VEL) + 3 * d);
        float qk = q[qa + k];
        q4 raw = quat_rot_axis(ang0, qk);
        q4 rk = qnormalize(raw);
        f3 pk = vel0 * qk;
        // acc_{k+1} = acc_k . (pk, rk)
        f3 ap0b, pkb;
        q4 ar0b, rkb;
        tf_do_vjp(acc_p[k], acc_r[k], pk, rk, apb, arb, ap0b, ar0b, pkb, rkb);
        q4 rawb = normalize4_vjp(raw, rkb);
        qb[qa + k] += quat_rot_axis_vjp_angle(ang0, qk, rawb) + dot3(pkb, vel0);
        apb = ap0b;
        arb = ar0b;
        f3 a_ = rotate(ang0, acc_r[k]);
        f3 apb2, ab2;
        cross_vjp(acc_p[k], a_, cvel0b[k], apb2, ab2);
        f3 t3;
        q4 arb2, arb3;
        rotate_vjp(vel0, acc_r[k], cvel0b[k], t3, arb2);
        rotate_vjp(ang0, acc_r[k], cang0b[k] + ab2, t3, arb3);
        apb = apb + apb2;
        arb = qadd(arb, qadd(arb2, arb3));
      }
    }
    // jj = parent . link.transform . link.joint
    f3 ljb;
    q4 arb1;
    rotate_vjp(ljp, ar, jjpb, ljb, arb1);
    f3 ppb_, ltpb;
    q4 prb_, ltrb;
    tf_do_vjp(pp, pr, ltp, ltr, jjpb, qadd(jjrb, arb1), ppb_, prb_, ltpb, ltrb);
    st3(ppb + 7 * l, ppb_);
    st4(ppb + 7 * l + 3, prb_);
  }
  tm.sync();
  // 5. cinr = x_i(pos - root_com).do(inertia) (brax/base.py:589-595)
  const float* cib = a.at(A.cib);
  const float* cpb = a.at(A.cpb);
  for (int l = tm.lane; l < nl; l += T) {
    f3 xip;
    q4 xir;
    tf_do(ld3(xp + 3 * l), ld4(xr + 4 * l), ld3(md.F(BXM_O_LI_POS) + 3 * l), ld4(md.F(BXM_O_LI_ROT) + 4 * l),
          xip, xir);
    float R[9];
    quat_to_3x3(xir, R);
    const float* I0 = md.F(BXM_O_LI_I) + 9 * l;
    const float* Cb = cib + 9 * l;
    float S[9], SR[9], Rb[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[3 * i + j] = Cb[3 * i + j] + Cb[3 * j + i];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) SR[3 * i + j] = S[3 * i] * R[j] + S[3 * i + 1] * R[3 + j] + S[3 * i + 2] * R[6 + j];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Rb[3 * i + j] = SR[3 * i] * I0[j] + SR[3 * i + 1] * I0[3 + j] + SR[3 * i + 2] * I0[6 + j];
    q4 xirb_ = quat_to_3x3_vjp(xir, Rb);
    f3 o = xip - ld3(rc + 3 * l);
    float trC = Cb[0] + Cb[4] + Cb[8];
    f3 So = mk3(S[0] * o.x + S[1] * o.y + S[2] * o.z, S[3] * o.x + S[4] * o.y + S[5] * o.z,
                S[6] * o.x + S[7] * o.y + S[8] * o.z);
    f3 ob = (o * (2.f * trC) - So) * mass[l] + ld3(cpb + 3 * l) * mass[l];
    st3(xipb + 3 * l, ob);
    st4(xirb + 4 * l, xirb_);
    add3(rcb + 3 * l, -ob);
  }
  tm.sync();
  // 6. root_com = sum(m x_i) / sum(m) over the link's tree
  for (int l = tm.lane; l < nl; l += T) {
    f3 tot = mk3(0.f, 0.f, 0.f);
    float mt = 0.f;
    for (int j = 0; j < nl; ++j) {
      if (root[j] != root[l]) continue;
      tot = tot + ld3(rcb + 3 * j);
      mt += mass[j];
    }
    add3(xipb + 3 * l, tot * (mass[l] / mt));
  }
  tm.sync();
  // 7. x_i = x.do(inertia.transform) and the parent-frame adjoints of step 4
  for (int l = tm.lane; l < nl; l += T) {
    f3 apb, t1;
    q4 arb, t2;
    tf_do_vjp(ld3(xp + 3 * l), ld4(xr + 4 * l), ld3(md.F(BXM_O_LI_POS) + 3 * l), ld4(md.F(BXM_O_LI_ROT) + 4 * l),
              ld3(xipb + 3 * l), ld4(xirb + 4 * l), apb, arb, t1, t2);
    add3(xpb + 3 * l, apb);
    add4(xrb + 4 * l, arb);
    for (int j = 0; j < nl; ++j) {  // links whose cdof frame is this link's frame
      int pj = ltype[j] == 0 ? j : parent[j];
      if (pj != l) continue;
      add3(xpb + 3 * l, ld3(ppb + 7 * j));
      add4(xrb + 4 * l, ld4(ppb + 7 * j + 3));
    }
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// kinematics.forward reverse (kinematics.py:31-108): x_bar -> q_bar
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void rev_fk(const int* mw, Ws w, AWs a) {
  const Model md(mw);
  const Team<T> tm;
  const AdjLayout& A = *a.A;
  const int nl = md.nl;
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* cstart = md.I(BXM_O_CHILD_START);
  const int* cidx = md.I(BXM_O_CHILD_IDX);
  const float* q = a.at(A.q0);
  float* qb = a.at(A.qb);
  float* jp3 = a.at(A.tmp);    // 3 nl
  float* jr3 = jp3 + 3 * nl;   // 4 nl
  float* xps = jr3 + 4 * nl;   // 3 nl (pos, as the forward tree built them)
  float* xraw = xps + 3 * nl;  // 4 nl (unnormalized rot)
  float* pbp = xraw + 4 * nl;  // 3 nl: parent contribution from this link
  float* pbr = pbp + 3 * nl;   // 4 nl
  float* xpt = pbr + 4 * nl;   // 3 nl: total adjoint of x pos
  float* xrt = xpt + 3 * nl;   // 4 nl: total adjoint of raw rot
  // forward recompute: jcalc + anchor + link transform, then the world tree
  for (int l = tm.lane; l < nl; l += T) {
    int typ = ltype[l], qa = qadr[l], da = dadr[l];
    f3 jp;
    q4 jr;
    if (typ == 0) {
      jp = ld3(q + qa);
      jr = ld4(q + qa + 3);
    } else {
      for (int k = 0; k < typ; ++k) {
        int d = da + k;
        float qk = q[qa + k];
        q4 rk = qnormalize(quat_rot_axis(ld3(md.F(BXM_O_D_ANG) + 3 * d), qk));
        f3 pk = ld3(md.F(BXM_O_D_VEL) + 3 * d) * qk;
        if (k == 0) {
          jp = pk;
          jr = rk;
        } else {
          f3 np_;
          q4 nr;
          tf_do(jp, jr, pk, rk, np_, nr);
          jp = np_;
          jr = nr;
        }
      }
    }
    f3 jpos = ld3(md.F(BXM_O_LJ_POS) + 3 * l);
    f3 jp2 = (jp + jpos) - rotate(jpos, jr);
    f3 op;
    q4 orr;
    tf_do(ld3(md.F(BXM_O_LT_POS) + 3 * l), ld4(md.F(BXM_O_LT_ROT) + 4 * l), jp2, jr, op, orr);
    st3(jp3 + 3 * l, op);
    st4(jr3 + 4 * l, orr);
  }
  tm.sync();
  for (int lv = 0; lv < md.nlevel; ++lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx], p = parent[l];
      if (p < 0) {
        st3(xps + 3 * l, ld3(jp3 + 3 * l));
        st4(xraw + 4 * l, ld4(jr3 + 4 * l));
      } else {
        f3 op;
        q4 orr;
        tf_do(ld3(xps + 3 * p), ld4(xraw + 4 * p), ld3(jp3 + 3 * l), ld4(jr3 + 4 * l), op, orr);
        st3(xps + 3 * l, op);
        st4(xraw + 4 * l, orr);
      }
    }
    tm.sync();
  }
  // reverse, leaf to root
  const float* xpb = a.at(A.xpb);
  const float* xrb = a.at(A.xrb);
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx], p = parent[l];
      f3 tp = ld3(xpb + 3 * l);
      q4 tr = normalize4_vjp(ld4(xraw + 4 * l), ld4(xrb + 4 * l));
      for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
        tp = tp + ld3(pbp + 3 * cidx[c]);
        tr = qadd(tr, ld4(pbr + 4 * cidx[c]));
      }
      f3 jp3b;
      q4 jr3b;
      if (p < 0) {
        jp3b = tp;
        jr3b = tr;
      } else {
        f3 ppb;
        q4 prb;
        tf_do_vjp(ld3(xps + 3 * p), ld4(xraw + 4 * p), ld3(jp3 + 3 * l), ld4(jr3 + 4 * l), tp, tr, ppb, prb, jp3b,
                  jr3b);
        st3(pbp + 3 * l, ppb);
        st4(pbr + 4 * l, prb);
      }
      st3(xpt + 3 * l, jp3b);
      st4(xrt + 4 * l, jr3b);
    }
    tm.sync();
  }
  for (int l = tm.lane; l < nl; l += T) {
    int typ = ltype[l], qa = qadr[l], da = dadr[l];
    // recompute jcalc pieces
    f3 jp;
    q4 jr;
    f3 accp[4];
    q4 accr[4];
    if (typ == 0) {
      jp = ld3(q + qa);
      jr = ld4(q + qa + 3);
    } else {
      for (int k = 0; k < typ; ++k) {
        int d = da + k;
        float qk = q[qa + k];
        q4 rk = qnormalize(quat_rot_axis(ld3(md.F(BXM_O_D_ANG) + 3 * d), qk));
        f3 pk = ld3(md.F(BXM_O_D_VEL) + 3 * d) * qk;
        if (k == 0) {
          jp = pk;
          jr = rk;
        } else {
          f3 np_;
          q4 nr;
          tf_do(jp, jr, pk, rk, np_, nr);
          jp = np_;
          jr = nr;
        }
        accp[k] = jp;
        accr[k] = jr;
      }
    }
    f3 jpos = ld3(md.F(BXM_O_LJ_POS) + 3 * l);
    f3 jp2 = (jp + jpos) - rotate(jpos, jr);
    q4 ltr = ld4(md.F(BXM_O_LT_ROT) + 4 * l);
    f3 jp2b;
    q4 t1;
    rotate_vjp(jp2, ltr, ld3(xpt + 3 * l), jp2b, t1);
    q4 t2, jrb;
    qmul_vjp(ltr, jr, ld4(xrt + 4 * l), t2, jrb);
    f3 t3;
    q4 jrb2;
    rotate_vjp(jpos, jr, -jp2b, t3, jrb2);
    jrb = qadd(jrb, jrb2);
    f3 jpb = jp2b;
    if (typ == 0) {
      add3(qb + qa, jpb);
      add4(qb + qa + 3, jrb);
      continue;
    }
    for (int k = typ - 1; k >= 0; --k) {
      int d = da + k;
      f3 ang0 = ld3(md.F(BXM_O_D_ANG) + 3 * d), vel0 = ld3(md.F(BXM_O_D_VEL) + 3 * d);
      float qk = q[qa + k];
      q4 raw = quat_rot_axis(ang0, qk);
      q4 rk = qnormalize(raw);
      f3 pk = vel0 * qk;
      f3 pkb;
      q4 rkb;
      if (k == 0) {
        pkb = jpb;
        rkb = jrb;
      } else {
        f3 apb;
        q4 arb;
        tf_do_vjp(accp[k - 1], accr[k - 1], pk, rk, jpb, jrb, apb, arb, pkb, rkb);
        jpb = apb;
        jrb = arb;
      }
      q4 rawb = normalize4_vjp(raw, rkb);
      qb[qa + k] += quat_rot_axis_vjp_angle(ang0, qk, rawb) + dot3(pkb, vel0);
    }
  }
  tm.sync();
}

}  // namespace braxg
