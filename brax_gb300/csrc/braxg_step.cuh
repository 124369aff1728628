// The fused generalized-coordinates step: one team of T lanes per env, all
// per-env working state in shared memory, the packed model in shared memory
// once per CTA.  Each stage cites the reference function it restates.
#pragma once
#include "braxg_check.h"
#include "braxg_math.cuh"
#include "model_layout.h"

namespace braxg {

// ---------------------------------------------------------------------------
// model accessor
// ---------------------------------------------------------------------------
struct Model {
  const int* w;
  int nl, nq, nv, nu, ncon, nlim, m, nlevel, ns_iters, pg_iters, pg_maxls, fluid;
  float dt, pg_tol, visc, dens;
  f3 g;
  __device__ explicit Model(const int* w_) : w(w_) {
    nl = w[BXM_H_NL];
    nq = w[BXM_H_NQ];
    nv = w[BXM_H_NV];
    nu = w[BXM_H_NU];
    ncon = w[BXM_H_NCON];
    nlim = w[BXM_H_NLIM];
    m = w[BXM_H_M];
    nlevel = w[BXM_H_NLEVEL];
    ns_iters = w[BXM_H_NS_ITERS];
    pg_iters = w[BXM_H_PG_ITERS];
    pg_maxls = w[BXM_H_PG_MAXLS];
    dt = __int_as_float(w[BXM_H_DT]);
    pg_tol = __int_as_float(w[BXM_H_PG_TOL]);
    fluid = w[BXM_H_FLUID];
    visc = __int_as_float(w[BXM_H_VISC]);
    dens = __int_as_float(w[BXM_H_DENS]);
    g = mk3(__int_as_float(w[BXM_H_GX]), __int_as_float(w[BXM_H_GY]), __int_as_float(w[BXM_H_GZ]));
  }
  __device__ __forceinline__ const int* I(int k) const { return w + w[k]; }
  __device__ __forceinline__ const float* F(int k) const {
    return reinterpret_cast<const float*>(w + w[k]);
  }
  __device__ __forceinline__ uint64_t anc(int l) const {
    const unsigned* a = reinterpret_cast<const unsigned*>(I(BXM_O_LINK_ANC));
    return (uint64_t)a[2 * l] | ((uint64_t)a[2 * l + 1] << 32);
  }
};

// ---------------------------------------------------------------------------
// per-env shared-memory layout (word offsets)
// ---------------------------------------------------------------------------
struct Layout {
  int ldm, ldj;
  int q, qd, act, qfs, qfc, qdd, tau, v1, v2, misc;
  int xp, xr, xa, xv, rc, ci, cp, cd, cdof, cdofd;
  int M, Minv;
  int J, jcap, jovf, rdiag, raref, rmap;
  int prm;  // per-env parameters: friction [ncon], actuator gain, bias_q, bias_qd [nu each]
  // per-env dynamics parameters (randomised calls only; -1 otherwise): link
  // mass [nl], link inertia [nl * 9], dof armature, damping, stiffness [nv each]
  int dprm;
  int scr, scr_words, itmp;
  int mrows;   // constraint rows of the model (4 ncon + nlim)
  int canary;  // the checked build's canary words (kCanaryWords) follow the arena here
  int total;
  // 1: the Jacobian rows beyond jcap live outside the arena, at word jovf of
  // the env's slot of the output state's cache (global memory)
  int ovf_g;
};

__host__ __device__ inline int al4(int x) { return (x + 3) & ~3; }
// Row stride of the explicit projected-gradient matrix A: a multiple of 4
// (16-byte row loads) that is 4 mod 8, so that the 8 lanes of each quarter
// warp's 16-byte loads of 8 consecutive rows cover all 32 banks once.
__host__ __device__ inline int explicit_lda(int nrow) {
  const int la = al4(nrow);
  return (la & 7) == 0 ? la + 4 : la;
}
// Row stride of the Newton-Schulz iterates: covers the register tile's
// columns (up to the dof bucket 16 / 32 / 64) with 16-byte aligned rows.
__host__ __device__ inline int ns_ldb(int nv) {
  const int nvb = nv <= 16 ? 16 : (nv <= 32 ? 32 : 64);
  return explicit_lda(nv > nvb ? nv : nvb);
}
__host__ __device__ inline int imax(int a, int b) { return a > b ? a : b; }
// words reserved after the model descriptor for the shared Layout
constexpr int kLayoutWords = 64;
// the projected-gradient solve forms A explicitly while at most this many
// constraint rows are active (else it applies A = J Minv J^T + diag implicitly)
constexpr int kMaxExplicitRows = 32;

// Per-env shared-memory arena.  The constraint Jacobian keeps its first
// kMaxExplicitRows active rows in their own slot (all the explicit solve and
// the adjoint ever see); rows beyond that exist only on the implicit path and
// sit at the end of the scratch region, which that path leaves free.  The mass
// matrix lives in scratch too (from CRBA to the inverse, and to the outputs),
// except for models whose integrator solves with M itself (ns_iters == 0).
__host__ __device__ inline Layout make_layout(int nl, int nq, int nv, int nu, int ncon, int nlim, int ns_iters,
                                              int fluid = 0, int ovf_global = 0, int dyn_dr = 0) {
  Layout L;
  const int m = 4 * ncon + nlim;
  L.ldm = nv | 1;  // odd leading dimension: conflict-free strided lane access
  L.ldj = nv | 1;
  int o = 0;
  auto take = [&](int words) {
    int at = o;
    o += al4(words);
    return at;
  };
  L.q = take(nq);
  L.qd = take(nv);
  L.act = take(nu);
  L.qfs = take(nv);
  L.qfc = take(nv);
  L.qdd = take(nv);
  L.tau = take(nv);
  L.v1 = take(nv);
  L.v2 = take(nv);
  // [0] active rows, [1] NS resets, [2..8] env-step task state, [9..10] PG
  // cycles, [11] cache tag, [12] solves stopped at maxiter, [13] bounds flags
  L.misc = take(16);
  L.xp = take(3 * nl);
  L.xr = take(4 * nl);
  L.xa = take(3 * nl);
  L.xv = take(3 * nl);
  L.rc = take(3 * nl);
  L.ci = take(9 * nl);
  L.cp = take(3 * nl);
  L.cd = take(6 * nl);
  L.cdof = take(6 * nv);
  L.cdofd = take(6 * nv);
  const bool own_m = ns_iters == 0;
  L.M = own_m ? take(nv * L.ldm) : -1;
  L.Minv = take(nv * L.ldm);
  L.jcap = m < kMaxExplicitRows ? m : kMaxExplicitRows;
  L.J = take(L.jcap * L.ldj);
  L.rdiag = take(m);
  L.raref = take(m);
  L.rmap = take(m);
  L.prm = take(ncon + 3 * nu);
  L.dprm = dyn_dr ? take(10 * nl + 3 * nv) : -1;
  // overflow Jacobian rows: at the scratch end, or outside the arena
  const int ovf = ovf_global ? 0 : (m - L.jcap) * L.ldj;
  const int nn = nv * L.ldm;
  // inverse temporaries: the sweep's rows (nv x explicit_lda(nv)), the
  // Newton-Schulz iterates and residual (3 nv x ns_ldb(nv) up to 16 dofs,
  // else 2 nv x ldm), the integrator's factor pair (2 nv x ldm)
  const int inv_tmp = imax(imax(2 * nn + 4, nv * explicit_lda(nv)), nv <= 16 ? 3 * nv * ns_ldb(nv) : 0);
  // Scratch users, each with the regions it needs at once.  The mass matrix
  // (when it lives in scratch) must survive from CRBA to the inverse and to
  // the outputs, past the contacts of the Jacobian stage; two placements are
  // tried: after the inverse temporaries, or before them.
  const int head = imax(imax(13 * nl + 6 * nv, 14 * ncon + 16), m + 4);  // CRBA, contacts, output row map
  int common = al4(14 * nl) + 4 * nv;                       // FK / com temporaries, joint quaternions
  common = imax(common, (fluid ? 21 : 12) * nl + al4(nu) + ovf);  // RNE (+ fluid forces)
  common = imax(common, 14 * ncon + 16 + ovf);              // contacts + Jacobian rows
  common = imax(common, 8 * al4(m) + 2 * al4(nv) + 16 + ovf);  // projected gradient (implicit A)
  {
    const int na = L.jcap;  // explicit A = (J Minv) J^T + diag; W shares its words with the PG vectors
    common = imax(common, na * explicit_lda(na) + al4(na) + imax(na * L.ldm, 9 * al4(na)) + 16);
  }
  common = imax(common, m + 4 + ovf);                       // output row map
  int m_off = 0, inv_off = 0, s;
  if (own_m) {
    s = imax(common, imax(head, inv_tmp));                  // inverse temporaries; integrator factor
  } else {
    const int ma = al4(imax(head, inv_tmp));                // A: M after the inverse temporaries
    const int sa = imax(common, ma + nn + ovf);
    const int mb = al4(head), ib = al4(mb + nn);            // B: M, then the inverse temporaries
    const int sb = imax(common, imax(mb + nn + ovf, ib + inv_tmp));
    if (sa <= sb) {
      m_off = ma;
      s = sa;
    } else {
      m_off = mb;
      inv_off = ib;
      s = sb;
    }
  }
  L.scr_words = al4(s);
  L.scr = take(L.scr_words);
  if (!own_m) L.M = L.scr + m_off;
  L.itmp = L.scr + inv_off;
  L.mrows = m;
  L.canary = al4(o);
  L.total = L.canary + kCanaryWords;
  L.ovf_g = ovf_global ? 1 : 0;
  L.jovf = ovf_global ? L.total : L.scr + L.scr_words - ovf;
  return L;
}

// The scratch words each stage lays its temporaries into ([start, end) arena
// offsets, the carve-outs of the stage code below), and what it must leave
// intact: the overflow Jacobian rows (live from the Jacobian stage through
// the constraint solve and the outputs) and the mass matrix when it lives in
// scratch (live from CRBA through the inverse, the Jacobian stage and the
// outputs).  The layout sizes scratch for all of them; the checked build
// verifies each against the layout and each stage's actual pointers against
// its declaration.
struct ScratchUse {
  int start, end;
  bool keep_ovf, keep_m;
};
__host__ __device__ inline ScratchUse scratch_fk(const Layout& L, int nl, int nv) {  // and transform_com
  return {L.scr, L.scr + al4(14 * nl) + 4 * nv, false, false};
}
__host__ __device__ inline ScratchUse scratch_crba(const Layout& L, int nl, int nv) {
  return {L.scr, L.scr + 13 * nl + 6 * nv, false, true};
}
__host__ __device__ inline ScratchUse scratch_inverse(const Layout& L, int nv, bool exact, bool rows4) {
  const int words = exact ? nv * explicit_lda(nv) : (rows4 ? 3 * nv * ns_ldb(nv) : 2 * nv * L.ldm);
  return {L.itmp, L.itmp + words, false, true};
}
__host__ __device__ inline ScratchUse scratch_jacobian(const Layout& L, int ncon) {
  return {L.scr, L.scr + al4(ncon) + al4(3 * ncon) + al4(9 * ncon) + ncon, true, true};
}
__host__ __device__ inline ScratchUse scratch_smooth(const Layout& L, int nl, int nu, bool fluid) {
  return {L.scr, L.scr + 12 * nl + al4(nu) + (fluid ? 9 * nl : 0), true, false};
}
__host__ __device__ inline ScratchUse scratch_pg_explicit(const Layout& L, int nrow) {
  const int a = nrow * explicit_lda(nrow) + al4(nrow);
  const int wv = nrow * L.ldm > 9 * al4(nrow) ? nrow * L.ldm : 9 * al4(nrow);
  return {L.scr, L.scr + a + wv, false, false};
}
__host__ __device__ inline ScratchUse scratch_pg_implicit(const Layout& L, int m, int nv) {
  return {L.scr, L.scr + 8 * al4(m) + 2 * al4(nv), true, false};
}
__host__ __device__ inline ScratchUse scratch_integrate(const Layout& L, int nv) {  // M + diag(damping) dt
  return {L.scr, L.scr + nv * L.ldm, false, false};
}
__host__ __device__ inline ScratchUse scratch_outputs(const Layout& L, int m, int ncon) {
  // the row map (before the outputs read the overflow rows), then the contacts
  const int c = al4(ncon) + al4(3 * ncon) + 9 * ncon;
  return {L.scr, L.scr + (m > c ? m : c), true, false};
}
// Whether a stage's declared use fits the layout (scratch_ok of braxg_check.h).
__host__ __device__ inline bool scratch_use_ok(const Layout& L, const ScratchUse& u, int nv) {
  const bool m_in = u.keep_m && L.M >= L.scr;
  return scratch_ok(L.scr, L.scr_words, L.jovf, L.ovf_g == 0, u.keep_ovf, u.start, u.end, m_in ? L.M : 0,
                    m_in ? L.M + nv * L.ldm : 0);
}

// Layout of a packed model descriptor (header words).
__host__ __device__ inline Layout layout_of(const int* w, int ovf_global = 0, int dyn_dr = 0) {
  return make_layout(w[BXM_H_NL], w[BXM_H_NQ], w[BXM_H_NV], w[BXM_H_NU], w[BXM_H_NCON], w[BXM_H_NLIM],
                     w[BXM_H_NS_ITERS], w[BXM_H_FLUID], ovf_global, dyn_dr);
}
static_assert(sizeof(Layout) <= kLayoutWords * 4, "Layout must fit its shared slot");

// ---------------------------------------------------------------------------
// team of T lanes (T in {8, 16, 32}) inside one warp
// ---------------------------------------------------------------------------
template <int T>
struct Team {
  unsigned mask;
  int lane, base;
  __device__ Team() {
    int wl = threadIdx.x & 31;
    base = (wl / T) * T;
    lane = wl - base;
    mask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << base);
  }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ float sum(float v) const {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, T);
    return v;
  }
  __device__ __forceinline__ bool all(bool p) const {
    return (__ballot_sync(mask, p) & mask) == mask;
  }
  __device__ __forceinline__ bool any(bool p) const { return (__ballot_sync(mask, p) & mask) != 0u; }
  __device__ __forceinline__ unsigned ballot(bool p) const {
    return (__ballot_sync(mask, p) & mask) >> base;
  }
};

// The dynamics parameters of an env: its own copy (randomised calls) or the
// model's.
__device__ __forceinline__ const float* link_mass(const Model& md, const Layout& L, const float* b) {
  return L.dprm >= 0 ? b + L.dprm : md.F(BXM_O_LI_MASS);
}
__device__ __forceinline__ const float* link_inertia(const Model& md, const Layout& L, const float* b) {
  return L.dprm >= 0 ? b + L.dprm + md.nl : md.F(BXM_O_LI_I);
}
__device__ __forceinline__ const float* dof_armature(const Model& md, const Layout& L, const float* b) {
  return L.dprm >= 0 ? b + L.dprm + 10 * md.nl : md.F(BXM_O_D_ARM);
}
__device__ __forceinline__ const float* dof_damping(const Model& md, const Layout& L, const float* b) {
  return L.dprm >= 0 ? b + L.dprm + 10 * md.nl + md.nv : md.F(BXM_O_D_DAMP);
}
__device__ __forceinline__ const float* dof_stiffness(const Model& md, const Layout& L, const float* b) {
  return L.dprm >= 0 ? b + L.dprm + 10 * md.nl + 2 * md.nv : md.F(BXM_O_D_STIFF);
}

// Per-env workspace handle: the env's arena base and the (shared) layout.
// Passed by value so out-of-line stages keep it in registers.
struct Ws {
  float* b;
  const Layout* L;
  float* g = nullptr;  // the env's slot of the output state's cache (overflow rows, L->ovf_g)
  __device__ __forceinline__ float* at(int off) const { return b + off; }
  // checked build: record a failed check (misc[13]) / whether one failed
  __device__ __forceinline__ void flag(unsigned bit) const {
    if (kChecked) atomicOr(reinterpret_cast<unsigned*>(b + L->misc) + 13, bit);
  }
  __device__ __forceinline__ bool failed() const {
    return kChecked && reinterpret_cast<const volatile unsigned*>(b + L->misc)[13] != 0u;
  }
  // active constraint row r of the Jacobian (first jcap rows in their slot,
  // the rest at the end of scratch or in the env's cache slot)
  __device__ __forceinline__ float* jrow(int r) const {
    if (kChecked && (r < 0 || r >= L->mrows)) {
      flag(kBoundsRow);
      return b + L->scr;
    }
    if (r < L->jcap) return b + L->J + r * L->ldj;
    return (L->ovf_g ? g : b) + L->jovf + (r - L->jcap) * L->ldj;
  }
};

// Checked build: the entry test of every stage (the canary after the arena,
// then any failed check of the env); true if the stage must return at once.
template <int T>
__device__ __forceinline__ bool bx_stop(Ws w) {
  if (!kChecked) return false;
  const Team<T> tm;
  tm.sync();
  const unsigned* c = reinterpret_cast<const unsigned*>(w.b + w.L->canary);
  bool ok = true;
  for (int i = tm.lane; i < kCanaryWords; i += T) ok = ok && c[i] == kCanary;
  if (!tm.all(ok)) w.flag(kBoundsCanary);
  tm.sync();
  return w.failed();
}

// Checked build: a stage's declared scratch use against the layout, and the
// end of its actual last region against the declaration; true (after
// flagging) if either fails, and the stage must then return before writing.
template <int T>
__device__ __forceinline__ bool bx_scratch(Ws w, const ScratchUse& u, const float* actual_end, int nv) {
  if (!kChecked) return false;
  const bool bad = !scratch_use_ok(*w.L, u, nv) || actual_end > w.b + u.end;
  if (bad) w.flag(kBoundsScratch);
  Team<T>().sync();
  return bad;
}

// Checked build: 16-byte alignment of float4 operands; true (after flagging)
// if one is misaligned.
template <int T>
__device__ __forceinline__ bool bx_misaligned(Ws w, const void* p0, const void* p1 = nullptr) {
  if (!kChecked) return false;
  const bool bad = ((reinterpret_cast<uintptr_t>(p0) | reinterpret_cast<uintptr_t>(p1)) & 15u) != 0u;
  if (bad) w.flag(kBoundsAlign);
  Team<T>().sync();
  return bad;
}

// ---------------------------------------------------------------------------
// kinematics.forward: brax/kinematics.py:31-108
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void stage_fk(const int* mw, Ws w) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  float* q = w.at(L.q);
  float* qd = w.at(L.qd);
  float* jp_ = w.at(L.scr);
  float* jr_ = jp_ + 3 * md.nl;
  float* ja_ = jr_ + 4 * md.nl;
  float* jv_ = ja_ + 3 * md.nl;
  float* jq_ = w.at(L.scr) + al4(14 * md.nl);  // [nv][4] joint rotation of each stacked dof
  if (bx_stop<T>(w) || bx_scratch<T>(w, scratch_fk(L, md.nl, md.nv), jq_ + 4 * md.nv, md.nv)) return;
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const float* dang = md.F(BXM_O_D_ANG);
  const float* dvel = md.F(BXM_O_D_VEL);
  for (int l = tm.lane; l < md.nl; l += T) {
    int typ = ltype[l], qa = qadr[l], da = dadr[l];
    f3 jp, ja, jv;
    q4 jr;
    if (typ == 0) {  // kinematics.py:47-50
      jp = ld3(q + qa);
      jr = ld4(q + qa + 3);
      ja = ld3(qd + da + 3);
      jv = ld3(qd + da);
    } else {  // kinematics.py:51-76
      for (int k = 0; k < typ; ++k) {
        int d = da + k;
        f3 ang = ld3(dang + 3 * d), vel = ld3(dvel + 3 * d);
        float qk = q[qa + k], qdk = qd[d];
        q4 rk = qnormalize(quat_rot_axis(ang, qk));
        st4(jq_ + 4 * d, rk);  // reused by transform_com's cdof
        f3 pk = vel * qk;
        f3 dak = ang * qdk, dvk = vel * qdk;
        if (k == 0) {
          jp = pk;
          jr = rk;
          ja = dak;
          jv = dvk;
        } else {
          f3 np_;
          q4 nr;
          tf_do(jp, jr, pk, rk, np_, nr);
          jp = np_;
          jr = nr;
          ja = ja + rotate(dak, rk);
          jv = jv + rotate(dvk + cross3(pk, dak), rk);
        }
      }
    }
    // joint anchor offset and link transform: kinematics.py:80-82
    f3 jpos = ld3(md.F(BXM_O_LJ_POS) + 3 * l);
    f3 anchor = rotate(jpos, jr);
    jp = (jp + jpos) - anchor;
    f3 op;
    q4 orr;
    tf_do(ld3(md.F(BXM_O_LT_POS) + 3 * l), ld4(md.F(BXM_O_LT_ROT) + 4 * l), jp, jr, op, orr);
    st3(jp_ + 3 * l, op);
    st4(jr_ + 4 * l, orr);
    st3(ja_ + 3 * l, ja);
    st3(jv_ + 3 * l, jv);
  }
  tm.sync();
  // world transforms, root-to-leaf level order (kinematics.py:84-102)
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  float* xp = w.at(L.xp);
  float* xr = w.at(L.xr);
  float* xa = w.at(L.xa);
  float* xv = w.at(L.xv);
  for (int lv = 0; lv < md.nlevel; ++lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      int p = parent[l];
      f3 jp = ld3(jp_ + 3 * l), ja = ld3(ja_ + 3 * l), jv = ld3(jv_ + 3 * l);
      q4 jr = ld4(jr_ + 4 * l);
      if (p < 0) {
        st3(xp + 3 * l, jp);
        st4(xr + 4 * l, jr);
        st3(xa + 3 * l, rotate(ja, jr));
        st3(xv + 3 * l, jv);
      } else {
        f3 pp = ld3(xp + 3 * p), pa = ld3(xa + 3 * p), pv = ld3(xv + 3 * p);
        q4 pr = ld4(xr + 4 * p);
        f3 op;
        q4 orr;
        tf_do(pp, pr, jp, jr, op, orr);
        f3 vel = pv + cross3(pa, op - pp);
        vel = vel + rotate(jv, pr);
        st3(xp + 3 * l, op);
        st4(xr + 4 * l, orr);
        st3(xa + 3 * l, pa + rotate(ja, orr));
        st3(xv + 3 * l, vel);
      }
    }
    tm.sync();
  }
  for (int l = tm.lane; l < md.nl; l += T) st4(xr + 4 * l, qnormalize(ld4(xr + 4 * l)));  // :106
  tm.sync();
}

// ---------------------------------------------------------------------------
// dynamics.transform_com: brax/generalized/dynamics.py:27-134
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void stage_com(const int* mw, Ws w) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nl = md.nl;
  float* xip = w.at(L.scr);
  float* xir = xip + 3 * nl;
  float* jjp = xir + 4 * nl;
  float* jjr = jjp + 3 * nl;
  if (bx_stop<T>(w) || bx_scratch<T>(w, scratch_fk(L, nl, md.nv), jjr + 4 * nl, md.nv)) return;
  const float* xp = w.at(L.xp);
  const float* xr = w.at(L.xr);
  const float* mass = link_mass(md, L, w.b);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  for (int l = tm.lane; l < nl; l += T) {  // x_i = x.do(inertia.transform)  :37
    f3 op;
    q4 orr;
    tf_do(ld3(xp + 3 * l), ld4(xr + 4 * l), ld3(md.F(BXM_O_LI_POS) + 3 * l),
          ld4(md.F(BXM_O_LI_ROT) + 4 * l), op, orr);
    st3(xip + 3 * l, op);
    st4(xir + 4 * l, orr);
    // parent frame for the dof motions: :47-52
    int pi = (ltype[l] == 0) ? l : parent[l];
    f3 pp = pi >= 0 ? ld3(xp + 3 * pi) : mk3(0.f, 0.f, 0.f);
    q4 pr = pi >= 0 ? ld4(xr + 4 * pi) : qident();
    f3 ap;
    q4 ar;
    tf_do(pp, pr, ld3(md.F(BXM_O_LT_POS) + 3 * l), ld4(md.F(BXM_O_LT_ROT) + 4 * l), ap, ar);
    st3(jjp + 3 * l, ap + rotate(ld3(md.F(BXM_O_LJ_POS) + 3 * l), ar));
    st4(jjr + 4 * l, ar);  // joint rotation is identity
  }
  tm.sync();
  const int* root = md.I(BXM_O_LINK_ROOT);
  float* rc = w.at(L.rc);
  float* ci = w.at(L.ci);
  float* cp = w.at(L.cp);
  for (int l = tm.lane; l < nl; l += T) {
    // root_com by segment sum over the link's tree: :38-43
    int r = root[l];
    f3 s = mk3(0.f, 0.f, 0.f);
    float ms = 0.f;
    for (int j = 0; j < nl; ++j) {
      if (root[j] != r) continue;
      s = s + mass[j] * ld3(xip + 3 * j);
      ms = ms + mass[j];
    }
    f3 com = mk3(s.x / ms, s.y / ms, s.z / ms);
    st3(rc + 3 * l, com);
    // cinr = x_i(pos - root_com).do(inertia): :44, brax/base.py:589-595
    f3 off = ld3(xip + 3 * l) - com;
    float R[9], RI[9];
    quat_to_3x3(ld4(xir + 4 * l), R);
    const float* I = link_inertia(md, L, w.b) + 9 * l;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) RI[3 * a + b] = R[3 * a] * I[b] + R[3 * a + 1] * I[3 + b] + R[3 * a + 2] * I[6 + b];
    f3 h[3];
    h[0] = cross3(off, mk3(-1.f, -0.f, -0.f));
    h[1] = cross3(off, mk3(-0.f, -1.f, -0.f));
    h[2] = cross3(off, mk3(-0.f, -0.f, -1.f));
    float m_ = mass[l];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b)
        ci[9 * l + 3 * a + b] = (RI[3 * a] * R[3 * b] + RI[3 * a + 1] * R[3 * b + 1] + RI[3 * a + 2] * R[3 * b + 2]) +
                                dot3(h[a], h[b]) * m_;
    st3(cp + 3 * l, off * m_);
  }
  tm.sync();
  // cdof via stacked joints: :55-89
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const float* dang = md.F(BXM_O_D_ANG);
  const float* dvel = md.F(BXM_O_D_VEL);
  const float* q = w.at(L.q);
  const float* qd = w.at(L.qd);
  const float* jq = w.at(L.scr) + al4(14 * nl);
  float* cdof = w.at(L.cdof);
  for (int l = tm.lane; l < nl; l += T) {
    int typ = ltype[l], da = dadr[l], qa = qadr[l];
    q4 jr = ld4(jjr + 4 * l);
    f3 off = ld3(rc + 3 * l) - ld3(jjp + 3 * l);
    int nd = typ == 0 ? 6 : typ;
    f3 ap = mk3(0.f, 0.f, 0.f);
    q4 ar = qident();
    for (int k = 0; k < nd; ++k) {
      int d = da + k;
      f3 ang = ld3(dang + 3 * d), vel = ld3(dvel + 3 * d);
      f3 ca, cv;
      if (typ == 0) {
        ca = ang;
        cv = vel;
      } else {  // inv_do(Motion) of the accumulated joint transform, brax/base.py:580-584
        ca = rotate(ang, ar);
        cv = rotate(vel, ar) + cross3(ap, ca);
        float qk = q[qa + k];
        const q4 rk = ld4(jq + 4 * d);  // forward kinematics' joint rotation of this dof
        f3 np_;
        q4 nr;
        tf_do(ap, ar, vel * qk, rk, np_, nr);
        ap = np_;
        ar = nr;
      }
      ca = rotate(ca, jr);        // :86
      cv = cv - cross3(off, ca);  // :88-89
      float* c = cdof + 6 * d;
      st3(c, ca);
      st3(c + 3, cv);
    }
  }
  tm.sync();
  // cd: root-to-leaf, cd = cd[parent] + sum(cdof * qd): :93-103
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  float* cd = w.at(L.cd);
  for (int lv = 0; lv < md.nlevel; ++lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      int p = parent[l];
      f3 a = p >= 0 ? ld3(cd + 6 * p) : mk3(0.f, 0.f, 0.f);
      f3 v = p >= 0 ? ld3(cd + 6 * p + 3) : mk3(0.f, 0.f, 0.f);
      int nd = ltype[l] == 0 ? 6 : ltype[l];
      for (int k = 0; k < nd; ++k) {
        int d = dadr[l] + k;
        a = a + ld3(cdof + 6 * d) * qd[d];
        v = v + ld3(cdof + 6 * d + 3) * qd[d];
      }
      st3(cd + 6 * l, a);
      st3(cd + 6 * l + 3, v);
    }
    tm.sync();
  }
  // cdofd: :106-130
  float* cdofd = w.at(L.cdofd);
  for (int l = tm.lane; l < nl; l += T) {
    int typ = ltype[l], da = dadr[l];
    if (typ == 0) {
      f3 sa = ld3(cdof + 6 * da) * qd[da] + ld3(cdof + 6 * (da + 1)) * qd[da + 1];
      sa = sa + ld3(cdof + 6 * (da + 2)) * qd[da + 2];
      f3 sv = ld3(cdof + 6 * da + 3) * qd[da] + ld3(cdof + 6 * (da + 1) + 3) * qd[da + 1];
      sv = sv + ld3(cdof + 6 * (da + 2) + 3) * qd[da + 2];
      for (int k = 0; k < 6; ++k) {
        int d = da + k;
        f3 ra = mk3(0.f, 0.f, 0.f), rv = mk3(0.f, 0.f, 0.f);
        if (k >= 3) motion_cross(sa, sv, ld3(cdof + 6 * d), ld3(cdof + 6 * d + 3), ra, rv);
        st3(cdofd + 6 * d, ra);
        st3(cdofd + 6 * d + 3, rv);
      }
    } else {
      int p = parent[l];
      f3 sa = p >= 0 ? ld3(cd + 6 * p) : mk3(0.f, 0.f, 0.f);
      f3 sv = p >= 0 ? ld3(cd + 6 * p + 3) : mk3(0.f, 0.f, 0.f);
      for (int k = 0; k < typ; ++k) {
        int d = da + k;
        f3 ca = ld3(cdof + 6 * d), cv = ld3(cdof + 6 * d + 3);
        f3 ra, rv;
        motion_cross(sa, sv, ca, cv, ra, rv);
        st3(cdofd + 6 * d, ra);
        st3(cdofd + 6 * d + 3, rv);
        sa = sa + ca * qd[d];
        sv = sv + cv * qd[d];
      }
    }
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// mass.matrix (CRBA): brax/generalized/mass.py:27-83
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void stage_crba(const int* mw, Ws w) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nl = md.nl, nv = md.nv, ld = L.ldm;
  float* crbi = w.at(L.scr);
  float* crbp = crbi + 9 * nl;
  float* crbm = crbp + 3 * nl;
  if (bx_stop<T>(w) || bx_scratch<T>(w, scratch_crba(L, nl, nv), crbm + nl + 6 * nv, nv)) return;
  const float* ci = w.at(L.ci);
  const float* cp = w.at(L.cp);
  const float* mass = link_mass(md, L, w.b);
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* cstart = md.I(BXM_O_CHILD_START);
  const int* cidx = md.I(BXM_O_CHILD_IDX);
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {  // leaf-to-root: crb = cinr + sum(children)
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      float si[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      f3 sp = mk3(0.f, 0.f, 0.f);
      float sm = 0.f;
      for (int c = cstart[l]; c < cstart[l + 1]; ++c) {
        int ch = cidx[c];
#pragma unroll
        for (int k = 0; k < 9; ++k) si[k] += crbi[9 * ch + k];
        sp = sp + ld3(crbp + 3 * ch);
        sm += crbm[ch];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) crbi[9 * l + k] = ci[9 * l + k] + si[k];
      st3(crbp + 3 * l, ld3(cp + 3 * l) + sp);
      crbm[l] = mass[l] + sm;
    }
    tm.sync();
  }
  const int* dlink = md.I(BXM_O_DOF_LINK);
  const float* cdof = w.at(L.cdof);
  const float* arm = dof_armature(md, L, w.b);
  float* M = w.at(L.M);
  float* F = crbm + nl;  // per dof: crb[link] * cdof (the row's force), after crb's words
  for (int r = tm.lane; r < nv; r += T) {
    int l = dlink[r];
    f3 fa, fv;
    inertia_mul(crbi + 9 * l, ld3(crbp + 3 * l), crbm[l], ld3(cdof + 6 * r), ld3(cdof + 6 * r + 3), fa, fv);
    st3(F + 6 * r, fa);
    st3(F + 6 * r + 3, fv);
  }
  tm.sync();
  // lower-triangle entries (r >= c) over the lanes, entry e = r(r+1)/2 + c
  // walked incrementally; M[r][c] = cdof[c] . F[r] for ancestor dofs
  int r = 0, c = tm.lane;
  while (c > r) {
    c -= r + 1;
    ++r;
  }
  while (r < nv) {
    const int l = dlink[r];
    float v = 0.f;
    if ((md.anc(l) >> c) & 1ull) v = dot3(ld3(cdof + 6 * c + 3), ld3(F + 6 * r + 3)) + dot3(ld3(cdof + 6 * c), ld3(F + 6 * r));
    if (c == r) v = v + arm[r];
    M[r * ld + c] = v;
    M[c * ld + r] = v;
    c += T;
    while (c > r) {
      c -= r + 1;
      ++r;
    }
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// dense helpers on nv x nv matrices (leading dimension ld)
// ---------------------------------------------------------------------------
// op 0: C = A B;  op 1: C = I - A B;  op 2: C = A (I + B)
// Register-tiled: the lanes form an RB x CB grid, each lane owns a TR x TC
// block of C (TR = NVB / RB, TC = NVB / CB).  Shapes whose tile would hold
// more than 32 accumulators use one column per lane instead.  `rows4`: B's
// rows are 16-byte aligned and zero from column n up to NVB, so a tile's
// row of B is read with 16-byte loads (the same values, the same sums).
template <int T, int NVB>
struct MMTile {
  static constexpr int RB = (T == 32) ? 8 : 4;
  static constexpr int CB = T / RB;
  static constexpr int TR = NVB / RB;
  static constexpr int TC = NVB / CB;
  static constexpr bool tiled = TR * TC <= 32;
};

template <int T, int NVB>
__device__ void matmul(const Team<T>& tm, int n, const float* A, int lda, const float* B, int ldb, float* C,
                       int ldc, int op, bool rows4 = false) {
  using G = MMTile<T, NVB>;
  if constexpr (G::tiled) {
    const int rb = tm.lane / G::CB, cb = tm.lane - (tm.lane / G::CB) * G::CB;
    const int i0 = rb * G::TR, j0 = cb * G::TC;
    if (i0 < n && j0 < n) {
      float acc[G::TR][G::TC];
#pragma unroll
      for (int r = 0; r < G::TR; ++r)
#pragma unroll
        for (int c = 0; c < G::TC; ++c) acc[r][c] = 0.f;
      for (int k = 0; k < n; ++k) {
        float a[G::TR], b[G::TC];
#pragma unroll
        for (int r = 0; r < G::TR; ++r) a[r] = (i0 + r < n) ? A[(i0 + r) * lda + k] : 0.f;
        if constexpr (G::TC % 4 == 0) {
          if (rows4) {
            const float4* b4 = reinterpret_cast<const float4*>(B + k * ldb + j0);
#pragma unroll
            for (int c = 0; c < G::TC / 4; ++c) {
              const float4 v = b4[c];
              b[4 * c] = v.x;
              b[4 * c + 1] = v.y;
              b[4 * c + 2] = v.z;
              b[4 * c + 3] = v.w;
            }
          } else {
#pragma unroll
            for (int c = 0; c < G::TC; ++c) b[c] = (j0 + c < n) ? B[k * ldb + j0 + c] : 0.f;
          }
        } else {
#pragma unroll
          for (int c = 0; c < G::TC; ++c) b[c] = (j0 + c < n) ? B[k * ldb + j0 + c] : 0.f;
        }
        if (op == 2) {
#pragma unroll
          for (int c = 0; c < G::TC; ++c)
            if (k == j0 + c) b[c] = b[c] + 1.f;
        }
#pragma unroll
        for (int r = 0; r < G::TR; ++r)
#pragma unroll
          for (int c = 0; c < G::TC; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
      }
#pragma unroll
      for (int r = 0; r < G::TR; ++r)
#pragma unroll
        for (int c = 0; c < G::TC; ++c) {
          int i = i0 + r, j = j0 + c;
          if (i < n && j < n) C[i * ldc + j] = (op == 1) ? ((i == j ? 1.f : 0.f) - acc[r][c]) : acc[r][c];
        }
    }
  } else {
    for (int j = tm.lane; j < n; j += T) {
      float acc[NVB];
#pragma unroll
      for (int i = 0; i < NVB; ++i) acc[i] = 0.f;
      for (int k = 0; k < n; ++k) {
        float b = B[k * ldb + j];
        if (op == 2 && k == j) b = b + 1.f;
#pragma unroll
        for (int i = 0; i < NVB; ++i)
          if (i < n) acc[i] = fmaf(A[i * lda + k], b, acc[i]);
      }
#pragma unroll
      for (int i = 0; i < NVB; ++i)
        if (i < n) C[i * ldc + j] = (op == 1) ? ((i == j ? 1.f : 0.f) - acc[i]) : acc[i];
    }
  }
  tm.sync();
}

template <int T, int NVB>
__device__ void matmul(const Team<T>& tm, int n, int ld, const float* A, const float* B, float* C, int op) {
  matmul<T, NVB>(tm, n, A, ld, B, ld, C, ld, op);
}

// safe_norm (brax/math.py:308-328) of an n x n matrix
template <int T>
__device__ float safe_norm_mat(const Team<T>& tm, int n, int ld, const float* R) {
  float s = 0.f;
  bool small = true;
  for (int j = tm.lane; j < n; j += T)
    for (int i = 0; i < n; ++i) {
      float v = R[i * ld + j];
      small = small && (fabsf(v) <= 1e-8f);
      s += v * v;
    }
  bool z = tm.all(small);
  s = tm.sum(s);
  return z ? 0.f : sqrtf(s);
}

// In-place lower Cholesky of the n x n matrix in A (lower triangle used).
// Returns false (team-uniform) when a pivot is not positive.
template <int T>
__device__ bool cholesky(const Team<T>& tm, int n, int ld, float* A) {
  bool ok = true;
  for (int k = 0; k < n; ++k) {
    float piv = A[k * ld + k];
    ok = ok && (piv > 0.f);
    float d = sqrtf(fmaxf(piv, 1e-30f));
    tm.sync();
    for (int i = k + 1 + tm.lane; i < n; i += T) A[i * ld + k] = A[i * ld + k] / d;
    if (tm.lane == 0) A[k * ld + k] = d;
    tm.sync();
    for (int i = k + 1 + tm.lane; i < n; i += T) {
      float lik = A[i * ld + k];
      for (int j = k + 1; j <= i; ++j) A[i * ld + j] = A[i * ld + j] - lik * A[j * ld + k];
    }
    tm.sync();
  }
  return ok;
}

// Exact SPD inverse by the symmetric sweep operator (Gauss-Jordan
// elimination kept symmetric), full rows, lanes over rows: for k = 0..n-1,
// with r = 1 / B[k][k],
//   B[i][j] -= (B[i][k] B[k][j]) r   (i, j != k),
//   B[i][k] *= r,  B[k][j] *= r  (i, j != k),   B[k][k] = -r,
// after which B = -M^-1.  The product B[i][k] B[k][j] is the same for (i, j)
// and (j, i), so B stays symmetric bit for bit and row k doubles as column k
// (one broadcast row read per step).  Plain Gauss-Jordan, whose rows drift
// apart from its columns, loses an order of magnitude of accuracy on the
// ill-conditioned mass matrices of long hanging chains.  B is n rows of
// stride explicit_lda(n) (16-byte, conflict-free row loads and stores); the
// pivots are the Schur-complement pivots that a Cholesky factorisation takes
// the square roots of, so a pivot <= 0 flags a matrix that is not positive
// definite.  Returns false (team-uniform) on a non-positive pivot.
template <int T>
__device__ bool spd_inverse_sweep(const Team<T>& tm, int n, int ld, const float* Msrc, float* B, float* Minv) {
  const int lb = explicit_lda(n), w4 = al4(n);
  for (int e = tm.lane; e < n * w4; e += T) {
    const int i = e / w4, j = e - i * w4;
    B[i * lb + j] = j < n ? Msrc[i * ld + j] : 0.f;
  }
  tm.sync();
  bool ok = true;
  for (int k = 0; k < n; ++k) {
    const float d = B[k * lb + k];
    ok = ok && (d > 0.f);
    const float r = 1.f / d;
    const float4* rk = reinterpret_cast<const float4*>(B + k * lb);
    for (int i = tm.lane; i < n; i += T) {  // every row but k, from the old row k
      if (i == k) continue;
      float4* ri = reinterpret_cast<float4*>(B + i * lb);
      const float bik = B[i * lb + k];
      for (int c = 0; c < w4 / 4; ++c) {
        const float4 a = rk[c];
        float4 v = ri[c];
        v.x = fmaf(-(bik * a.x), r, v.x);
        v.y = fmaf(-(bik * a.y), r, v.y);
        v.z = fmaf(-(bik * a.z), r, v.z);
        v.w = fmaf(-(bik * a.w), r, v.w);
        ri[c] = v;
      }
      B[i * lb + k] = bik * r;
    }
    tm.sync();
    for (int j = tm.lane; j < n; j += T) B[k * lb + j] = j == k ? -r : B[k * lb + j] * r;  // row k
    tm.sync();
  }
  for (int e = tm.lane; e < n * n; e += T) {  // Minv = -B (symmetric)
    const int i = e / n, j = e - i * n;
    Minv[i * ld + j] = -B[i * lb + j];
  }
  tm.sync();
  return ok;
}

// Words of ns_update's tape for n dofs and num_iter iterations, and the row
// stride of its matrices (the stride the iteration itself uses).
__host__ __device__ inline int ns_tape_stride(int n, int nvb) { return nvb <= 16 ? ns_ldb(n) : (n | 1); }
__host__ __device__ inline int ns_tape_words(int n, int nvb, int num_iter) {
  return 4 + al4(num_iter) + 2 * num_iter * n * ns_tape_stride(n, nvb);
}

// Newton-Schulz update of the carried inverse P (n x n, stride ld) against M
// (brax/math.py:278-305): r0 = I - M P; when |r0| > 1, P restarts from
// 0.5 M^T / tr(M M^T) (r0 is kept, as the reference does); then num_iter
// updates x <- x (I + r), r <- I - M x, each kept only if its residual norm
// is below the previous one.  S1: scratch of 3 n x ns_ldb(n) words up to 16
// dofs (iterates and residuals in rows of that stride: 16-byte loads of every
// product's right-hand operand, columns n .. stride zero), 2 n x ld above
// (the iterate stays in P).  `tape` (optional; the gradient's recompute, in
// global memory): word 0 the reset, words 4 .. 4 + num_iter whether each
// iteration was kept, then per iteration its iterate and residual at the
// iteration's start (n x ns_tape_stride each).  The same calls in the same
// order with or without a tape, so a recompute from the same inputs takes the
// same decisions bit for bit.  Returns whether it reset.
template <int T, int NVB>
__device__ bool ns_update(const Team<T>& tm, int n, const float* M, int ld, float* P, float* S1, int num_iter,
                          float* tape) {
  constexpr bool kRows4 = NVB <= 16;
  const int lb = kRows4 ? ns_ldb(n) : ld;
  float* cur = kRows4 ? S1 : P;
  float* nxt = kRows4 ? S1 + n * lb : S1 + n * ld;
  float* R = kRows4 ? S1 + 2 * n * lb : S1;
  if (kRows4) {
    for (int e = tm.lane; e < 3 * n * lb; e += T) {
      const int i = e / lb, j = e - i * lb;  // rows of the three buffers in turn
      S1[e] = (j < n && i < n) ? P[i * ld + j] : 0.f;
    }
    tm.sync();
  }
  matmul<T, NVB>(tm, n, M, ld, cur, lb, R, lb, 1, kRows4);  // r0 = I - A A_inv
  float nr0 = safe_norm_mat<T>(tm, n, lb, R);
  const bool reset = nr0 > 1.f;
  if (reset) {  // reset to 0.5 A^T / tr(A A^T) (r0 is kept, as the reference does)
    float s = 0.f;
    for (int j = tm.lane; j < n; j += T)
      for (int i = 0; i < n; ++i) {
        float v = M[i * ld + j];
        s += v * v;
      }
    s = tm.sum(s);
    for (int j = tm.lane; j < n; j += T)
      for (int i = 0; i < n; ++i) cur[i * lb + j] = 0.5f * M[j * ld + i] / s;
    tm.sync();
  }
  if (tape != nullptr && tm.lane == 0) tape[0] = reset ? 1.f : 0.f;
  float err = 1.f;
  for (int it = 0; it < num_iter; ++it) {
    if (tape != nullptr) {  // the iteration's iterate and residual at its start
      float* xk = tape + 4 + al4(num_iter) + 2 * it * n * lb;
      float* rk = xk + n * lb;
      for (int e = tm.lane; e < n * lb; e += T) {
        xk[e] = cur[e];
        rk[e] = R[e];
      }
      tm.sync();
    }
    matmul<T, NVB>(tm, n, cur, lb, R, lb, nxt, lb, 2, kRows4);  // a_inv (I + r)
    matmul<T, NVB>(tm, n, M, ld, nxt, lb, R, lb, 1, kRows4);    // I - a a_inv_next
    float e = safe_norm_mat<T>(tm, n, lb, R);
    const bool keep = e < err;
    if (tape != nullptr && tm.lane == 0) tape[4 + it] = keep ? 1.f : 0.f;
    if (keep) {
      float* t = cur;
      cur = nxt;
      nxt = t;
    }
    err = e;
  }
  if (cur != P) {
    for (int j = tm.lane; j < n; j += T)
      for (int i = 0; i < n; ++i) P[i * ld + j] = cur[i * lb + j];
    tm.sync();
  }
  return reset;
}

// ---------------------------------------------------------------------------
// mass.matrix_inv: brax/generalized/mass.py:86-106 + brax/math.py:278-305
// mode 0 keeps/updates Minv by Newton-Schulz (num_iter iterations; 0 keeps
// the input); mode 1 recomputes the exact SPD inverse.
// ---------------------------------------------------------------------------
template <int T, int NVB>
__device__ __noinline__ bool stage_inverse(const int* mw, Ws w, bool exact, int num_iter) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int n = md.nv, ld = L.ldm;
  float* M = w.at(L.M);
  float* P = w.at(L.Minv);
  float* S1 = w.at(L.itmp);
  if (n == 0) return true;
  if (bx_stop<T>(w)) return true;
  if (exact) {
    if (bx_scratch<T>(w, scratch_inverse(L, n, true, false), S1 + n * explicit_lda(n), n) ||
        bx_misaligned<T>(w, S1))
      return true;
    return spd_inverse_sweep<T>(tm, n, ld, M, S1, P);
  }
  if (num_iter <= 0) return true;
  constexpr bool kRows4 = NVB <= 16;
  const int lb = kRows4 ? ns_ldb(n) : ld;
  if (bx_scratch<T>(w, scratch_inverse(L, n, false, kRows4), S1 + (kRows4 ? 3 * n * lb : 2 * n * ld), n) ||
      bx_misaligned<T>(w, kRows4 ? S1 : nullptr))
    return true;
  if (ns_update<T, NVB>(tm, n, M, ld, P, S1, num_iter, nullptr) && tm.lane == 0)
    reinterpret_cast<int*>(w.at(L.misc))[1] += 1;
  return true;
}

// ---------------------------------------------------------------------------
// constraint._imp_aref: brax/generalized/constraint.py:29-65
// ---------------------------------------------------------------------------
__device__ __forceinline__ void imp_aref(const float* p, float pos, float vel, float& imp, float& aref) {
  float timeconst = p[0], dampratio = p[1], dmin = p[2], dmax = p[3], width = p[4], mid = p[5], power = p[6];
  float imp_x = fabsf(pos) / width;
  float imp_a = (1.f / pow_fast(mid, power - 1.f)) * pow_fast(imp_x, power);
  float imp_b = 1.f - (1.f / pow_fast(1.f - mid, power - 1.f)) * pow_fast(1.f - imp_x, power);
  float imp_y = imp_x < mid ? imp_a : imp_b;
  imp = dmin + imp_y * (dmax - dmin);
  imp = fminf(fmaxf(imp, dmin), dmax);
  imp = imp_x > 1.f ? dmax : imp;
  float b = 2.f / (dmax * timeconst);
  float k = 1.f / (dmax * dmax * timeconst * timeconst * dampratio * dampratio);
  b = dampratio <= 0.f ? -dampratio / dmax : b;
  k = timeconst <= 0.f ? -timeconst / (dmax * dmax) : k;
  aref = -b * vel - k * imp * pos;
}

// ---------------------------------------------------------------------------
// contact.get + mujoco.mjx primitive collisions: brax/contact.py:28-67
// ---------------------------------------------------------------------------
__device__ __forceinline__ void geom_pose(const float* xp, const float* xr, int link, const float* gp,
                                         const float* gq, f3& pos, float* R) {
  f3 lp = link >= 0 ? ld3(xp + 3 * link) : mk3(0.f, 0.f, 0.f);
  q4 lr = link >= 0 ? ld4(xr + 4 * link) : qident();
  pos = lp + rotate(ld3(gp), lr);
  quat_to_3x3(qmul(lr, ld4(gq)), R);
}

__device__ __forceinline__ void plane_sphere(f3 n, f3 pp, f3 sp, float r, float& dist, f3& pos) {
  dist = dot3(sp - pp, n) - r;
  pos = sp - n * (r + 0.5f * dist);
}

__device__ __forceinline__ void sphere_sphere(f3 p1, float r1, f3 p2, float r2, float& dist, f3& pos, f3& n) {
  float d;
  n = normalize_with_norm(p2 - p1, d);
  if (d == 0.f) n = mk3(1.f, 0.f, 0.f);
  dist = d - (r1 + r2);
  pos = p1 + n * (r1 + 0.5f * dist);
}

__device__ __forceinline__ f3 closest_segment_point(f3 a, f3 b, f3 pt) {
  f3 ab = b - a;
  float t = dot3(pt - a, ab) / (dot3(ab, ab) + 1e-6f);
  return a + fminf(fmaxf(t, 0.f), 1.f) * ab;
}

__device__ __forceinline__ void closest_seg_seg(f3 a0, f3 a1, f3 b0, f3 b1, f3& ba, f3& bb) {
  float la, lb;
  f3 da = normalize_with_norm(a1 - a0, la);
  f3 db = normalize_with_norm(b1 - b0, lb);
  float ha = la * 0.5f, hb = lb * 0.5f;
  f3 am = a0 + da * ha, bm = b0 + db * hb;
  f3 tr = am - bm;
  float dd = dot3(da, db), dat = dot3(da, tr), dbt = dot3(db, tr);
  float denom = 1.f - dd * dd;
  float ta0 = (-dat + dd * dbt) / (denom + 1e-6f);
  float tb0 = dbt + ta0 * dd;
  float ta = fminf(fmaxf(ta0, -ha), ha), tb = fminf(fmaxf(tb0, -hb), hb);
  f3 besta = am + da * ta, bestb = bm + db * tb;
  f3 na = closest_segment_point(a0, a1, bestb);
  f3 nb = closest_segment_point(b0, b1, besta);
  float d1 = dot3(bestb - na, bestb - na), d2 = dot3(besta - nb, besta - nb);
  if (d1 < d2) {
    ba = na;
  } else {
    ba = besta;
    bestb = nb;
  }
  bb = bestb;
}

// mujoco.mjx plane-box (mujoco-mjx _src/collision_convex.py: the
// plane-convex routine and its 4-point manifold): the box's 8 vertices (x
// slowest, itertools.product order), in the box frame, against the plane of
// normal n through p1; a vertex is a candidate when it lies below the plane
// or within a 1 mm skin above it.  The manifold is a (the first candidate),
// b (the candidate furthest from a), c (furthest from the line ab in the
// plane), d (furthest from the edges bc or ac, bc's first); every argmax
// keeps the first of equal values.  Slot `sub` takes the sub-th of (a, b, c,
// d); a vertex already taken by an earlier slot gets dist 1 (inactive).
__device__ __forceinline__ f3 box_vertex(int v, f3 h) {
  return mk3((v & 4) ? h.x : -h.x, (v & 2) ? h.y : -h.y, (v & 1) ? h.z : -h.z);
}
__device__ __forceinline__ void plane_box(f3 p1, f3 n, f3 p2, const float* R2, f3 h, int sub, float& dist, f3& pos,
                                          int* vert = nullptr) {
  const f3 dp = p1 - p2;  // box frame: R2^T (p1 - p2), R2^T n
  const f3 rel = mk3(R2[0] * dp.x + R2[3] * dp.y + R2[6] * dp.z, R2[1] * dp.x + R2[4] * dp.y + R2[7] * dp.z,
                     R2[2] * dp.x + R2[5] * dp.y + R2[8] * dp.z);
  const f3 nl = mk3(R2[0] * n.x + R2[3] * n.y + R2[6] * n.z, R2[1] * n.x + R2[4] * n.y + R2[7] * n.z,
                    R2[2] * n.x + R2[5] * n.y + R2[8] * n.z);
  float support[8];
  unsigned cand = 0u;
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    support[v] = dot3(rel - box_vertex(v, h), nl);
    if (support[v] > -1e-3f) cand |= 1u << v;
  }
  auto dm = [&](int v) { return ((cand >> v) & 1u) ? 0.f : -1e6f; };
  int ia = 0;  // first candidate (vertex 0 when there is none)
  for (int v = 0; v < 8; ++v)
    if ((cand >> v) & 1u) {
      ia = v;
      break;
    }
  const f3 a = box_vertex(ia, h);
  int ib = 0;
  float best = -INFINITY;
  for (int v = 0; v < 8; ++v) {
    const f3 e = a - box_vertex(v, h);
    const float s = dot3(e, e) + dm(v);
    if (s > best) {
      best = s;
      ib = v;
    }
  }
  const f3 b = box_vertex(ib, h);
  const f3 ab = cross3(nl, a - b);
  int ic = 0;
  best = -INFINITY;
  for (int v = 0; v < 8; ++v) {
    const float s = fabsf(dot3(a - box_vertex(v, h), ab)) + dm(v);
    if (s > best) {
      best = s;
      ic = v;
    }
  }
  const f3 c = box_vertex(ic, h);
  const f3 ac = cross3(nl, a - c), bc = cross3(nl, b - c);
  int id = 0;
  best = -INFINITY;
  for (int v = 0; v < 16; ++v) {  // [|(b - p).bc| over p, then |(a - p).ac| over p]
    const f3 pv = box_vertex(v & 7, h);
    const float s = (v < 8 ? fabsf(dot3(b - pv, bc)) : fabsf(dot3(a - pv, ac))) + dm(v & 7);
    if (s > best) {
      best = s;
      id = v & 7;
    }
  }
  const int idx[4] = {ia, ib, ic, id};
  const int i = idx[sub];
  bool unique = true;
  for (int j = 0; j < sub; ++j) unique = unique && idx[j] != i;
  dist = unique ? -support[i] : 1.f;
  if (vert != nullptr) *vert = unique ? i : -1;  // the slot's vertex (box frame, box_vertex order)
  const f3 vl = box_vertex(i, h);
  const f3 vw = mk3(R2[0] * vl.x + R2[1] * vl.y + R2[2] * vl.z, R2[3] * vl.x + R2[4] * vl.y + R2[5] * vl.z,
                    R2[6] * vl.x + R2[7] * vl.y + R2[8] * vl.z);
  pos = p2 + vw - n * (0.5f * dist);
}

// Writes dist[k], pos[k*3], frame[k*9] for every contact slot.
template <int T>
__device__ __noinline__ void stage_contacts(const int* mw, Ws w, float* dist, float* cpos, float* frame) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const float* xp = w.at(L.xp);
  const float* xr = w.at(L.xr);
  const int* kind = md.I(BXM_O_CON_KIND);
  const int* sub = md.I(BXM_O_CON_SUB);
  const int* la = md.I(BXM_O_CON_LA);
  const int* lb = md.I(BXM_O_CON_LB);
  const float* g1p = md.F(BXM_O_CON_G1POS);
  const float* g1q = md.F(BXM_O_CON_G1QUAT);
  const float* g1s = md.F(BXM_O_CON_G1SIZE);
  const float* g2p = md.F(BXM_O_CON_G2POS);
  const float* g2q = md.F(BXM_O_CON_G2QUAT);
  const float* g2s = md.F(BXM_O_CON_G2SIZE);
  for (int k = tm.lane; k < md.ncon; k += T) {
    f3 p1, p2;
    float R1[9], R2[9];
    geom_pose(xp, xr, la[k], g1p + 3 * k, g1q + 4 * k, p1, R1);
    geom_pose(xp, xr, lb[k], g2p + 3 * k, g2q + 4 * k, p2, R2);
    float* F = frame + 9 * k;
    float d = 0.f;
    f3 pos = mk3(0.f, 0.f, 0.f);
    int kd = kind[k];
    if (kd == BXM_CON_PLANE_SPHERE) {
      f3 n = mk3(R1[2], R1[5], R1[8]);
      plane_sphere(n, p1, p2, g2s[3 * k], d, pos);
      make_frame(n, F);
    } else if (kd == BXM_CON_PLANE_CAPSULE) {
      f3 n = mk3(R1[2], R1[5], R1[8]), axis = mk3(R2[2], R2[5], R2[8]);
      float bn;
      f3 b = normalize_with_norm(axis - n * dot3(n, axis), bn);
      if (bn < 0.5f) b = (-0.5f < n.y && n.y < 0.5f) ? mk3(0.f, 1.f, 0.f) : mk3(0.f, 0.f, 1.f);
      f3 seg = axis * g2s[3 * k + 1];
      f3 c = sub[k] == 0 ? p2 + seg : p2 - seg;
      plane_sphere(n, p1, c, g2s[3 * k], d, pos);
      st3(F, n);
      st3(F + 3, b);
      st3(F + 6, cross3(n, b));
    } else if (kd == BXM_CON_PLANE_BOX) {
      f3 n = mk3(R1[2], R1[5], R1[8]);
      plane_box(p1, n, p2, R2, mk3(g2s[3 * k], g2s[3 * k + 1], g2s[3 * k + 2]), sub[k], d, pos);
      make_frame(n, F);
    } else if (kd == BXM_CON_SPHERE_SPHERE) {
      f3 n;
      sphere_sphere(p1, g1s[3 * k], p2, g2s[3 * k], d, pos, n);
      make_frame(n, F);
    } else if (kd == BXM_CON_SPHERE_CAPSULE) {
      f3 seg = mk3(R2[2], R2[5], R2[8]) * g2s[3 * k + 1];
      f3 pt = closest_segment_point(p2 - seg, p2 + seg, p1);
      f3 n;
      sphere_sphere(p1, g1s[3 * k], pt, g2s[3 * k], d, pos, n);
      make_frame(n, F);
    } else {  // capsule-capsule
      f3 s1 = mk3(R1[2], R1[5], R1[8]) * g1s[3 * k + 1];
      f3 s2 = mk3(R2[2], R2[5], R2[8]) * g2s[3 * k + 1];
      f3 a, b, n;
      closest_seg_seg(p1 - s1, p1 + s1, p2 - s2, p2 + s2, a, b);
      sphere_sphere(a, g1s[3 * k], b, g2s[3 * k], d, pos, n);
      make_frame(n, F);
    }
    dist[k] = d;
    st3(cpos + 3 * k, pos);
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// constraint.jacobian (active rows only, compacted): constraint.py:101-191.
// Rows whose mask (dist < 0 / pos < 0) is off are exactly zero in the
// reference (jac, diag and aref are multiplied by the mask), so they add
// nothing to A x + b; only the active rows are stored, in reference order.
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void stage_jacobian(const int* mw, Ws w) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nv = md.nv, ncon = md.ncon;
  float* dist = w.at(L.scr);
  float* cpos = dist + al4(ncon);
  float* frame = cpos + al4(3 * ncon);
  int* rcon = reinterpret_cast<int*>(frame + al4(9 * ncon));
  if (bx_stop<T>(w) || bx_scratch<T>(w, scratch_jacobian(L, ncon), frame + al4(9 * ncon) + ncon, nv)) return;
  int* rmap = reinterpret_cast<int*>(w.at(L.rmap));
  float* rdiag = w.at(L.rdiag);
  float* raref = w.at(L.raref);
  const float* qd = w.at(L.qd);
  const float* q = w.at(L.q);
  int nact = 0;
  if (ncon > 0) {
    stage_contacts<T>(md.w, w, dist, cpos, frame);
    for (int base = 0; base < ncon; base += T) {
      int k = base + tm.lane;
      bool a = k < ncon && dist[k] < 0.f;
      unsigned bal = tm.ballot(a);
      if (a) rcon[nact + __popc(bal & ((1u << tm.lane) - 1u))] = k;
      nact += __popc(bal);
    }
    tm.sync();
    const int* la = md.I(BXM_O_CON_LA);
    const int* lb = md.I(BXM_O_CON_LB);
    const float* fric = w.at(L.prm);  // per-env sliding friction
    const float* rc = w.at(L.rc);
    const float* cdof = w.at(L.cdof);
    // constraint.py:154-164: lanes over the (active contact, dof) pairs, all
    // active contacts' 4 pyramid rows in one pass (pair e: contact e / nv,
    // dof e % nv, walked incrementally)
    int c = 0, d = tm.lane;
    while (d >= nv) {
      d -= nv;
      ++c;
    }
    for (; c < nact;) {
      const int k = rcon[c];
      const int a = la[k], b = lb[k];
      const uint64_t ma = a >= 0 ? md.anc(a) : 0ull, mb = md.anc(b);
      const f3 p = ld3(cpos + 3 * k);
      const f3 offa = a >= 0 ? p - ld3(rc + 3 * a) : mk3(0.f, 0.f, 0.f);
      const f3 offb = p - ld3(rc + 3 * b);
      const f3 n = ld3(frame + 9 * k), t1 = ld3(frame + 9 * k + 3), t2 = ld3(frame + 9 * k + 6);
      const float mu = fric[k];
      const f3 v0 = (-t1) * (-mu) + n, v1 = (-t1) * mu + n, v2 = (-t2) * (-mu) + n, v3 = (-t2) * mu + n;
      const f3 ca = ld3(cdof + 6 * d), cv = ld3(cdof + 6 * d + 3);
      const f3 jb = ((mb >> d) & 1ull) ? cv - cross3(offb, ca) : mk3(0.f, 0.f, 0.f);
      const f3 ja = ((ma >> d) & 1ull) ? cv - cross3(offa, ca) : mk3(0.f, 0.f, 0.f);
      const f3 diff = jb - ja;
      w.jrow(4 * c)[d] = dot3(diff, v0);
      w.jrow(4 * c + 1)[d] = dot3(diff, v1);
      w.jrow(4 * c + 2)[d] = dot3(diff, v2);
      w.jrow(4 * c + 3)[d] = dot3(diff, v3);
      d += T;
      while (d >= nv) {
        d -= nv;
        ++c;
      }
    }
    for (int r = tm.lane; r < 4 * nact; r += T) rmap[r] = 4 * rcon[r >> 2] + (r & 3);
  }
  int nrow = 4 * nact;
  if (md.nlim > 0) {  // constraint.py:101-132
    const float* lo = md.F(BXM_O_LIM_LO);
    const float* hi = md.F(BXM_O_LIM_HI);
    const int* lq = md.I(BXM_O_LIM_QADR);
    const int* ldof = md.I(BXM_O_LIM_DOF);
    for (int base = 0; base < md.nlim; base += T) {
      int i = base + tm.lane;
      bool a = false;
      float side = 0.f;
      if (i < md.nlim) {
        float pmin = q[lq[i]] - lo[i], pmax = hi[i] - q[lq[i]];
        float pos = fminf(fminf(pmin, pmax), 0.f);
        a = pos < 0.f;
        side = pmin < pmax ? 1.f : -1.f;
      }
      unsigned bal = tm.ballot(a);
      tm.sync();
      if (a) {
        int r = nrow + __popc(bal & ((1u << tm.lane) - 1u));
        rmap[r] = 4 * ncon + i;
        float* jr = w.jrow(r);
        for (int d = 0; d < nv; ++d) jr[d] = (d == ldof[i]) ? side : 0.f;
      }
      nrow += __popc(bal);
    }
  }
  tm.sync();
  // per-row impedance, reference acceleration and A diagonal
  const float* csolp = md.F(BXM_O_CON_SOLP);
  const float* cinvw = md.F(BXM_O_CON_INVW);
  const float* fric = w.at(L.prm);
  for (int r = tm.lane; r < nrow; r += T) {
    int orig = rmap[r];
    float vel = 0.f;
    const float* jr = w.jrow(r);
    for (int d = 0; d < nv; ++d) vel += jr[d] * qd[d];
    float imp, aref, diag;
    if (orig < 4 * ncon) {  // constraint.py:167-174
      int k = orig >> 2;
      imp_aref(csolp + 7 * k, dist[k], vel, imp, aref);
      float mu = fric[k], tw = cinvw[k];
      diag = (tw + mu * mu * tw) * (2.f * mu * mu * (1.f - imp) / (imp + 1e-8f));
    } else {  // constraint.py:121-130
      int i = orig - 4 * ncon;
      const int* lq = md.I(BXM_O_LIM_QADR);
      float pmin = q[lq[i]] - md.F(BXM_O_LIM_LO)[i], pmax = md.F(BXM_O_LIM_HI)[i] - q[lq[i]];
      float pos = fminf(fminf(pmin, pmax), 0.f);
      imp_aref(md.F(BXM_O_LIM_SOLP) + 7 * i, pos, vel, imp, aref);
      diag = md.F(BXM_O_LIM_INVW)[i] * (1.f - imp) / (imp + 1e-8f);
    }
    rdiag[r] = diag;
    raref[r] = aref;
  }
  if (tm.lane == 0) reinterpret_cast<int*>(w.at(L.misc))[0] = nrow;
  tm.sync();
}

// ---------------------------------------------------------------------------
// actuator.to_tau (brax/actuator.py:23-57), dynamics.forward with _passive
// and inverse/RNE (brax/generalized/dynamics.py:137-236) -> qf_smooth
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ void stage_smooth(const int* mw, Ws w, bool has_act) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nl = md.nl, nv = md.nv;
  float* cdd = w.at(L.scr);
  float* cf = cdd + 6 * nl;
  float* force = cf + 6 * nl;
  if (bx_stop<T>(w) ||
      bx_scratch<T>(w, scratch_smooth(L, nl, md.nu, md.fluid), force + al4(md.nu) + (md.fluid ? 9 * nl : 0), nv))
    return;
  const float* q = w.at(L.q);
  const float* qd = w.at(L.qd);
  const float* act = w.at(L.act);
  const int* aqid = md.I(BXM_O_ACT_QID);
  const int* aqdid = md.I(BXM_O_ACT_QDID);
  if (has_act) {
    for (int a = tm.lane; a < md.nu; a += T) {
      const float* cr = md.F(BXM_O_ACT_CR) + 2 * a;
      const float* fr = md.F(BXM_O_ACT_FR) + 2 * a;
      float gear = md.F(BXM_O_ACT_GEAR)[a];
      float u = fminf(fmaxf(act[a], cr[0]), cr[1]);
      const float* prm = w.at(L.prm) + md.ncon;  // per-env gain, bias_q, bias_qd
      float bias = gear * (q[aqid[a]] * prm[md.nu + a] + qd[aqdid[a]] * prm[2 * md.nu + a]);
      float f = prm[a] * u + bias;
      f = fminf(fmaxf(f, fr[0]), fr[1]);
      force[a] = f * gear;
    }
  }
  // cdd root-to-leaf: dynamics.py:153-165
  const int* lstart = md.I(BXM_O_LEVEL_START);
  const int* llinks = md.I(BXM_O_LEVEL_LINKS);
  const int* parent = md.I(BXM_O_LINK_PARENT);
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  const float* cdofd = w.at(L.cdofd);
  for (int lv = 0; lv < md.nlevel; ++lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      int p = parent[l];
      f3 a = p >= 0 ? ld3(cdd + 6 * p) : mk3(0.f, 0.f, 0.f);
      f3 v = p >= 0 ? ld3(cdd + 6 * p + 3) : -md.g;
      int nd = ltype[l] == 0 ? 6 : ltype[l];
      for (int k = 0; k < nd; ++k) {
        int d = dadr[l] + k;
        a = a + ld3(cdofd + 6 * d) * qd[d];
        v = v + ld3(cdofd + 6 * d + 3) * qd[d];
      }
      st3(cdd + 6 * l, a);
      st3(cdd + 6 * l + 3, v);
    }
    tm.sync();
  }
  // cfrc_flat = cinr * cdd + cd x (cinr * cd): dynamics.py:168-171
  const float* ci = w.at(L.ci);
  const float* cp = w.at(L.cp);
  const float* cd = w.at(L.cd);
  const float* mass = link_mass(md, L, w.b);
  for (int l = tm.lane; l < nl; l += T) {
    f3 p = ld3(cp + 3 * l);
    f3 fa, fv, ga, gv, xa, xv;
    inertia_mul(ci + 9 * l, p, mass[l], ld3(cdd + 6 * l), ld3(cdd + 6 * l + 3), fa, fv);
    f3 cda = ld3(cd + 6 * l), cdv = ld3(cd + 6 * l + 3);
    inertia_mul(ci + 9 * l, p, mass[l], cda, cdv, ga, gv);
    force_cross(cda, cdv, ga, gv, xa, xv);
    st3(cf + 6 * l, fa + xa);
    st3(cf + 6 * l + 3, fv + xv);
  }
  tm.sync();
  // leaf-to-root sum: dynamics.py:174-179
  const int* cstart = md.I(BXM_O_CHILD_START);
  const int* cidx = md.I(BXM_O_CHILD_IDX);
  for (int lv = md.nlevel - 1; lv >= 0; --lv) {
    for (int idx = lstart[lv] + tm.lane; idx < lstart[lv + 1]; idx += T) {
      int l = llinks[idx];
      if (cstart[l] == cstart[l + 1]) continue;
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
  // fluid forces (dynamics.py:198-211 with fluid.py:53-82): per link, the
  // inertia-box drag of its com point's velocity in the inertia frame,
  // rotated back to world, stored with the point's offset from the tree's com
  float* ff = force + al4(md.nu);  // [nl][9]: force ang, force vel, offset
  if (md.fluid) {
    const float* xp = w.at(L.xp);
    const float* xr = w.at(L.xr);
    const float* rc = w.at(L.rc);
    const float* lip = md.F(BXM_O_LI_POS);
    const float* lir = md.F(BXM_O_LI_ROT);
    const float* box = md.F(BXM_O_LI_BOX);
    for (int l = tm.lane; l < nl; l += T) {
      f3 ip;
      q4 ir;
      tf_do(ld3(xp + 3 * l), ld4(xr + 4 * l), ld3(lip + 3 * l), ld4(lir + 4 * l), ip, ir);
      const f3 off = ip - ld3(rc + 3 * l);
      const q4 rt = q4{ir.w, -ir.x, -ir.y, -ir.z};  // quat_inv
      const f3 ca = ld3(cd + 6 * l), cv = ld3(cd + 6 * l + 3);
      const f3 wa = rotate(ca, rt);
      const f3 wv = rotate(cv - cross3(off, ca), rt);
      const f3 b = ld3(box + 3 * l);
      const float diam = (b.x + b.y + b.z) / 3.f;
      const float ang_scale = -kPi * (diam * diam * diam) * md.visc;  // fluid.py:26-34
      const float vel_scale = -3.f * kPi * diam * md.visc;
      f3 fa = ang_scale * wa, fv = vel_scale * wv;
      const float dv = -0.5f * md.dens;  // fluid.py:37-50
      fv = fv + mk3(dv * (b.y * b.z) * fabsf(wv.x) * wv.x, dv * (b.x * b.z) * fabsf(wv.y) * wv.y,
                    dv * (b.x * b.y) * fabsf(wv.z) * wv.z);
      const float b4x = (b.x * b.x) * (b.x * b.x), b4y = (b.y * b.y) * (b.y * b.y),
                  b4z = (b.z * b.z) * (b.z * b.z);
      const float da = -1.f * md.dens;
      fa = fa + mk3(da * (b.x * (b4y + b4z)) * fabsf(wa.x) * wa.x / 64.f,
                    da * (b.y * (b4x + b4z)) * fabsf(wa.y) * wa.y / 64.f,
                    da * (b.z * (b4x + b4y)) * fabsf(wa.z) * wa.z / 64.f);
      st3(ff + 9 * l, rotate(fa, ir));  // fluid.py:80
      st3(ff + 9 * l + 3, rotate(fv, ir));
      st3(ff + 9 * l + 6, off);
    }
    tm.sync();
  }
  // qf_smooth = passive - bias + tau: dynamics.py:182, 190-196, 232-234
  const int* dlink = md.I(BXM_O_DOF_LINK);
  const float* cdof = w.at(L.cdof);
  const float* stiff = dof_stiffness(md, L, w.b);
  const float* damp = dof_damping(md, L, w.b);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  float* qfs = w.at(L.qfs);
  for (int d = tm.lane; d < nv; d += T) {
    int l = dlink[d];
    float bias = dot3(ld3(cdof + 6 * d + 3), ld3(cf + 6 * l + 3)) + dot3(ld3(cdof + 6 * d), ld3(cf + 6 * l));
    float pas = 0.f;
    if (ltype[l] != 0) pas = -q[qadr[l] + (d - dadr[l])] * stiff[d];
    pas = pas - damp[d] * qd[d];
    if (md.fluid) {  // sum over links of point_jacobian(x_i.pos) . force (dynamics.py:206-211)
      const f3 ca = ld3(cdof + 6 * d), cv = ld3(cdof + 6 * d + 3);
      float fl = 0.f;
      for (int k = 0; k < nl; ++k) {
        if (!((md.anc(k) >> d) & 1ull)) continue;  // dof d does not move link k
        const f3 jv = cv - cross3(ld3(ff + 9 * k + 6), ca);
        fl = fl + (dot3(jv, ld3(ff + 9 * k + 3)) + dot3(ca, ld3(ff + 9 * k)));
      }
      pas = pas + fl;
    }
    float tau = 0.f;
    if (has_act)
      for (int a = 0; a < md.nu; ++a)
        if (aqdid[a] == d) tau = tau + force[a];
    qfs[d] = (pas - bias) + tau;
  }
  tm.sync();
}

// ---------------------------------------------------------------------------
// constraint.force: brax/generalized/constraint.py:194-240, with the
// jaxopt.ProjectedGradient (FISTA + backtracking) iteration restated.
// ---------------------------------------------------------------------------
// out = A v (trans: A^T v) for A = J Minv J^T + diag, without forming A; A^T
// differs from A where the carried Newton-Schulz Minv is not symmetric.
template <int T>
__device__ __noinline__ void matvec_A(const int* mw, Ws w, int nrow, const float* v, float* out, float* t1,
                                      float* t2, bool trans = false) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nv = md.nv, ld = L.ldm;
  const float* Minv = w.at(L.Minv);
  const float* rdiag = w.at(L.rdiag);
  for (int d = tm.lane; d < nv; d += T) {  // t1 = J^T v
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int r = 0;
    for (; r + 3 < nrow; r += 4) {
      s0 = fmaf(w.jrow(r)[d], v[r], s0);
      s1 = fmaf(w.jrow(r + 1)[d], v[r + 1], s1);
      s2 = fmaf(w.jrow(r + 2)[d], v[r + 2], s2);
      s3 = fmaf(w.jrow(r + 3)[d], v[r + 3], s3);
    }
    for (; r < nrow; ++r) s0 = fmaf(w.jrow(r)[d], v[r], s0);
    t1[d] = (s0 + s1) + (s2 + s3);
  }
  tm.sync();
  // t2 = Minv t1 (trans: Minv^T t1)
  const int sr = trans ? 1 : ld, sc = trans ? ld : 1;
  for (int d = tm.lane; d < nv; d += T) {
    float s0 = 0.f, s1 = 0.f;
    int k = 0;
    for (; k + 1 < nv; k += 2) {
      s0 = fmaf(Minv[d * sr + k * sc], t1[k], s0);
      s1 = fmaf(Minv[d * sr + (k + 1) * sc], t1[k + 1], s1);
    }
    if (k < nv) s0 = fmaf(Minv[d * sr + k * sc], t1[k], s0);
    t2[d] = s0 + s1;
  }
  tm.sync();
  for (int r = tm.lane; r < nrow; r += T) {  // out = J t2 + diag v
    float s0 = 0.f, s1 = 0.f;
    const float* jr = w.jrow(r);
    int k = 0;
    for (; k + 1 < nv; k += 2) {
      s0 = fmaf(jr[k], t2[k], s0);
      s1 = fmaf(jr[k + 1], t2[k + 1], s1);
    }
    if (k < nv) s0 = fmaf(jr[k], t2[k], s0);
    out[r] = (s0 + s1) + rdiag[r] * v[r];
  }
  tm.sync();
}

// PG tape (reverse pass only) of a solve with `rows` active rows: [0]
// iterations run, [1] rows, then x* (tape_stride(rows) words), then per
// iteration 4 scalars (step, beta) and y, r(y), [z > 0], each
// tape_stride(rows) words.  Both solve paths (explicit A up to
// kMaxExplicitRows rows, implicit above) write the same tape; a model's tape
// buffer holds tape_words(m, pg_iters) words, and a frame snapshot copies
// only the tape_words(rows, iterations) its solve wrote.
__host__ __device__ inline int tape_stride(int rows) { return al4(rows); }
__host__ __device__ inline int tape_head_words(int rows) { return 4 + tape_stride(rows); }
__host__ __device__ inline int tape_iter_words(int rows) { return 4 + 3 * tape_stride(rows); }
__host__ __device__ inline int tape_words(int rows, int iters) {
  return al4(tape_head_words(rows) + iters * tape_iter_words(rows));
}

// Projected gradient with A formed explicitly, in the reference's association:
// W = J Minv, A = W J^T + diag(d), b = W qf_smooth - aref (constraint.py:208-210).
// Used when nrow <= kMaxExplicitRows; each matvec is then one team pass.

// `sym`: Minv is symmetric bit for bit (the exact inverse), so A is built
// from its lower triangle and A^T v is A v; otherwise (the carried
// Newton-Schulz iterate, whose two triangles differ by rounding) every entry
// of A is formed and the gradient A^T r of 0.5 |A x + b|^2 is a column matvec,
// as the reference computes it.
template <int T>
__device__ __noinline__ int pg_explicit(const int* mw, Ws w, int nrow, float* tape, bool sym) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nv = md.nv, ldj = L.ldj, ld = L.ldm, la = explicit_lda(nrow), n4 = al4(nrow) / 4;
  float* A = w.at(L.scr);
  float* b = A + nrow * la;
  float* W = b + al4(nrow);  // J Minv, dead once A and b are formed
  // FISTA iterates and, by linearity of A, their residuals A v + b and
  // gradients A (A v + b): x, y, the trial point nx; rx, ry, rn; gx, gy, gn
  float* x = W;
  float* y = x + al4(nrow);
  float* nx = y + al4(nrow);
  float* rx = nx + al4(nrow);
  float* ry = rx + al4(nrow);
  float* rn = ry + al4(nrow);
  float* gx = rn + al4(nrow);
  float* gy = gx + al4(nrow);
  float* gn = gy + al4(nrow);
  if (bx_scratch<T>(w, scratch_pg_explicit(L, nrow), (gn + al4(nrow) > W + nrow * ld) ? gn + al4(nrow) : W + nrow * ld,
                    nv) ||
      bx_misaligned<T>(w, A, A + la) || bx_misaligned<T>(w, b, x))
    return 0;
  const float* J = w.at(L.J);
  const float* Minv = w.at(L.Minv);
  const float* rdiag = w.at(L.rdiag);
  const float* raref = w.at(L.raref);
  const float* qfs = w.at(L.qfs);
  float* qfc = w.at(L.qfc);
  // cycles spent forming W, A, b and iterating, for the stage profile
  unsigned* pg_cycles = reinterpret_cast<unsigned*>(w.at(L.misc)) + 9;
  const long long t_build = clock64();
  // W = J Minv, lanes over the nrow x nv entries (entry e: row e / nv, column
  // e % nv, walked incrementally); each entry's sum is the same two-chain
  // dot product in the same order as with one lane per column
  {
    int i = 0, k = tm.lane;
    while (k >= nv) {
      k -= nv;
      ++i;
    }
    for (; i < nrow;) {
      float s0 = 0.f, s1 = 0.f;
      int d = 0;
      for (; d + 1 < nv; d += 2) {
        s0 = fmaf(J[i * ldj + d], Minv[d * ld + k], s0);
        s1 = fmaf(J[i * ldj + d + 1], Minv[(d + 1) * ld + k], s1);
      }
      if (d < nv) s0 = fmaf(J[i * ldj + d], Minv[d * ld + k], s0);
      W[i * ld + k] = s0 + s1;
      k += T;
      while (k >= nv) {
        k -= nv;
        ++i;
      }
    }
  }
  tm.sync();
  if (!sym) {  // A = W J^T + diag, every entry (lanes over them)
    for (int e = tm.lane; e < nrow * nrow; e += T) {
      const int i = e / nrow, c = e - i * nrow;
      float s0 = 0.f, s1 = 0.f;
      int k = 0;
      for (; k + 1 < nv; k += 2) {
        s0 = fmaf(W[i * ld + k], J[c * ldj + k], s0);
        s1 = fmaf(W[i * ld + k + 1], J[c * ldj + k + 1], s1);
      }
      if (k < nv) s0 = fmaf(W[i * ld + k], J[c * ldj + k], s0);
      A[i * la + c] = (s0 + s1) + (i == c ? rdiag[i] : 0.f);
    }
    for (int e = tm.lane; e < nrow * (4 * n4 - nrow); e += T) {
      const int r = e / (4 * n4 - nrow);
      A[r * la + nrow + (e - r * (4 * n4 - nrow))] = 0.f;
    }
  } else {  // A = W J^T + diag: the lower triangle (row i, column c <= i), lanes over
     // its entries, mirrored into the upper one, so that A is symmetric bit
     // for bit (J Minv J^T is symmetric) and A^T v is A v
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
      A[i * la + c] = v;
      A[c * la + i] = v;
      c += T;
      while (c > i) {
        c -= i + 1;
        ++i;
      }
    }
    // zero padding: columns nrow .. 4 n4 of every row (the float4 matvecs read them)
    for (int e = tm.lane; e < nrow * (4 * n4 - nrow); e += T) {
      const int r = e / (4 * n4 - nrow);
      A[r * la + nrow + (e - r * (4 * n4 - nrow))] = 0.f;
    }
  }
  for (int c = tm.lane; c < nrow; c += T) {  // b[c] = W[c] qf_smooth - aref[c]
    float s0 = 0.f, s1 = 0.f;
    int k = 0;
    for (; k + 1 < nv; k += 2) {
      s0 = fmaf(W[c * ld + k], qfs[k], s0);
      s1 = fmaf(W[c * ld + k + 1], qfs[k + 1], s1);
    }
    if (k < nv) s0 = fmaf(W[c * ld + k], qfs[k], s0);
    b[c] = (s0 + s1) - raref[c];
  }
  for (int c = nrow + tm.lane; c < 4 * n4; c += T) b[c] = 0.f;  // padding (b is a matvec input)
  tm.sync();
  // W is dead: its words become x, y, ...; every vector's padding up to
  // 4 n4 stays zero (the matvecs read it)
  for (int c = tm.lane; c < 9 * al4(nrow); c += T) x[c] = 0.f;
  tm.sync();
  const long long t_iter = clock64();
  if (tm.lane == 0) pg_cycles[0] += (unsigned)(t_iter - t_build);
  // A v (lanes over rows; 16-byte row and vector loads, even and odd
  // columns in two chains), plus b when `add_b`
  auto matvec = [&](const float* v, float* out, bool add_b) {
    const float4* v4 = reinterpret_cast<const float4*>(v);
    for (int i = tm.lane; i < nrow; i += T) {
      const float4* a4 = reinterpret_cast<const float4*>(A + i * la);
      float s0 = 0.f, s1 = 0.f;
      for (int c = 0; c < n4; ++c) {
        const float4 a = a4[c], u = v4[c];
        s0 = fmaf(a.x, u.x, s0);
        s1 = fmaf(a.y, u.y, s1);
        s0 = fmaf(a.z, u.z, s0);
        s1 = fmaf(a.w, u.w, s1);
      }
      out[i] = add_b ? (s0 + s1) + b[i] : s0 + s1;
    }
    tm.sync();
  };
  // A^T v by columns (lanes over the output entries, consecutive columns)
  auto matvec_t = [&](const float* v, float* out) {
    for (int c = tm.lane; c < nrow; c += T) {
      float s0 = 0.f, s1 = 0.f;
      int i = 0;
      for (; i + 1 < nrow; i += 2) {
        s0 = fmaf(A[i * la + c], v[i], s0);
        s1 = fmaf(A[(i + 1) * la + c], v[i + 1], s1);
      }
      if (i < nrow) s0 = fmaf(A[i * la + c], v[i], s0);
      out[c] = s0 + s1;
    }
    tm.sync();
  };
  auto resid = [&](const float* v, float* out) { matvec(v, out, true); };  // A v + b
  auto grad = [&](const float* v, float* out) {                           // A^T v
    if (sym) {
      matvec(v, out, false);
    } else {
      matvec_t(v, out);
    }
  };
  float t = 1.f, ss = 1.f, err = INFINITY;
  int matvecs = 0;
  int iters = 0;
  const int kA = tape_stride(nrow);
  // x = y = 0: residual b, gradient A b
  for (int i = tm.lane; i < nrow; i += T) {
    rx[i] = b[i];
    ry[i] = b[i];
  }
  tm.sync();
  grad(b, gy);
  matvecs += 1;
  float fy;  // f(y) = |A y + b|^2 / 2 of the current y
  {
    float fs = 0.f;
    for (int i = tm.lane; i < nrow; i += T) {
      gx[i] = gy[i];
      fs += 0.5f * ry[i] * ry[i];
    }
    fy = tm.sum(fs);
  }
  for (int it = 0; it < md.pg_iters; ++it) {
    if (it > 0 && !(err > md.pg_tol)) break;
    float* rec = tape != nullptr ? tape + tape_head_words(nrow) + it * tape_iter_words(nrow) : nullptr;
    if (rec != nullptr)
      for (int i = tm.lane; i < nrow; i += T) {
        rec[4 + i] = y[i];
        rec[4 + kA + i] = ry[i];
      }
    float cur = ss;
    for (int i = tm.lane; i < nrow; i += T) nx[i] = fmaxf(y[i] + (-cur) * gy[i], 0.f);
    tm.sync();
    bool accepted = false;  // rn = A nx + b for the accepted trial point
    for (int ls = 0; ls < md.pg_maxls; ++ls) {
      resid(nx, rn);
      matvecs += 1;
      float fn = 0.f, dv = 0.f, sq = 0.f;
      for (int i = tm.lane; i < nrow; i += T) {
        fn += 0.5f * rn[i] * rn[i];
        float dx = nx[i] - y[i];
        dv += dx * gy[i];
        sq += dx * dx;
      }
      fn = tm.sum(fn);
      dv = tm.sum(dv);
      sq = tm.sum(sq);
      // sq == 0: the trial point is y itself, where the reference evaluates
      // f twice identically and accepts; here fy comes from the momentum
      // recurrence, so the test could see rounding instead of 0
      if (!(cur * (fn - fy) > cur * dv + 0.5f * sq) || sq == 0.f) {
        accepted = true;
        break;
      }
      cur = cur * 0.5f;
      for (int i = tm.lane; i < nrow; i += T) nx[i] = fmaxf(y[i] + (-cur) * gy[i], 0.f);
      tm.sync();
    }
    const float nss = cur <= 1e-6f ? 1.f : cur / 0.5f;
    const float nt = 0.5f * (1.f + sqrtf(1.f + 4.f * t * t));
    const float beta = (t - 1.f) / nt;
    if (rec != nullptr) {
      for (int i = tm.lane; i < nrow; i += T) rec[4 + 2 * kA + i] = (y[i] + (-cur) * gy[i]) > 0.f ? 1.f : 0.f;
      if (tm.lane == 0) {
        rec[0] = cur;
        rec[1] = beta;
      }
    }
    iters = it + 1;
    if (!accepted) {  // the last halving's point has not been evaluated
      resid(nx, rn);
      matvecs += 1;
    }
    grad(rn, gn);
    matvecs += 1;
    // stopping error at nx; then the momentum step, applied to the point, its
    // residual and its gradient alike (A is linear), so that y's residual and
    // gradient cost no matvec
    // (and f at the new y, reduced alongside: the same sum, in the same order,
    // as over the stored residual)
    float es = 0.f, fs = 0.f;
    for (int i = tm.lane; i < nrow; i += T) {
      const float xn = nx[i], r1 = rn[i], g1 = gn[i];
      const float e = fmaxf(xn + (-1.f) * g1, 0.f) - xn;
      es += e * e;
      y[i] = xn + beta * (xn - x[i]);
      const float r2 = r1 + beta * (r1 - rx[i]);
      ry[i] = r2;
      fs += 0.5f * r2 * r2;
      gy[i] = g1 + beta * (g1 - gx[i]);
      x[i] = xn;
      rx[i] = r1;
      gx[i] = g1;
    }
    err = sqrtf(tm.sum(es));
    fy = tm.sum(fs);
    tm.sync();
    t = nt;
    ss = nss;
  }
  for (int d = tm.lane; d < nv; d += T) {  // qf_constraint = J^T x
    float s = 0.f;
    for (int i = 0; i < nrow; ++i) s = fmaf(J[i * ldj + d], x[i], s);
    qfc[d] = s;
  }
  // the solve ran out of iterations with the error above tol
  if (tm.lane == 0 && iters == md.pg_iters && err > md.pg_tol) reinterpret_cast<int*>(w.at(L.misc))[12] += 1;
  if (tape != nullptr) {
    for (int i = tm.lane; i < nrow; i += T) tape[4 + i] = x[i];
    if (tm.lane == 0) {
      tape[0] = (float)iters;
      tape[1] = (float)nrow;
    }
  }
  if (tm.lane == 0) pg_cycles[1] += (unsigned)(clock64() - t_iter);
  tm.sync();
  return matvecs;
}

// `sym`: Minv is the exact (bitwise symmetric) inverse; false for the
// carried Newton-Schulz iterate (see pg_explicit).
template <int T>
__device__ __noinline__ int stage_constraint(const int* mw, Ws w, float* tape, bool sym) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nv = md.nv, ld = L.ldm;
  const int nrow = reinterpret_cast<const int*>(w.at(L.misc))[0];
  float* qfc = w.at(L.qfc);
  if (bx_stop<T>(w)) return 0;
  if (kChecked && (nrow < 0 || nrow > md.m)) {
    w.flag(kBoundsRow);
    return 0;
  }
  if (nrow == 0) {
    for (int d = tm.lane; d < nv; d += T) qfc[d] = 0.f;
    if (tape != nullptr && tm.lane == 0) {
      tape[0] = 0.f;
      tape[1] = 0.f;
    }
    tm.sync();
    return 0;
  }
  if (nrow <= kMaxExplicitRows) return pg_explicit<T>(md.w, w, nrow, tape, sym);
  const int m = md.m;
  const int kA = tape_stride(nrow);
  float* b = w.at(L.scr);
  float* x = b + al4(m);
  float* y = x + al4(m);
  float* gy = y + al4(m);
  float* r = gy + al4(m);
  float* nx = r + al4(m);
  float* gx = nx + al4(m);
  float* ny = gx + al4(m);
  float* t1 = ny + al4(m);
  float* t2 = t1 + al4(nv);
  if (bx_scratch<T>(w, scratch_pg_implicit(L, m, nv), t2 + al4(nv), nv)) return 0;
  const float* Minv = w.at(L.Minv);
  const float* raref = w.at(L.raref);
  const float* qfs = w.at(L.qfs);
  // b = J Minv qf_smooth - aref
  for (int d = tm.lane; d < nv; d += T) {
    float s = 0.f;
    for (int k = 0; k < nv; ++k) s = fmaf(Minv[d * ld + k], qfs[k], s);
    t2[d] = s;
  }
  tm.sync();
  for (int i = tm.lane; i < nrow; i += T) {
    float s = 0.f;
    const float* ji = w.jrow(i);
    for (int k = 0; k < nv; ++k) s = fmaf(ji[k], t2[k], s);
    b[i] = s - raref[i];
    x[i] = 0.f;
    y[i] = 0.f;
  }
  tm.sync();
  float t = 1.f, ss = 1.f, err = INFINITY;
  int matvecs = 0;
  int iters = 0;
  for (int it = 0; it < md.pg_iters; ++it) {
    if (it > 0 && !(err > md.pg_tol)) break;
    // value and gradient at y
    matvec_A<T>(md.w, w, nrow, y, r, t1, t2);
    float fs = 0.f;
    float* rec = tape != nullptr ? tape + tape_head_words(nrow) + it * tape_iter_words(nrow) : nullptr;
    for (int i = tm.lane; i < nrow; i += T) {
      r[i] = r[i] + b[i];
      fs += 0.5f * r[i] * r[i];
      if (rec != nullptr) {
        rec[4 + i] = y[i];
        rec[4 + kA + i] = r[i];
      }
    }
    float fy = tm.sum(fs);
    tm.sync();
    matvec_A<T>(md.w, w, nrow, r, gy, t1, t2, !sym);
    matvecs += 2;
    float cur = ss;
    for (int i = tm.lane; i < nrow; i += T) nx[i] = fmaxf(y[i] + (-cur) * gy[i], 0.f);
    tm.sync();
    bool accepted = false;  // r = A nx for the accepted trial point
    for (int ls = 0; ls < md.pg_maxls; ++ls) {
      matvec_A<T>(md.w, w, nrow, nx, r, t1, t2);
      matvecs += 1;
      float fn = 0.f, dv = 0.f, sq = 0.f;
      for (int i = tm.lane; i < nrow; i += T) {
        float ri = r[i] + b[i];
        fn += 0.5f * ri * ri;
        float dx = nx[i] - y[i];
        dv += dx * gy[i];
        sq += dx * dx;
      }
      fn = tm.sum(fn);
      dv = tm.sum(dv);
      sq = tm.sum(sq);
      bool cond = cur * (fn - fy) > cur * dv + 0.5f * sq;
      if (!cond) {
        accepted = true;
        break;
      }
      cur = cur * 0.5f;
      for (int i = tm.lane; i < nrow; i += T) nx[i] = fmaxf(y[i] + (-cur) * gy[i], 0.f);
      tm.sync();
    }
    float nss = cur <= 1e-6f ? 1.f : cur / 0.5f;
    float nt = 0.5f * (1.f + sqrtf(1.f + 4.f * t * t));
    float beta = (t - 1.f) / nt;
    for (int i = tm.lane; i < nrow; i += T) ny[i] = nx[i] + beta * (nx[i] - x[i]);
    if (rec != nullptr) {
      for (int i = tm.lane; i < nrow; i += T) rec[4 + 2 * kA + i] = (y[i] + (-cur) * gy[i]) > 0.f ? 1.f : 0.f;
      if (tm.lane == 0) {
        rec[0] = cur;
        rec[1] = beta;
      }
    }
    iters = it + 1;
    tm.sync();
    // gradient at the new iterate and the stopping error
    if (!accepted) {  // an accepted trial already left A nx in r
      matvec_A<T>(md.w, w, nrow, nx, r, t1, t2);
      matvecs += 1;
    }
    for (int i = tm.lane; i < nrow; i += T) r[i] = r[i] + b[i];
    tm.sync();
    matvec_A<T>(md.w, w, nrow, r, gx, t1, t2, !sym);
    matvecs += 1;
    float es = 0.f;
    for (int i = tm.lane; i < nrow; i += T) {
      float e = fmaxf(nx[i] + (-1.f) * gx[i], 0.f) - nx[i];
      es += e * e;
      x[i] = nx[i];
      y[i] = ny[i];
    }
    err = sqrtf(tm.sum(es));
    tm.sync();
    t = nt;
    ss = nss;
  }
  // qf_constraint = J^T x
  for (int d = tm.lane; d < nv; d += T) {
    float s = 0.f;
    for (int i = 0; i < nrow; ++i) s = fmaf(w.jrow(i)[d], x[i], s);
    qfc[d] = s;
  }
  if (tm.lane == 0 && iters == md.pg_iters && err > md.pg_tol) reinterpret_cast<int*>(w.at(L.misc))[12] += 1;
  if (tape != nullptr) {
    for (int i = tm.lane; i < nrow; i += T) tape[4 + i] = x[i];
    if (tm.lane == 0) {
      tape[0] = (float)iters;
      tape[1] = (float)nrow;
    }
  }
  tm.sync();
  return matvecs;
}

// ---------------------------------------------------------------------------
// integrator.integrate: brax/generalized/integrator.py:26-84
// ---------------------------------------------------------------------------
template <int T>
__device__ __noinline__ bool stage_integrate(const int* mw, Ws w) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nv = md.nv, ld = L.ldm;
  const float h = md.dt;
  float* qfs = w.at(L.qfs);
  float* qfc = w.at(L.qfc);
  float* qdd = w.at(L.qdd);
  float* v = w.at(L.v1);
  float* qd = w.at(L.qd);
  float* q = w.at(L.q);
  bool ok = true;
  if (bx_stop<T>(w)) return true;
  for (int d = tm.lane; d < nv; d += T) v[d] = qfs[d] + qfc[d];
  tm.sync();
  if (md.ns_iters == 0) {  // (M + diag(damping) dt)^-1: integrator.py:58-62
    float* A = w.at(L.scr);
    if (bx_scratch<T>(w, scratch_integrate(L, nv), A + nv * ld, nv)) return true;
    const float* M = w.at(L.M);
    const float* damp = dof_damping(md, L, w.b);
    for (int idx = tm.lane; idx < nv * nv; idx += T) {
      int i = idx / nv, j = idx - i * nv;
      A[i * ld + j] = M[i * ld + j] + (i == j ? damp[i] * h : 0.f);
    }
    tm.sync();
    ok = cholesky<T>(tm, nv, ld, A);
    // forward / backward substitution on the vector (single lane, nv small)
    if (tm.lane == 0) {
      for (int i = 0; i < nv; ++i) {
        float s = v[i];
        for (int k = 0; k < i; ++k) s -= A[i * ld + k] * qdd[k];
        qdd[i] = s / A[i * ld + i];
      }
      for (int i = nv - 1; i >= 0; --i) {
        float s = qdd[i];
        for (int k = i + 1; k < nv; ++k) s -= A[k * ld + i] * qdd[k];
        qdd[i] = s / A[i * ld + i];
      }
    }
    tm.sync();
  } else {
    const float* Minv = w.at(L.Minv);
    for (int d = tm.lane; d < nv; d += T) {
      float s = 0.f;
      for (int k = 0; k < nv; ++k) s = fmaf(Minv[d * ld + k], v[k], s);
      qdd[d] = s;
    }
    tm.sync();
  }
  for (int d = tm.lane; d < nv; d += T) qd[d] = qd[d] + qdd[d] * h;
  tm.sync();
  const int* ltype = md.I(BXM_O_LINK_TYPE);
  const int* qadr = md.I(BXM_O_LINK_QADR);
  const int* dadr = md.I(BXM_O_LINK_DADR);
  for (int l = tm.lane; l < md.nl; l += T) {
    int typ = ltype[l], qa = qadr[l], da = dadr[l];
    if (typ == 0) {
      q4 rot = ld4(q + qa + 3);
      f3 ang = ld3(qd + da + 3);
      float an = sqrtf(dot3(ang, ang)) + 1e-8f;
      f3 axis = mk3(ang.x / an, ang.y / an, ang.z / an);
      q4 qr = quat_rot_axis(axis, h * an);
      rot = qmul(rot, qr);
      float rn = sqrtf(rot.w * rot.w + rot.x * rot.x + rot.y * rot.y + rot.z * rot.z);
      rot = q4{rot.w / rn, rot.x / rn, rot.y / rn, rot.z / rn};
      f3 pos = ld3(q + qa) + ld3(qd + da) * h;
      st3(q + qa, pos);
      st4(q + qa + 3, rot);
    } else {
      for (int k = 0; k < typ; ++k) q[qa + k] = q[qa + k] + qd[da + k] * h;
    }
  }
  tm.sync();
  return ok;
}

}  // namespace braxg
