// Fused forward + reverse of an n-step rollout (the gradient of a loss on the
// trajectory w.r.t. the actions and the initial state), checkpointed every
// ckpt_every env steps with recompute.  One team of 32 lanes per env; the CTA
// walks the stages in lockstep like the forward kernel.
#pragma once
#include "braxg_adjoint.cuh"
#include "braxg_kernel.cuh"

namespace braxg {



// `sym`: the inverse is the exact (bitwise symmetric) one; false in
// Newton-Schulz mode, where the solve forms every entry of A and takes A^T r.
template <int T, int NVB>
__device__ __forceinline__ void fwd_frame(const int* mw, Ws w, bool active, bool has_act, float* tape, bool& ok,
                                          bool sym = true) {
  if (active) stage_smooth<T>(mw, w, has_act);
  __syncthreads();
  if (active) stage_constraint<T>(mw, w, tape, sym);
  __syncthreads();
  if (active) ok = stage_integrate<T>(mw, w) && ok;
  __syncthreads();
}

// Position terms of the arena's q.  ns_iters 0: the exact inverse of M;
// else the Newton-Schulz update of the arena's (carried) inverse, after
// copying M and that inverse to `rec` (the frame's record, for the reverse)
// and the inverse to `minv_out` (a checkpoint's, n x n) when given.
template <int T, int NVB>
__device__ __forceinline__ bool pos_stage(const int* mw, Ws w, bool active, int ns_iters = 0, float* rec = nullptr,
                                          float* minv_out = nullptr) {
  bool ok = true;
  if (active) stage_fk<T>(mw, w);
  __syncthreads();
  if (active) stage_com<T>(mw, w);
  __syncthreads();
  if (active) stage_crba<T>(mw, w);
  __syncthreads();
  if (ns_iters > 0) {
    if (active) {
      const Model md(mw);
      const Team<T> tm;
      const Layout& L = *w.L;
      const int n = md.nv, ld = L.ldm;
      const float* M = w.at(L.M);
      const float* P = w.at(L.Minv);
      if (rec != nullptr)
        for (int e = tm.lane; e < n * ld; e += T) {
          rec[e] = M[e];
          rec[n * ld + e] = P[e];
        }
      if (minv_out != nullptr)
        for (int e = tm.lane; e < n * n; e += T) {
          const int i = e / n, j = e - i * n;
          minv_out[e] = P[i * ld + j];
        }
      tm.sync();
      stage_inverse<T, NVB>(mw, w, false, ns_iters);
    }
  } else if (active) {
    ok = stage_inverse<T, NVB>(mw, w, true, 0);
  }
  __syncthreads();
  if (active) stage_jacobian<T>(mw, w);
  __syncthreads();
  return ok;
}

template <int T>
__device__ __forceinline__ void copy_vec(const Team<T>& tm, float* dst, const float* src, int n) {
  for (int i = tm.lane; i < n; i += T) dst[i] = src[i];
}

// A frame snapshot is the env's whole forward arena (every stage's values
// after the frame's smooth, constraint and integrate stages) followed by the
// projected-gradient tape; the reverse of that frame restores it instead of
// recomputing the frame.  Of the tape only the words the frame's solve wrote
// are copied (its header gives the iterations and rows), at most
// `tape_cap` words.  All parts are whole float4s (al4 sizes, 16-byte aligned
// arenas and slots).
__device__ __forceinline__ int tape_used(const float* head, int tape_cap) {
  const int iters = max((int)head[0], 0), rows = max((int)head[1], 0);
  return min(tape_words(rows, iters), tape_cap);
}
template <int T>
__device__ __forceinline__ void snap_save(const Team<T>& tm, float* slot, const float* arena, int arena_words,
                                          const float* tape, int tape_cap) {
  float4* d = reinterpret_cast<float4*>(slot);
  const float4* x = reinterpret_cast<const float4*>(arena);
  const float4* t = reinterpret_cast<const float4*>(tape);
  const int used = tape_used(tape, tape_cap);
  for (int i = tm.lane; i < arena_words / 4; i += T) d[i] = x[i];
  for (int i = tm.lane; i < used / 4; i += T) d[arena_words / 4 + i] = t[i];
}
// 16 bytes global -> shared without a register round trip; every copy a lane
// issues is in flight at once until its cp.async.wait_all.
__device__ __forceinline__ void copy16_async(float4* smem_dst, const float4* gmem_src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
// The arena and the tape are in shared memory; the snapshot, the arena and
// the tape start on 16-byte boundaries (the checked build verifies the first
// two and the slot stride).  The caller's team sync makes the copies visible
// to the other lanes.
template <int T>
__device__ __forceinline__ void snap_load(const Team<T>& tm, const float* slot, float* arena, int arena_words,
                                          float* tape, int tape_cap) {
  const float4* d = reinterpret_cast<const float4*>(slot);
  float4* x = reinterpret_cast<float4*>(arena);
  float4* t = reinterpret_cast<float4*>(tape);
  const int used = tape_used(slot + arena_words, tape_cap);
  for (int i = tm.lane; i < arena_words / 4; i += T) copy16_async(x + i, d + i);
  for (int i = tm.lane; i < used / 4; i += T) copy16_async(t + i, d + arena_words / 4 + i);
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <int T, int NVB>
__global__ void __launch_bounds__(256, 1) vjp_kernel(const VjpArgs a) {
  extern __shared__ __align__(16) int smem[];
  for (int i = threadIdx.x; i < a.model_words; i += blockDim.x) smem[i] = a.model[i];
  Layout* sl = reinterpret_cast<Layout*>(smem + al4(a.model_words));
  AdjLayout* sal = reinterpret_cast<AdjLayout*>(smem + al4(a.model_words) + kLayoutWords);
  if (threadIdx.x == 0) {
    const int* w0 = a.model;
    *sl = layout_of(w0);
    *sal = make_adj_layout(w0[BXM_H_NL], w0[BXM_H_NQ], w0[BXM_H_NV], w0[BXM_H_NU], w0[BXM_H_NCON], w0[BXM_H_NLIM],
                           w0[BXM_H_PG_ITERS], a.ns_iters > 0 ? ns_rev_smem_words(w0[BXM_H_NV], NVB) : 0);
  }
  __syncthreads();
  const int* mw = smem;
  const Model md(mw);
  const Team<T> tm;
  const int team = threadIdx.x / T;
  long long env = (long long)blockIdx.x * a.envs_per_cta + team;
  const bool active = env < a.n_env;
  if (!active) env = 0;
  Ws w;
  w.L = sl;
  AWs aw;
  aw.A = sal;
  float* base = reinterpret_cast<float*>(smem + al4(a.model_words) + 2 * kLayoutWords);
  w.b = base + (size_t)team * (sl->total + sal->total);
  aw.b = w.b + sl->total;
  const Layout& L = *sl;
  const AdjLayout& A = *sal;
  const int nq = md.nq, nv = md.nv, nu = md.nu;
  const int S = nq + nv;
  const int SC = a.ckpt_words;  // a checkpoint: q, qd (and the carried inverse in Newton-Schulz mode)
  const bool ns = a.ns_iters > 0;
  const long long n = a.n_env;
  const bool has_act = a.act != nullptr && nu > 0;
  bool ok = true, taped = true;
  Prof pf(a.prof, active && tm.lane == 0);
  const int n_ckpt = (a.n_steps + a.ckpt_every - 1) / a.ckpt_every;
  // the last `resident` segments are taped and snapshotted by the checkpoint
  // pass itself; earlier segments are recomputed into the first block
  const int first_res = n_ckpt - a.resident;
  const int res_s0 = first_res * a.ckpt_every;
  float* tape = aw.at(A.tape);
  const int tape_words = a.snap_words - L.total;
  // ---- set-up (every phase: a reverse-only launch recomputes segments from
  // the checkpoints with the model's parameters) ----
  if (active) {
    if (tm.lane == 0) {  // the solve counter and the checked build's flags
      reinterpret_cast<int*>(w.at(L.misc))[12] = 0;
      reinterpret_cast<int*>(w.at(L.misc))[13] = 0;
    }
    tm.sync();
    if (kChecked)
      for (int i = tm.lane; i < kCanaryWords; i += T) reinterpret_cast<unsigned*>(w.b + L.canary)[i] = kCanary;
    if (kChecked && ((reinterpret_cast<uintptr_t>(w.b) | reinterpret_cast<uintptr_t>(a.snap) |
                      (uintptr_t)(a.snap_words * 4)) & 15u) != 0u)
      w.flag(kBoundsAlign);
    copy_vec<T>(tm, w.at(L.q), a.q0 + env * nq, nq);
    copy_vec<T>(tm, w.at(L.qd), a.qd0 + env * nv, nv);
    load_params<T>(tm, braxg_randomization{}, md, w, env);  // the model's parameters
  }
  tm.sync();
  __syncthreads();
  // ---- forward with checkpoints ----
  if (a.phases & 1) ok = pos_stage<T, NVB>(mw, w, active) && ok;
  for (int s = 0; (a.phases & 1) && s < a.n_steps; ++s) {
    if (active && s % a.ckpt_every == 0) {
      float* c = a.ckpt + ((long long)(s / a.ckpt_every) * n + env) * SC;
      copy_vec<T>(tm, c, w.at(L.q), nq);
      copy_vec<T>(tm, c + nq, w.at(L.qd), nv);
    }
    if (active && has_act) copy_vec<T>(tm, w.at(L.act), a.act + ((long long)s * n + env) * nu, nu);
    tm.sync();
    // resident segments are taped and snapshotted here, so they need no recompute
    const bool snap = s >= res_s0;
    for (int f = 0; f < a.n_frames; ++f) {
      const long long slot = (long long)((s - res_s0) * a.n_frames + f) * n + env;
      if (active && snap) {
        copy_vec<T>(tm, a.seg + slot * S, w.at(L.q), nq);
        copy_vec<T>(tm, a.seg + slot * S + nq, w.at(L.qd), nv);
      }
      tm.sync();
      fwd_frame<T, NVB>(mw, w, active, has_act, snap ? tape : nullptr, ok, !ns);
      if (active && snap) snap_save<T>(tm, a.snap + slot * a.snap_words, w.b, L.total, tape, tape_words);
      // the next frame's position terms; in Newton-Schulz mode its record
      // (when it is snapshotted) and, at a checkpoint's step, the carried
      // inverse the checkpoint restarts from
      float* rec = nullptr;
      float* cmi = nullptr;
      if (ns && active) {
        const int sn = f + 1 < a.n_frames ? s : s + 1, fn = f + 1 < a.n_frames ? f + 1 : 0;
        if (sn >= res_s0 && sn < a.n_steps)
          rec = a.nsrec + ((long long)((sn - res_s0) * a.n_frames + fn) * n + env) * a.ns_rec_words;
        if (fn == 0 && sn < a.n_steps && sn % a.ckpt_every == 0)
          cmi = a.ckpt + ((long long)(sn / a.ckpt_every) * n + env) * SC + S;
      }
      ok = pos_stage<T, NVB>(mw, w, active, a.ns_iters, rec, cmi) && ok;
    }
    if (active && a.traj_q != nullptr) copy_vec<T>(tm, a.traj_q + ((long long)s * n + env) * nq, w.at(L.q), nq);
    if (active && a.traj_qd != nullptr) copy_vec<T>(tm, a.traj_qd + ((long long)s * n + env) * nv, w.at(L.qd), nv);
  }
  pf.mark(BRAXG_PROF_VJP_CHECKPOINT);
  if (!(a.phases & 2)) {  // forward only: the reverse runs in a later launch on this workspace
    if (active && a.status != nullptr && tm.lane == 0)
      a.status[env] = (ok ? 0 : BRAXG_ENV_NOT_SPD) | (w.failed() ? BRAXG_ENV_BOUNDS : 0);
    return;
  }
  // ---- backward ----
  float* qbo = aw.at(A.qbo);
  float* qdbo = aw.at(A.qdbo);
  if (active) {
    for (int i = tm.lane; i < md.nv * L.ldm; i += T) aw.at(A.Minvbc)[i] = 0.f;
    for (int i = tm.lane; i < nq; i += T)
      qbo[i] = a.q_bar ? a.q_bar[((long long)(a.n_steps - 1) * n + env) * nq + i] : 0.f;
    for (int i = tm.lane; i < nv; i += T)
      qdbo[i] = a.qd_bar ? a.qd_bar[((long long)(a.n_steps - 1) * n + env) * nv + i] : 0.f;
  }
  tm.sync();
  for (int sg = n_ckpt - 1; sg >= 0; --sg) {
    const int s0 = sg * a.ckpt_every;
    const int s1 = min(s0 + a.ckpt_every, a.n_steps);
    // frame slots of this segment: resident segments where the checkpoint
    // pass put them, recomputed ones from the first block
    const int base_s = sg >= first_res ? res_s0 : s0;
    if (sg < first_res) {  // recompute the segment, taping and snapshotting every frame
      if (active) {
        const float* c = a.ckpt + ((long long)sg * n + env) * SC;
        copy_vec<T>(tm, w.at(L.q), c, nq);
        copy_vec<T>(tm, w.at(L.qd), c + nq, nv);
        if (ns && s0 > 0)  // the carried inverse the segment's first update starts from
          for (int e = tm.lane; e < md.nv * md.nv; e += T) {
            const int i = e / md.nv, j = e - i * md.nv;
            w.at(L.Minv)[i * L.ldm + j] = c[S + e];
          }
      }
      tm.sync();
      __syncthreads();
      // the rollout's first frame takes the exact inverse (pipeline.init)
      pos_stage<T, NVB>(mw, w, active, s0 > 0 ? a.ns_iters : 0,
                        ns && s0 > 0 && active ? a.nsrec + ((long long)0 * n + env) * a.ns_rec_words : nullptr);
      for (int s = s0; s < s1; ++s) {
        if (active && has_act) copy_vec<T>(tm, w.at(L.act), a.act + ((long long)s * n + env) * nu, nu);
        for (int f = 0; f < a.n_frames; ++f) {
          const long long slot = (long long)((s - base_s) * a.n_frames + f) * n + env;
          if (active) {
            copy_vec<T>(tm, a.seg + slot * S, w.at(L.q), nq);
            copy_vec<T>(tm, a.seg + slot * S + nq, w.at(L.qd), nv);
          }
          tm.sync();
          bool dummy = true;
          fwd_frame<T, NVB>(mw, w, active, has_act, tape, dummy, !ns);
          if (active) snap_save<T>(tm, a.snap + slot * a.snap_words, w.b, L.total, tape, tape_words);
          float* rec = nullptr;
          if (ns && active) {
            const int sn = f + 1 < a.n_frames ? s : s + 1, fn = f + 1 < a.n_frames ? f + 1 : 0;
            if (sn < s1) rec = a.nsrec + ((long long)((sn - base_s) * a.n_frames + fn) * n + env) * a.ns_rec_words;
          }
          pos_stage<T, NVB>(mw, w, active, a.ns_iters, rec);
        }
      }
    }
    pf.mark(BRAXG_PROF_VJP_RECOMPUTE);
    for (int s = s1 - 1; s >= s0; --s) {
      if (active) {
        if (has_act) copy_vec<T>(tm, w.at(L.act), a.act + ((long long)s * n + env) * nu, nu);
        for (int i = tm.lane; i < nu; i += T) aw.at(A.actb)[i] = 0.f;
      }
      tm.sync();
      for (int f = a.n_frames - 1; f >= 0; --f) {
        if (active) {
          const long long slot = (long long)((s - base_s) * a.n_frames + f) * n + env;
          const float* sp = a.seg + slot * S;
          snap_load<T>(tm, a.snap + slot * a.snap_words, w.b, L.total, tape, tape_words);
          copy_vec<T>(tm, aw.at(A.q0), sp, nq);
          copy_vec<T>(tm, aw.at(A.qd0), sp + nq, nv);
          // zero the accumulated adjoints of this step
          for (int i = tm.lane; i < nq; i += T) aw.at(A.qb)[i] = 0.f;
          for (int i = tm.lane; i < nv; i += T) aw.at(A.qdb)[i] = 0.f;
          for (int i = tm.lane; i < 3 * md.nl; i += T) {
            aw.at(A.xpb)[i] = 0.f;
            aw.at(A.cpb)[i] = 0.f;
            aw.at(A.rcb)[i] = 0.f;
          }
          for (int i = tm.lane; i < 4 * md.nl; i += T) aw.at(A.xrb)[i] = 0.f;
          for (int i = tm.lane; i < 9 * md.nl; i += T) aw.at(A.cib)[i] = 0.f;
          for (int i = tm.lane; i < 6 * md.nl; i += T) aw.at(A.cdb)[i] = 0.f;
          for (int i = tm.lane; i < 6 * nv; i += T) {
            aw.at(A.cdofb)[i] = 0.f;
            aw.at(A.cdofdb)[i] = 0.f;
          }
        }
        tm.sync();
        __syncthreads();
        pf.mark(BRAXG_PROF_VJP_RESTORE);
        if (active) rev_integrate<T>(mw, w, aw);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_INTEGRATE);
        if (active) rev_qdd<T>(mw, w, aw);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_QDD);
        if (active) taped = rev_constraint<T>(mw, w, aw, !ns) && taped;
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_CONSTRAINT);
        if (active) rev_smooth<T>(mw, w, aw, has_act);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_SMOOTH);
        if (active) {
          if (ns) {  // the cotangent the next frame's update carried back to this frame's inverse
            float* mib = aw.at(A.Minvb);
            const float* mic = aw.at(A.Minvbc);
            for (int i = tm.lane; i < md.nv * L.ldm; i += T) mib[i] += mic[i];
            tm.sync();
          }
          if (ns && (s > 0 || f > 0)) {
            const long long slot = (long long)((s - base_s) * a.n_frames + f) * n + env;
            rev_ns<T, NVB>(mw, w, aw, a.nsrec + slot * a.ns_rec_words, a.nsscr + env * a.ns_scr_words, a.ns_iters);
          } else {
            rev_inverse<T, NVB>(mw, w, aw);  // the exact inverse (the rollout's first frame: pipeline.init)
          }
        }
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_INVERSE);
        if (active) rev_crba<T>(mw, w, aw);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_CRBA);
        if (active) rev_rows<T>(mw, w, aw);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_ROWS);
        if (active) rev_com<T>(mw, w, aw);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_COM);
        if (active) rev_fk<T>(mw, w, aw);
        __syncthreads();
        pf.mark(BRAXG_PROF_REV_FK);
        if (active) {
          copy_vec<T>(tm, qbo, aw.at(A.qb), nq);
          copy_vec<T>(tm, qdbo, aw.at(A.qdb), nv);
        }
        tm.sync();
      }
      if (active) {
        if (a.act_bar != nullptr) copy_vec<T>(tm, a.act_bar + ((long long)s * n + env) * nu, aw.at(A.actb), nu);
        if (s > 0) {
          for (int i = tm.lane; i < nq; i += T)
            if (a.q_bar) qbo[i] += a.q_bar[((long long)(s - 1) * n + env) * nq + i];
          for (int i = tm.lane; i < nv; i += T)
            if (a.qd_bar) qdbo[i] += a.qd_bar[((long long)(s - 1) * n + env) * nv + i];
        }
      }
      tm.sync();
    }
  }
  if (!active) return;
  if (a.q0_bar != nullptr) copy_vec<T>(tm, a.q0_bar + env * nq, qbo, nq);
  if (a.qd0_bar != nullptr) copy_vec<T>(tm, a.qd0_bar + env * nv, qdbo, nv);
  if (a.status != nullptr && tm.lane == 0) {
    const int st = (ok ? 0 : BRAXG_ENV_NOT_SPD) | (taped ? 0 : BRAXG_ENV_NO_GRADIENT) |
                   (w.failed() ? BRAXG_ENV_BOUNDS : 0);
    a.status[env] = (a.phases & 1) ? st : (a.status[env] | st);  // reverse only: adds to the forward's
  }
}

template <int T, int NVB>
cudaError_t launch_vjp(const VjpArgs& a, int grid, int smem, cudaStream_t st) {
  auto k = vjp_kernel<T, NVB>;
  static SmemOptIn opt_in;
  cudaError_t e = opt_in.ensure(k, [](int* b) {
    *b = kMaxSmemBytes;
    return cudaSuccess;
  });
  if (e != cudaSuccess) return e;
  k<<<grid, a.envs_per_cta * T, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace braxg
