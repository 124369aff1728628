// The fused step kernel: loads one env per team, runs n_steps x n_frames
// pipeline steps (brax/generalized/pipeline.py:64-94) and writes the State.
#pragma once
#include "braxg_launch.h"
#include "braxg_step.cuh"

namespace braxg {

template <int T>
__device__ void load_vec(const Team<T>& tm, float* dst, const float* src, int n) {
  for (int i = tm.lane; i < n; i += T) dst[i] = src[i];
}
template <int T>
__device__ void store_vec(const Team<T>& tm, float* dst, const float* src, int n) {
  if (dst == nullptr) return;
  for (int i = tm.lane; i < n; i += T) dst[i] = src[i];
}
template <int T>
__device__ void store_mat(const Team<T>& tm, float* dst, const float* src, int n, int ld) {
  if (dst == nullptr) return;
  for (int idx = tm.lane; idx < n * n; idx += T) {
    int i = idx / n, j = idx - i * n;
    dst[idx] = src[i * ld + j];
  }
}

// The env's copy of the parameters per-env randomisation may override
// (contact friction, actuator gain / bias_q / bias_qd): the [n, k] rows of the
// randomisation arrays where given, else the model's values.
template <int T>
__device__ __forceinline__ void load_params(const Team<T>& tm, const braxg_randomization& dr, const Model& md, Ws w,
                                            long long env) {
  float* p = w.at(w.L->prm);
  const int nc = md.ncon, nu = md.nu;
  for (int i = tm.lane; i < nc; i += T) p[i] = dr.friction ? dr.friction[env * nc + i] : md.F(BXM_O_CON_FRIC)[i];
  for (int i = tm.lane; i < nu; i += T) {
    p[nc + i] = dr.act_gain ? dr.act_gain[env * nu + i] : md.F(BXM_O_ACT_GAIN)[i];
    p[nc + nu + i] = dr.act_bias_q ? dr.act_bias_q[env * nu + i] : md.F(BXM_O_ACT_BQ)[i];
    p[nc + 2 * nu + i] = dr.act_bias_qd ? dr.act_bias_qd[env * nu + i] : md.F(BXM_O_ACT_BQD)[i];
  }
  if (w.L->dprm >= 0) {  // dynamics parameters: link mass, inertia; dof armature, damping, stiffness
    float* d = w.at(w.L->dprm);
    const int nl = md.nl, nv = md.nv;
    for (int i = tm.lane; i < nl; i += T) d[i] = dr.link_mass ? dr.link_mass[env * nl + i] : md.F(BXM_O_LI_MASS)[i];
    for (int i = tm.lane; i < 9 * nl; i += T)
      d[nl + i] = dr.link_inertia ? dr.link_inertia[env * 9 * nl + i] : md.F(BXM_O_LI_I)[i];
    for (int i = tm.lane; i < nv; i += T) {
      d[10 * nl + i] = dr.dof_armature ? dr.dof_armature[env * nv + i] : md.F(BXM_O_D_ARM)[i];
      d[10 * nl + nv + i] = dr.dof_damping ? dr.dof_damping[env * nv + i] : md.F(BXM_O_D_DAMP)[i];
      d[10 * nl + 2 * nv + i] = dr.dof_stiffness ? dr.dof_stiffness[env * nv + i] : md.F(BXM_O_D_STIFF)[i];
    }
  }
}

// Whether an env's arena, just restored from the input state's cache, holds
// the position terms of exactly this call's input: q, qd (and, when the
// inverse is carried, mass_mx_inv) and the per-env parameters equal the cached
// ones bit for bit (team-uniform).
template <int T>
__device__ __forceinline__ bool cache_matches(const StepArgs& a, const EnvBase& B, const int* mw, Ws w, long long env,
                                           bool carried_minv) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nq = md.nq, nv = md.nv, nc = md.ncon, nu = md.nu, ld = L.ldm;
  auto same = [](float x, float y) { return __float_as_uint(x) == __float_as_uint(y); };
  bool eq = true;
  for (int i = tm.lane; i < nq; i += T) eq = eq && same(w.at(L.q)[i], a.q_in[B.q + env * nq + i]);
  for (int i = tm.lane; i < nv; i += T) eq = eq && same(w.at(L.qd)[i], a.qd_in[B.v + env * nv + i]);
  if (carried_minv)
    for (int idx = tm.lane; idx < nv * nv; idx += T) {
      int i = idx / nv, j = idx - i * nv;
      eq = eq && same(w.at(L.Minv)[i * ld + j], a.minv_in[B.vv + env * nv * nv + idx]);
    }
  const float* p = w.at(L.prm);
  const braxg_randomization& dr = a.dr;
  for (int i = tm.lane; i < nc; i += T)
    eq = eq && same(p[i], dr.friction ? dr.friction[env * nc + i] : md.F(BXM_O_CON_FRIC)[i]);
  for (int i = tm.lane; i < nu; i += T) {
    eq = eq && same(p[nc + i], dr.act_gain ? dr.act_gain[env * nu + i] : md.F(BXM_O_ACT_GAIN)[i]);
    eq = eq && same(p[nc + nu + i], dr.act_bias_q ? dr.act_bias_q[env * nu + i] : md.F(BXM_O_ACT_BQ)[i]);
    eq = eq && same(p[nc + 2 * nu + i], dr.act_bias_qd ? dr.act_bias_qd[env * nu + i] : md.F(BXM_O_ACT_BQD)[i]);
  }
  if (L.dprm >= 0) {
    const float* d = w.at(L.dprm);
    const int nl = md.nl;
    for (int i = tm.lane; i < nl; i += T)
      eq = eq && same(d[i], dr.link_mass ? dr.link_mass[env * nl + i] : md.F(BXM_O_LI_MASS)[i]);
    for (int i = tm.lane; i < 9 * nl; i += T)
      eq = eq && same(d[nl + i], dr.link_inertia ? dr.link_inertia[env * 9 * nl + i] : md.F(BXM_O_LI_I)[i]);
    for (int i = tm.lane; i < nv; i += T) {
      eq = eq && same(d[10 * nl + i], dr.dof_armature ? dr.dof_armature[env * nv + i] : md.F(BXM_O_D_ARM)[i]);
      eq = eq && same(d[10 * nl + nv + i], dr.dof_damping ? dr.dof_damping[env * nv + i] : md.F(BXM_O_D_DAMP)[i]);
      eq = eq && same(d[10 * nl + 2 * nv + i],
                      dr.dof_stiffness ? dr.dof_stiffness[env * nv + i] : md.F(BXM_O_D_STIFF)[i]);
    }
  }
  return tm.all(eq);
}

template <int T>
__device__ __forceinline__ void copy_arena(const Team<T>& tm, float* dst, const float* src, int words) {
  float4* d = reinterpret_cast<float4*>(dst);
  const float4* s = reinterpret_cast<const float4*>(src);
  for (int i = tm.lane; i < words / 4; i += T) d[i] = s[i];
}
// copy_arena from global into shared memory as cp.async 16-byte copies, all in
// flight at once, waited for before it returns (the caller's team sync makes
// them visible to the other lanes)
template <int T>
__device__ __forceinline__ void copy_arena_to_shared(const Team<T>& tm, float* dst, const float* src, int words) {
  for (int i = tm.lane; i < words / 4; i += T) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + 4 * i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + 4 * i) : "memory");
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Copies the words of an arena that hold position-level terms: everything
// before the scratch region, the mass matrix (in scratch unless the
// integrator owns it) and the active overflow Jacobian rows.  Those rows are
// copied from `ovf_src` to `ovf_dst` (the arena's scratch end, or the env's
// cache slots when they live there; no copy when the two are the same).
// The active row count is read from `arena` (the destination on a restore,
// the source on a store) once the part before scratch is there, and clamped
// to the model's row count.
// kRestore: `dst` is the env's arena in shared memory and `src` its global
// cache slot.
template <int T, bool kRestore>
__device__ __forceinline__ void copy_position_terms(const Team<T>& tm, float* dst, const float* src, const Layout& L,
                                                    int nv, int m, const float* arena, float* ovf_dst,
                                                    const float* ovf_src) {
  if (kRestore)
    copy_arena_to_shared<T>(tm, dst, src, L.scr);
  else
    copy_arena<T>(tm, dst, src, L.scr);
  tm.sync();
  const int nrow = min(max(reinterpret_cast<const int*>(arena + L.misc)[0], 0), m);
  if (L.M >= L.scr) {
    if (kRestore)
      copy_arena_to_shared<T>(tm, dst + L.M, src + L.M, al4(nv * L.ldm));
    else
      copy_arena<T>(tm, dst + L.M, src + L.M, al4(nv * L.ldm));
  }
  const int novf = nrow - L.jcap;
  if (novf > 0 && ovf_dst != ovf_src) {
    const int o0 = L.jovf & ~3, o1 = al4(L.jovf + novf * L.ldj);
    copy_arena<T>(tm, ovf_dst + o0, ovf_src + o0, o1 - o0);
  }
}

// Tag of a cached arena (misc[11]): the team width that computed it (lane
// reductions make the terms depend on it bit for bit), the arena layout
// (where its overflow Jacobian rows live, whether it holds per-env dynamics
// parameters), and whether its mass_mx_inv is the exact inverse of its mass
// matrix.  An env whose launch flagged a non-finite value stores tag 0,
// which no launch accepts.
template <int T>
__device__ __forceinline__ int cache_tag(const Layout& L, bool exact_minv) {
  return (L.dprm >= 0 ? 256 : 0) + 4 * T + (L.ovf_g ? 2 : 0) + (exact_minv ? 1 : 0);
}

// Restores the env's arena from the input state's cache; true if it applies.
// In exact-inverse mode the cached mass_mx_inv must be exact; in
// Newton-Schulz mode it must equal the carried one.
template <int T>
__device__ __noinline__ bool restore_cache(const StepArgs& a, const EnvBase& B, const int* mw, Ws w, long long env,
                                           bool exact) {
  const Team<T> tm;
  const Model md(mw);
  const float* slot = a.cache_in + (B.env + env) * a.cache_stride;
  // checked build: a misaligned slot is not used (and is flagged by the caller)
  if (kChecked && ((reinterpret_cast<uintptr_t>(slot) | reinterpret_cast<uintptr_t>(w.b)) & 15u) != 0u) return false;
  // overflow rows: into the arena, or from the input's cache slot to the output's
  copy_position_terms<T, true>(tm, w.b, slot, *w.L, md.nv, md.m, w.b, w.L->ovf_g ? w.g : w.b, slot);
  tm.sync();
  const int tag = reinterpret_cast<const int*>(w.at(w.L->misc))[11];
  const int want = cache_tag<T>(*w.L, true);
  const bool tag_ok = exact ? tag == want : (tag >> 1) == (want >> 1);
  return cache_matches<T>(a, B, mw, w, env, !exact) && tag_ok;
}

// Stores the env's arena (the output state's position terms) into its cache.
template <int T>
__device__ __noinline__ void store_cache(const StepArgs& a, const EnvBase& B, const int* mw, Ws w, long long env,
                                        bool exact, bool ok) {
  const Team<T> tm;
  const Model md(mw);
  tm.sync();
  if (tm.lane == 0) reinterpret_cast<int*>(w.at(w.L->misc))[11] = ok ? cache_tag<T>(*w.L, exact) : 0;
  tm.sync();
  float* slot = a.out.cache + (B.env + env) * a.cache_stride;
  if (bx_misaligned<T>(w, slot, w.b)) return;
  // overflow rows: from the arena's scratch end, or already in this slot
  copy_position_terms<T, false>(tm, slot, w.b, *w.L, md.nv, md.m, w.b, slot, w.L->ovf_g ? slot : w.b);
}

// Per-stage cycle accumulation (only when a profile buffer is passed): lane 0
// of each team adds the clock64 delta of every stage straight into the buffer.
struct Prof {
  unsigned long long* buf;  // null unless profiling; set only on lane 0 of each team
  long long t;
  __device__ Prof(unsigned long long* b, bool lead) : buf(lead ? b : nullptr), t(0) {
    if (buf != nullptr) t = clock64();
  }
  __device__ __forceinline__ void mark(int slot) {
    if (buf == nullptr) return;
    long long now = clock64();
    atomicAdd(buf + slot, (unsigned long long)(now - t));
    t = now;
  }
  __device__ __forceinline__ void count(int slot, unsigned long long v) {
    if (buf != nullptr) atomicAdd(buf + slot, v);
  }
};

// All teams of a CTA walk the stages in lockstep (a CTA barrier after every
// stage), so the warps of an SM execute the same stage's code at the same time
// and the instruction working set is one or two stages, not the whole kernel.
template <int T, int NVB>
__device__ __forceinline__ bool position_stage(const int* mw, Ws w, bool active, bool exact, int iters, Prof& pf) {
  bool ok = true;
  if (active) stage_fk<T>(mw, w);
  __syncthreads();
  pf.mark(BRAXG_PROF_FK);
  if (active) stage_com<T>(mw, w);
  __syncthreads();
  pf.mark(BRAXG_PROF_COM);
  if (active) stage_crba<T>(mw, w);
  __syncthreads();
  pf.mark(BRAXG_PROF_CRBA);
  if (active) ok = stage_inverse<T, NVB>(mw, w, exact, iters);
  __syncthreads();
  pf.mark(BRAXG_PROF_INVERSE);
  if (active) stage_jacobian<T>(mw, w);
  __syncthreads();
  pf.mark(BRAXG_PROF_JACOBIAN);
  if (active) pf.count(BRAXG_PROF_ROWS, (unsigned long long)reinterpret_cast<const int*>(w.at(w.L->misc))[0]);
  return ok;
}

// Writes the State outputs of one env (out-of-line: runs once per launch).
template <int T>
__device__ __noinline__ void write_outputs(const StepArgs& a, const EnvBase& B, const int* mw, Ws w, long long env,
                                           bool ok) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nq = md.nq, nv = md.nv, nl = md.nl, ld = L.ldm;
  // outputs
  const braxg_state& o = a.out;
  store_vec<T>(tm, o.q ? o.q + B.q + env * nq : nullptr, w.at(L.q), nq);
  store_vec<T>(tm, o.qd ? o.qd + B.v + env * nv : nullptr, w.at(L.qd), nv);
  store_mat<T>(tm, o.mass_mx_inv ? o.mass_mx_inv + B.vv + env * nv * nv : nullptr, w.at(L.Minv), nv, ld);
  store_mat<T>(tm, o.mass_mx ? o.mass_mx + B.vv + env * nv * nv : nullptr, w.at(L.M), nv, ld);
  store_vec<T>(tm, o.x_pos ? o.x_pos + 3 * B.l + env * nl * 3 : nullptr, w.at(L.xp), 3 * nl);
  store_vec<T>(tm, o.x_rot ? o.x_rot + 4 * B.l + env * nl * 4 : nullptr, w.at(L.xr), 4 * nl);
  store_vec<T>(tm, o.xd_ang ? o.xd_ang + 3 * B.l + env * nl * 3 : nullptr, w.at(L.xa), 3 * nl);
  store_vec<T>(tm, o.xd_vel ? o.xd_vel + 3 * B.l + env * nl * 3 : nullptr, w.at(L.xv), 3 * nl);
  store_vec<T>(tm, o.qf_smooth ? o.qf_smooth + B.v + env * nv : nullptr, w.at(L.qfs), nv);
  store_vec<T>(tm, o.qf_constraint ? o.qf_constraint + B.v + env * nv : nullptr, w.at(L.qfc), nv);
  store_vec<T>(tm, o.qdd ? o.qdd + B.v + env * nv : nullptr, w.at(L.qdd), nv);
  store_vec<T>(tm, o.root_com ? o.root_com + 3 * B.l + env * nl * 3 : nullptr, w.at(L.rc), 3 * nl);
  store_vec<T>(tm, o.cinr_pos ? o.cinr_pos + 3 * B.l + env * nl * 3 : nullptr, w.at(L.cp), 3 * nl);
  store_vec<T>(tm, o.cinr_i ? o.cinr_i + 9 * B.l + env * nl * 9 : nullptr, w.at(L.ci), 9 * nl);
  store_vec<T>(tm, o.cd ? o.cd + 6 * B.l + env * nl * 6 : nullptr, w.at(L.cd), 6 * nl);
  store_vec<T>(tm, o.cdof ? o.cdof + 6 * B.v + env * nv * 6 : nullptr, w.at(L.cdof), 6 * nv);
  store_vec<T>(tm, o.cdofd ? o.cdofd + 6 * B.v + env * nv * 6 : nullptr, w.at(L.cdofd), 6 * nv);
  if (o.cinr_rot != nullptr) {  // cinr.transform.rot = x_i.rot
    for (int l = tm.lane; l < nl; l += T) {
      f3 op;
      q4 orr;
      tf_do(ld3(w.at(L.xp) + 3 * l), ld4(w.at(L.xr) + 4 * l), ld3(md.F(BXM_O_LI_POS) + 3 * l),
            ld4(md.F(BXM_O_LI_ROT) + 4 * l), op, orr);
      st4(o.cinr_rot + 4 * B.l + (env * nl + l) * 4, orr);
    }
  }
  if (o.con_jac != nullptr || o.con_diag != nullptr || o.con_aref != nullptr) {
    const int m = md.m;
    const int nrow = reinterpret_cast<const int*>(w.at(L.misc))[0];
    const int* rmap = reinterpret_cast<const int*>(w.at(L.rmap));
    int* inv = reinterpret_cast<int*>(w.at(L.scr));
    if (bx_scratch<T>(w, scratch_outputs(L, m, md.ncon), w.at(L.scr) + m, nv)) return;
    for (int r = tm.lane; r < m; r += T) inv[r] = -1;
    tm.sync();
    for (int r = tm.lane; r < nrow; r += T) inv[rmap[r]] = r;
    tm.sync();
    if (o.con_jac != nullptr) {
      for (long long idx = tm.lane; idx < (long long)m * nv; idx += T) {
        int r = (int)(idx / nv), d = (int)(idx - (long long)r * nv);
        int c = inv[r];
        o.con_jac[B.mv + env * m * nv + idx] = c >= 0 ? w.jrow(c)[d] : 0.f;
      }
    }
    for (int r = tm.lane; r < m; r += T) {
      int c = inv[r];
      if (o.con_diag != nullptr) o.con_diag[B.m + env * m + r] = c >= 0 ? w.at(L.rdiag)[c] : 0.f;
      if (o.con_aref != nullptr) o.con_aref[B.m + env * m + r] = c >= 0 ? w.at(L.raref)[c] : 0.f;
    }
  }
  if (o.status != nullptr) {
    bool fin = true;
    for (int i = tm.lane; i < nq; i += T) fin = fin && isfinite(w.at(L.q)[i]);
    for (int i = tm.lane; i < nv; i += T) fin = fin && isfinite(w.at(L.qd)[i]);
    fin = tm.all(fin);
    const bool bounds = w.failed();
    if (tm.lane == 0)
      o.status[B.env + env] =
          (fin ? 0 : BRAXG_ENV_NONFINITE) | (ok ? 0 : BRAXG_ENV_NOT_SPD) | (bounds ? BRAXG_ENV_BOUNDS : 0);
  }
  if (o.solver_maxiter != nullptr && tm.lane == 0)
    o.solver_maxiter[B.env + env] = reinterpret_cast<const int*>(w.at(L.misc))[12];
  if ((o.contact_dist != nullptr || o.contact_pos != nullptr || o.contact_frame != nullptr) && md.ncon > 0) {
    // contact.get(sys, state.x) of the output state (brax/contact.py:28-67),
    // recomputed from x into scratch (free once the outputs above are read)
    const int nc = md.ncon;
    float* dist = w.at(L.scr);
    float* cpos = dist + al4(nc);
    float* frame = cpos + al4(3 * nc);
    tm.sync();
    if (bx_scratch<T>(w, scratch_outputs(L, md.m, nc), frame + 9 * nc, nv)) return;
    stage_contacts<T>(md.w, w, dist, cpos, frame);
    const long long e = B.env + env;
    store_vec<T>(tm, o.contact_dist ? o.contact_dist + e * nc : nullptr, dist, nc);
    store_vec<T>(tm, o.contact_pos ? o.contact_pos + e * nc * 3 : nullptr, cpos, 3 * nc);
    store_vec<T>(tm, o.contact_frame ? o.contact_frame + e * nc * 9 : nullptr, frame, 9 * nc);
  }
}

// The locomotion task after one env step (brax/envs/ant.py:233-279): every
// lane of the team computes the same scalars from shared memory, so the
// results are team-uniform.  pos0 is the torso (link 0) position before the
// env step, dt the env step's duration (PipelineEnv.dt = n_frames x timestep).
struct TaskOut {
  float reward, done, met[BRAXG_M_COUNT];
};

template <int T>
__device__ __forceinline__ TaskOut task_reward(const braxg_task& k, const Model& md, Ws w, f3 pos0, float dt,
                                               bool has_act) {
  const Layout& L = *w.L;
  const f3 p = ld3(w.at(L.xp));
  const f3 vel = mk3((p.x - pos0.x) / dt, (p.y - pos0.y) / dt, (p.z - pos0.z) / dt);
  float healthy = p.z < k.healthy_z_min ? 0.f : 1.f;
  healthy = p.z > k.healthy_z_max ? 0.f : healthy;
  const float survive = k.terminate_when_unhealthy ? k.healthy_reward : k.healthy_reward * healthy;
  float sq = 0.f;
  if (has_act)
    for (int i = 0; i < md.nu; ++i) sq += w.at(L.act)[i] * w.at(L.act)[i];
  const float ctrl = k.ctrl_cost_weight * sq;
  TaskOut o;
  o.reward = vel.x + survive - ctrl - 0.f;
  o.done = k.terminate_when_unhealthy ? 1.f - healthy : 0.f;
  const float dist2 = dot3(p, p);
  o.met[BRAXG_M_REWARD_FORWARD] = vel.x;
  o.met[BRAXG_M_REWARD_SURVIVE] = survive;
  o.met[BRAXG_M_REWARD_CTRL] = -ctrl;
  o.met[BRAXG_M_REWARD_CONTACT] = -0.f;
  o.met[BRAXG_M_X_POSITION] = p.x;
  o.met[BRAXG_M_Y_POSITION] = p.y;
  o.met[BRAXG_M_DISTANCE_FROM_ORIGIN] = dist2 > 0.f ? sqrtf(dist2) : 0.f;  // math.safe_norm
  o.met[BRAXG_M_X_VELOCITY] = vel.x;
  o.met[BRAXG_M_Y_VELOCITY] = vel.y;
  o.met[BRAXG_M_FORWARD_REWARD] = vel.x;
  return o;
}

// The fused env step's per-env bookkeeping, out of line so that the step
// loop's register allocation does not carry it.  State in the arena's misc
// words: [2..4] torso position before the env step, [5] reward sum, [6]
// episode steps, [7] done of the previous env step, [8] the task's done.
template <int T>
__device__ __noinline__ void task_begin(const StepArgs& a, Ws w, long long ei, bool first) {
  float* misc = w.at(w.L->misc);
  if (Team<T>().lane == 0) {
    if (first) {
      misc[6] = a.io.steps[ei];
      misc[7] = a.io.last_done[ei];
    }
    if (misc[7] != 0.f) misc[6] = 0.f;  // AutoResetWrapper: a new episode
    misc[5] = 0.f;
  }
}

template <int T>
__device__ __noinline__ void task_mark(Ws w) {  // torso position before the env step
  float* misc = w.at(w.L->misc);
  if (Team<T>().lane == 0) st3(misc + 2, ld3(w.at(w.L->xp)));
}

template <int T>
__device__ __noinline__ void task_after_rep(const StepArgs& a, const int* mw, Ws w, long long ei, bool last,
                                            float env_dt, bool has_act) {
  float* misc = w.at(w.L->misc);
  if (Team<T>().lane != 0) return;
  const Model md(mw);
  const TaskOut t = task_reward<T>(a.task, md, w, ld3(misc + 2), env_dt, has_act);
  misc[5] += t.reward;
  misc[8] = t.done;
  if (last && a.io.metrics != nullptr) {
#pragma unroll
    for (int i = 0; i < BRAXG_M_COUNT; ++i) a.io.metrics[ei * BRAXG_M_COUNT + i] = t.met[i];
  }
}

// EpisodeWrapper's step count and truncation, the outputs of the env step and
// AutoResetWrapper's return to the episode's first state; true if reset.
template <int T>
__device__ __noinline__ bool task_end(const StepArgs& a, const int* mw, Ws w, const EnvBase& B, long long env,
                                      int s, int reps, bool exact_mode) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  float* misc = w.at(L.misc);
  const long long ei = B.env + env;
  if (tm.lane == 0) {
    const float ep = misc[6] + (float)reps;
    const bool over = ep >= (float)a.task.episode_length;
    const float done = over ? 1.f : misc[8];
    a.io.reward[s * a.env_step_stride + ei] = misc[5];
    if (a.io.done != nullptr) a.io.done[s * a.env_step_stride + ei] = done;
    if (s == a.n_steps - 1) a.io.truncation[ei] = over ? 1.f - misc[8] : 0.f;
    misc[6] = ep;
    misc[7] = done;
  }
  tm.sync();
  const bool reset = a.task.auto_reset && misc[7] != 0.f;
  if (reset) {  // back to the episode's first state
    const int nq = md.nq, nv = md.nv, ld = L.ldm;
    load_vec<T>(tm, w.at(L.q), a.io.first_q + B.q + env * nq, nq);
    load_vec<T>(tm, w.at(L.qd), a.io.first_qd + B.v + env * nv, nv);
    if (!exact_mode) {
      const float* src = a.io.first_mass_mx_inv + B.vv + env * nv * nv;
      for (int idx = tm.lane; idx < nv * nv; idx += T) {
        int i = idx / nv, j = idx - i * nv;
        w.at(L.Minv)[i * ld + j] = src[idx];
      }
    }
  }
  tm.sync();
  return reset;
}

// obs of the (post-reset) final state and the wrappers' carried state.
template <int T>
__device__ __noinline__ void task_outputs(const StepArgs& a, const int* mw, Ws w, long long ei) {
  const Model md(mw);
  const Team<T> tm;
  const Layout& L = *w.L;
  const int nq = md.nq, nv = md.nv;
  const int ox = a.task.exclude_current_positions ? 2 : 0, osz = nq - ox + nv;
  float* obs = a.io.obs + ei * osz;
  for (int i = tm.lane; i < nq - ox; i += T) obs[i] = w.at(L.q)[ox + i];
  for (int i = tm.lane; i < nv; i += T) obs[nq - ox + i] = w.at(L.qd)[i];
  if (tm.lane == 0) {
    a.io.steps[ei] = w.at(L.misc)[6];
    a.io.last_done[ei] = w.at(L.misc)[7];
  }
}

// One env per team for n_steps x n_frames pipeline steps: load, step, write.
// `arena` is the first per-env shared-memory arena of the CTA; B offsets the
// env's rows in the (flat) global arrays.  Teams without an env (`active`
// false) still take every CTA barrier and return before the outputs.
template <int T, int NVB, bool TASK = false>
__device__ __forceinline__ void run_team(const StepArgs& a, const EnvBase& B, const int* smem, const Layout* sl,
                                         float* arena, int team, long long env, bool active, int n_frames) {
  const Model md(smem);
  const Team<T> tm;
  Ws w;
  w.L = sl;
  w.b = arena + (size_t)team * w.L->total;
  if (sl->ovf_g) w.g = a.out.cache + (B.env + env) * a.cache_stride;
  const Layout& L = *w.L;
  if (kChecked && active)
    for (int i = tm.lane; i < kCanaryWords; i += T) reinterpret_cast<unsigned*>(w.b + L.canary)[i] = kCanary;
  const int nq = md.nq, nv = md.nv, nu = md.nu, ld = L.ldm;
  Prof pf(a.prof, active && tm.lane == 0);

  const bool exact = a.exact_inverse || a.init || md.ns_iters == 0;
  // the input state's cached position terms, where they still apply
  bool cached = false;
  if (active && !a.init && a.cache_in != nullptr) cached = restore_cache<T>(a, B, smem, w, env, exact);
  if (active) {
    load_vec<T>(tm, w.at(L.q), a.q_in + B.q + env * nq, nq);
    load_vec<T>(tm, w.at(L.qd), a.qd_in + B.v + env * nv, nv);
    load_params<T>(tm, a.dr, md, w, env);
  }
  if (active && !exact) {
    const float* src = a.minv_in + B.vv + env * nv * nv;
    for (int idx = tm.lane; idx < nv * nv; idx += T) {
      int i = idx / nv, j = idx - i * nv;
      w.at(L.Minv)[i * ld + j] = src[idx];
    }
  }
  // teams without an env may have no arena slot (batch items narrower than
  // the block): every arena access below is behind `active`
  if (active && tm.lane == 0) {
    int* mi = reinterpret_cast<int*>(w.at(L.misc));
    mi[1] = mi[9] = mi[10] = mi[12] = mi[13] = 0;
    if (kChecked && !a.init && a.cache_in != nullptr &&
        ((reinterpret_cast<uintptr_t>(a.cache_in + (B.env + env) * a.cache_stride) | reinterpret_cast<uintptr_t>(w.b)) &
         15u) != 0u)
      mi[13] |= (int)kBoundsAlign;
  }
  tm.sync();
  pf.mark(BRAXG_PROF_IO);
  // position terms of the input state (envs that restored them from the
  // cache only take the stage's CTA barriers)
  bool ok = position_stage<T, NVB>(smem, w, active && !cached, exact, 0, pf);
  const long long ei = B.env + env;
  if (a.init) {
    for (int d = tm.lane; active && d < nv; d += T) {
      w.at(L.qfs)[d] = 0.f;
      w.at(L.qfc)[d] = 0.f;
      w.at(L.qdd)[d] = 0.f;
    }
    tm.sync();
  } else {
    const bool exact_mode = a.exact_inverse || md.ns_iters == 0;
    const int reps = TASK ? max(1, a.task.action_repeat) : 1;
    const float env_dt = (float)n_frames * md.dt;
    for (int s = 0; s < a.n_steps; ++s) {
      const bool has_act = a.act != nullptr && nu > 0;
      if (has_act && active) load_vec<T>(tm, w.at(L.act), a.act + s * a.act_step_stride + B.u + env * nu, nu);
      if (TASK && active) task_begin<T>(a, w, ei, s == 0);
      tm.sync();
      for (int r = 0; r < reps; ++r) {  // EpisodeWrapper's action repeat
        if (TASK && active) task_mark<T>(w);
        for (int f = 0; f < n_frames; ++f) {
          if (active) stage_smooth<T>(smem, w, has_act);
          __syncthreads();
          pf.mark(BRAXG_PROF_SMOOTH);
          int mvs = 0;
          if (active) mvs = stage_constraint<T>(smem, w, nullptr, exact_mode);
          if (!(a.relax & 1)) __syncthreads();  // launch-uniform condition
          pf.count(BRAXG_PROF_MATVECS, (unsigned long long)mvs);
          pf.mark(BRAXG_PROF_CONSTRAINT);
          if (active) ok = stage_integrate<T>(smem, w) && ok;
          if (!(a.relax & 2)) __syncthreads();
          pf.mark(BRAXG_PROF_INTEGRATE);
          ok = position_stage<T, NVB>(smem, w, active, exact_mode, md.ns_iters, pf) && ok;
          pf.count(BRAXG_PROF_SUBSTEPS, 1ull);
        }
        if (TASK && active)
          task_after_rep<T>(a, smem, w, ei, r == reps - 1 && s == a.n_steps - 1, env_dt, has_act);
      }
      if (TASK) {
        const bool reset = active && task_end<T>(a, smem, w, B, env, s, reps, exact_mode);
        // the reset envs' position terms (CTA-uniform: only when some env reset)
        if (__syncthreads_or(reset)) ok = position_stage<T, NVB>(smem, w, active && reset, exact_mode, 0, pf) && ok;
      }
      if (active && a.traj_q != nullptr)
        store_vec<T>(tm, a.traj_q + s * a.traj_q_stride + B.q + env * nq, w.at(L.q), nq);
      if (active && a.traj_qd != nullptr)
        store_vec<T>(tm, a.traj_qd + s * a.traj_qd_stride + B.v + env * nv, w.at(L.qd), nv);
    }
  }
  if (!active) return;  // no CTA barrier follows
  if (a.out.cache != nullptr) store_cache<T>(a, B, smem, w, env, exact, ok);  // before the outputs touch scratch
  if (TASK && a.n_steps > 0 && !a.init) task_outputs<T>(a, smem, w, ei);
  write_outputs<T>(a, B, smem, w, env, ok);
  pf.mark(BRAXG_PROF_IO);
  pf.count(BRAXG_PROF_NS_RESETS, (unsigned long long)reinterpret_cast<const int*>(w.at(L.misc))[1]);
  pf.count(BRAXG_PROF_PG_BUILD, (unsigned long long)reinterpret_cast<const unsigned*>(w.at(L.misc))[9]);
  pf.count(BRAXG_PROF_PG_ITERATE, (unsigned long long)reinterpret_cast<const unsigned*>(w.at(L.misc))[10]);
}

// TASK: the fused env step variant (braxg_env_rollout); the plain pipeline
// kernel compiles without any of its code.
template <int T, int NVB, bool TASK>
__global__ void __launch_bounds__(512, 1) step_kernel(const StepArgs a) {
  extern __shared__ __align__(16) int smem[];
  for (int i = threadIdx.x; i < a.model_words; i += blockDim.x) smem[i] = a.model[i];
  Layout* shared_layout = reinterpret_cast<Layout*>(smem + al4(a.model_words));
  if (threadIdx.x == 0) {
    const int* w0 = a.model;
    *shared_layout = layout_of(w0, a.ovf_global, a.dyn_dr);
  }
  __syncthreads();
  const int team = threadIdx.x / T;
  long long env = (long long)blockIdx.x * a.envs_per_cta + team;
  // teams past the batch keep hitting the CTA barriers but do no work
  const bool active = team < a.envs_per_cta && env < a.n_env;
  if (!active) env = 0;
  const EnvBase B{};
  float* arena = reinterpret_cast<float*>(smem + al4(a.model_words) + kLayoutWords);
  run_team<T, NVB, TASK>(a, B, smem, shared_layout, arena, team, env, active, a.n_frames);
}

constexpr int kMaxSmemBytes = 227 * 1024;

// One launch of a step-kernel variant; the first launch on a device opts the
// kernel into the large dynamic shared memory (the flag is per template
// instance, so per kernel).
template <int T, int NVB, bool TASK>
cudaError_t launch_step_variant(const StepArgs& a, int grid, int smem, cudaStream_t st) {
  auto k = step_kernel<T, NVB, TASK>;
  static SmemOptIn opt_in;
  cudaError_t e = opt_in.ensure(k, [](int* b) {
    *b = kMaxSmemBytes;
    return cudaSuccess;
  });
  if (e != cudaSuccess) return e;
  k<<<grid, a.envs_per_cta * T, smem, st>>>(a);
  return cudaGetLastError();
}

template <int T, int NVB>
cudaError_t launch_step(const StepArgs& a, int grid, int smem, cudaStream_t st) {
  if (a.has_task) return launch_step_variant<T, NVB, true>(a, grid, smem, st);
  return launch_step_variant<T, NVB, false>(a, grid, smem, st);
}

}  // namespace braxg
