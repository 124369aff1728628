// C ABI: gradients of rollouts (braxg_rollout_vjp and its workspace queries,
// the allocation-free entry point).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "braxg.h"
#include "braxg_host.h"
#include "braxg_launch.h"
#include "braxg_adjoint.cuh"

using braxg::host::cuda_fail;
using braxg::host::fail;
using braxg::host::kMaxSmem;

extern "C" {

// Words of one frame snapshot: the forward arena plus the projected-gradient tape.
static int vjp_snap_words(const braxg_model* m) {
  return m->L.total + braxg::tape_words(m->dims.m, m->h[BXM_H_PG_ITERS]);
}

// Workspace of braxg_rollout_vjp: checkpoints [n_ckpt, n, nq + nv], then the
// frame input states [frames, n, nq + nv] and frame snapshots
// [frames, n, snap_words] of the snapshot blocks: the last `resident` segments
// as the checkpoint pass leaves them, and the first block reused by every
// recomputed segment; each part starts on a 256-byte boundary.
static int vjp_n_ckpt(int n_steps, int ckpt_every) { return (n_steps + ckpt_every - 1) / ckpt_every; }

// In Newton-Schulz mode a checkpoint also holds the carried inverse
// (nv x nv), and two parts follow the snapshots: per snapshotted frame its
// record (M and the carried inverse its update started from, nv x ld each),
// and per env the reverse's scratch (ns_rev_scratch_words: the recompute's
// tape; the reverse's other matrices live in shared memory).
static int vjp_nvb(const braxg_model* m) { return m->dims.nv <= 16 ? 16 : 32; }
static int vjp_ns_rec_words(const braxg_model* m) {
  return braxg::al4(2 * m->dims.nv * (m->dims.nv | 1));
}
static int vjp_ns_scr_words(const braxg_model* m) {
  return braxg::al4(braxg::ns_rev_scratch_words(m->dims.nv, vjp_nvb(m), m->ns_iters));
}

struct VjpSizes {
  size_t ckpt, seg, snap, nsrec, nsscr;  // floats of each part (64-float multiples but the snapshots)
  size_t total() const { return (ckpt + seg + snap + nsrec + nsscr) * sizeof(float); }
};

static VjpSizes vjp_sizes(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every, int resident,
                          bool ns) {
  const size_t S = (size_t)m->dims.nq + m->dims.nv;
  const size_t SC = S + (ns ? (size_t)m->dims.nv * m->dims.nv : 0);
  const int n_ckpt = vjp_n_ckpt(n_steps, ckpt_every);
  const int first_res = n_ckpt - resident;
  const int steps = std::max(n_steps - first_res * ckpt_every, first_res > 0 ? ckpt_every : 0);
  const size_t frames = (size_t)steps * n_frames;
  VjpSizes z{};
  z.ckpt = ((size_t)n_ckpt * n_env * SC + 63) / 64 * 64;
  z.seg = (frames * n_env * S + 63) / 64 * 64;
  z.snap = frames * n_env * (size_t)vjp_snap_words(m);
  if (ns) {
    z.snap = (z.snap + 63) / 64 * 64;
    z.nsrec = (frames * n_env * (size_t)vjp_ns_rec_words(m) + 63) / 64 * 64;
    z.nsscr = (size_t)n_env * vjp_ns_scr_words(m);
  }
  return z;
}

static size_t vjp_bytes(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every, int resident,
                        bool ns = false) {
  return vjp_sizes(m, n_env, n_steps, n_frames, ckpt_every, resident, ns).total();
}

int braxg_rollout_vjp_workspace_resident(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every,
                                         int resident, size_t* bytes) {
  if (m == nullptr || bytes == nullptr) return fail(BRAXG_ERR_INVALID, "NULL argument");
  if (n_env < 0 || n_steps < 1 || n_frames < 1 || ckpt_every < 1)
    return fail(BRAXG_ERR_INVALID, "n_env >= 0, n_steps, n_frames and ckpt_every >= 1 required");
  const int n_ckpt = vjp_n_ckpt(n_steps, ckpt_every);
  if (resident <= 0 || resident > n_ckpt) resident = n_ckpt;
  *bytes = vjp_bytes(m, n_env, n_steps, n_frames, ckpt_every, resident);
  return BRAXG_OK;
}

int braxg_rollout_vjp_workspace(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every,
                                size_t* bytes) {
  return braxg_rollout_vjp_workspace_resident(m, n_env, n_steps, n_frames, ckpt_every, 1, bytes);
}

int braxg_rollout_vjp_workspace_mode(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every,
                                     int resident, int inverse_mode, size_t* bytes) {
  int rc = braxg_rollout_vjp_workspace_resident(m, n_env, n_steps, n_frames, ckpt_every, resident, bytes);
  if (rc) return rc;
  const int n_ckpt = vjp_n_ckpt(n_steps, ckpt_every);
  if (resident <= 0 || resident > n_ckpt) resident = n_ckpt;
  const bool ns = inverse_mode == BRAXG_INV_NEWTON_SCHULZ && m->ns_iters > 0;
  *bytes = vjp_bytes(m, n_env, n_steps, n_frames, ckpt_every, resident, ns);
  return BRAXG_OK;
}

// One launch of the gradient kernel: `phases` 3 (forward and reverse), 1 (the
// forward: checkpoints, snapshots and trajectory into the workspace) or 2 (the
// reverse, from a workspace a phase-1 launch with the same arguments filled).
static int run_vjp(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, int ckpt_every,
                   const float* act_seq, const float* q0, const float* qd0, const float* q_bar, const float* qd_bar,
                   float* act_bar, float* q0_bar, float* qd0_bar, float* traj_q, float* traj_qd, void* workspace,
                   size_t workspace_bytes, int32_t* status, const braxg_options* opt, int phases) {
  braxg::host::set_launches(0);
  size_t need = 0;
  int rc = braxg_rollout_vjp_workspace(m, n_env, n_steps, n_frames, ckpt_every, &need);
  if (rc) return rc;
  // the reference's inverse (Newton-Schulz, carried and updated every frame)
  // when asked for and the model has iterations; else the exact inverse
  const bool ns = opt != nullptr && opt->inverse_mode == BRAXG_INV_NEWTON_SCHULZ && m->ns_iters > 0;
  if (ns) need = vjp_bytes(m, n_env, n_steps, n_frames, ckpt_every, 1, true);
  if (n_env == 0) return BRAXG_OK;
  if (q0 == nullptr || qd0 == nullptr) return fail(BRAXG_ERR_INVALID, "q0 and qd0 are required");
  if (workspace == nullptr || workspace_bytes < need)
    return fail(BRAXG_ERR_INVALID, "workspace of %zu bytes required (got %zu)", need, workspace_bytes);
  if (m->dims.nv > 32) return fail(BRAXG_ERR_UNSUPPORTED, "gradients support nv <= 32");
  for (int k = 0; k < m->dims.ncon; ++k) {
    const int kind = m->h[m->h[BXM_O_CON_KIND] + k], la = m->h[m->h[BXM_O_CON_LA] + k];
    const bool plane =
        (kind == BXM_CON_PLANE_SPHERE || kind == BXM_CON_PLANE_CAPSULE || kind == BXM_CON_PLANE_BOX) && la < 0;
    const bool two = kind == BXM_CON_SPHERE_SPHERE || kind == BXM_CON_SPHERE_CAPSULE || kind == BXM_CON_CAPSULE_CAPSULE;
    if (!plane && !two)
      return fail(BRAXG_ERR_UNSUPPORTED,
                  "gradients support world-plane sphere/capsule/box contacts and sphere/capsule pairs only");
  }
  // as many trailing segments resident as the workspace holds
  const int n_ckpt = vjp_n_ckpt(n_steps, ckpt_every);
  int resident = 1;
  while (resident < n_ckpt &&
         vjp_bytes(m, n_env, n_steps, n_frames, ckpt_every, resident + 1, ns) <= workspace_bytes)
    ++resident;
  const VjpSizes z = vjp_sizes(m, n_env, n_steps, n_frames, ckpt_every, resident, ns);
  if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0)
    return fail(BRAXG_ERR_INVALID, "workspace must be 16-byte aligned");
  braxg::VjpArgs a{};
  a.model = m->d_desc;
  a.model_words = m->words;
  a.n_env = n_env;
  a.n_steps = n_steps;
  a.n_frames = n_frames;
  a.ckpt_every = ckpt_every;
  a.act = act_seq;
  a.q0 = q0;
  a.qd0 = qd0;
  a.q_bar = q_bar;
  a.qd_bar = qd_bar;
  a.act_bar = act_bar;
  a.q0_bar = q0_bar;
  a.qd0_bar = qd0_bar;
  float* ws = static_cast<float*>(workspace);
  a.ckpt = ws;
  a.seg = ws + z.ckpt;
  a.snap = ws + z.ckpt + z.seg;
  a.ckpt_words = m->dims.nq + m->dims.nv + (ns ? m->dims.nv * m->dims.nv : 0);
  a.ns_iters = ns ? m->ns_iters : 0;
  if (ns) {
    a.nsrec = a.snap + z.snap;
    a.ns_rec_words = vjp_ns_rec_words(m);
    a.nsscr = a.nsrec + z.nsrec;
    a.ns_scr_words = vjp_ns_scr_words(m);
  }
  a.snap_words = vjp_snap_words(m);
  a.resident = resident;
  a.traj_q = traj_q;
  a.traj_qd = traj_qd;
  a.status = status;
  a.prof = opt ? opt->stage_cycles : nullptr;
  a.phases = phases;
  braxg::AdjLayout A = braxg::make_adj_layout(m->dims.nl, m->dims.nq, m->dims.nv, m->dims.nu, m->dims.ncon,
                                              m->dims.nlim, m->h[BXM_H_PG_ITERS],
                                              ns ? braxg::ns_rev_smem_words(m->dims.nv, vjp_nvb(m)) : 0);
  int head = (braxg::al4(m->words) + 2 * braxg::kLayoutWords) * 4;
  int env_bytes = (m->L.total + A.total) * 4;
  int epc = (kMaxSmem - head) / env_bytes;
  if (epc < 1) return fail(BRAXG_ERR_UNSUPPORTED, "model too large for the gradient kernel's shared memory");
  if (epc > 8) epc = 8;
  if (m->sms > 0) epc = std::max(1, std::min(epc, (n_env + m->sms - 1) / m->sms));  // spread over every SM
  a.envs_per_cta = epc;
  int smem = head + epc * env_bytes;
  int grid = (n_env + epc - 1) / epc;
  int cur = 0;
  cudaError_t e = cudaGetDevice(&cur);
  if (e == cudaSuccess && cur != m->device) e = cudaSetDevice(m->device);
  if (e != cudaSuccess) return cuda_fail(e, "selecting the model's device");
  e = m->dims.nv <= 16 ? braxg::launch_vjp<32, 16>(a, grid, smem, static_cast<cudaStream_t>(stream))
                       : braxg::launch_vjp<32, 32>(a, grid, smem, static_cast<cudaStream_t>(stream));
  const cudaError_t back = cur != m->device ? cudaSetDevice(cur) : cudaSuccess;
  if (e != cudaSuccess) return cuda_fail(e, "gradient kernel launch");
  if (back != cudaSuccess) return cuda_fail(back, "restoring the current device");
  braxg::host::set_launches(1);
  return BRAXG_OK;
}

int braxg_rollout_vjp(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, int ckpt_every,
                      const float* act_seq, const float* q0, const float* qd0, const float* q_bar,
                      const float* qd_bar, float* act_bar, float* q0_bar, float* qd0_bar, float* traj_q,
                      float* traj_qd, void* workspace, size_t workspace_bytes, int32_t* status,
                      const braxg_options* opt) {
  return run_vjp(m, stream, n_env, n_steps, n_frames, ckpt_every, act_seq, q0, qd0, q_bar, qd_bar, act_bar, q0_bar,
                 qd0_bar, traj_q, traj_qd, workspace, workspace_bytes, status, opt, 3);
}

int braxg_rollout_vjp_fwd(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, int ckpt_every,
                          const float* act_seq, const float* q0, const float* qd0, float* traj_q, float* traj_qd,
                          void* workspace, size_t workspace_bytes, int32_t* status, const braxg_options* opt) {
  if (n_env > 0 && (traj_q == nullptr || traj_qd == nullptr))
    return fail(BRAXG_ERR_INVALID, "braxg_rollout_vjp_fwd: traj_q and traj_qd are required");
  return run_vjp(m, stream, n_env, n_steps, n_frames, ckpt_every, act_seq, q0, qd0, nullptr, nullptr, nullptr,
                 nullptr, nullptr, traj_q, traj_qd, workspace, workspace_bytes, status, opt, 1);
}

int braxg_rollout_vjp_bwd(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, int ckpt_every,
                          const float* act_seq, const float* q0, const float* qd0, const float* q_bar,
                          const float* qd_bar, float* act_bar, float* q0_bar, float* qd0_bar, void* workspace,
                          size_t workspace_bytes, int32_t* status, const braxg_options* opt) {
  return run_vjp(m, stream, n_env, n_steps, n_frames, ckpt_every, act_seq, q0, qd0, q_bar, qd_bar, act_bar, q0_bar,
                 qd0_bar, nullptr, nullptr, workspace, workspace_bytes, status, opt, 2);
}

// ---------------------------------------------------------------------------
// Allocation-free rollout gradient.  The checkpoint / segment workspace of
// braxg_rollout_vjp lives in one fixed device array of this library, so the
// caller passes only its inputs and outputs and nothing here allocates.  Each
// device that loads the library holds the array until the process exits.
// The array's device address is looked up once per device and kept for the
// process: cudaDeviceReset destroys the context that address belongs to, so
// after a reset this entry point (like every model handle) must not be used.
// ---------------------------------------------------------------------------
static constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // 8 MiB
static __device__ __align__(256) unsigned char g_vjp_scratch[kNoAllocScratchBytes];
static std::mutex g_scratch_mu;
static void* g_scratch_addr[64] = {nullptr};  // device address of g_vjp_scratch, per device

size_t braxg_rollout_vjp_noalloc_capacity(void) { return kNoAllocScratchBytes; }

int braxg_rollout_vjp_noalloc(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames,
                              int ckpt_every, const float* act_seq, const float* q0, const float* qd0,
                              const float* q_bar, const float* qd_bar, float* act_bar, float* q0_bar,
                              float* qd0_bar, float* traj_q, float* traj_qd, int32_t* status,
                              const braxg_options* opt) {
  size_t need = 0;
  int rc = braxg_rollout_vjp_workspace_mode(m, n_env, n_steps, n_frames, ckpt_every, 1,
                                            opt ? opt->inverse_mode : BRAXG_INV_CHOLESKY, &need);
  if (rc) return rc;
  if (need > kNoAllocScratchBytes)
    return fail(BRAXG_ERR_INVALID,
                "braxg_rollout_vjp_noalloc: %d envs x %d steps x %d frames (checkpoint every %d) need %zu bytes "
                "of scratch; the fixed array holds %zu bytes (pass a workspace to braxg_rollout_vjp instead)",
                n_env, n_steps, n_frames, ckpt_every, need, kNoAllocScratchBytes);
  if (m->device < 0 || m->device >= 64) return fail(BRAXG_ERR_INVALID, "device ordinal %d out of range", m->device);
  void* scratch = nullptr;
  {
    // first call on a device: look up the array's device address with that
    // device current (once; later calls reuse it)
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_addr[m->device] == nullptr) {
      int cur = 0;
      cudaError_t e = cudaGetDevice(&cur);
      if (e != cudaSuccess) return cuda_fail(e, "braxg_rollout_vjp_noalloc: cudaGetDevice");
      e = cudaSetDevice(m->device);
      void* addr = nullptr;
      if (e == cudaSuccess) e = cudaGetSymbolAddress(&addr, g_vjp_scratch);
      const cudaError_t back = cudaSetDevice(cur);
      if (e != cudaSuccess) return cuda_fail(e, "braxg_rollout_vjp_noalloc: cudaGetSymbolAddress");
      if (back != cudaSuccess) return cuda_fail(back, "braxg_rollout_vjp_noalloc: restoring the current device");
      g_scratch_addr[m->device] = addr;
    }
    scratch = g_scratch_addr[m->device];
  }
  // Every word of the checkpoint / segment workspace is written before it is
  // read, so the array's previous contents need no clearing.
  return braxg_rollout_vjp(m, stream, n_env, n_steps, n_frames, ckpt_every, act_seq, q0, qd0, q_bar, qd_bar,
                           act_bar, q0_bar, qd0_bar, traj_q, traj_qd, scratch, kNoAllocScratchBytes, status, opt);
}

}  // extern "C"
