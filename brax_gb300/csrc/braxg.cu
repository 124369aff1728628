// C ABI (include/braxg.h) and the fused step kernel launches.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "braxg.h"
#include "braxg_launch.h"
#include "braxg_step.cuh"
#include "braxg_adjoint.cuh"


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct braxg_model {
  int device;
  int* d_desc;
  int words;
  std::vector<int> h;
  braxg_dims dims;
  int ns_iters;
  int sms;  // multiprocessors of the model's device
  braxg::Layout L;
};

namespace {

thread_local std::string g_err;
thread_local int g_launches = 0;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(BRAXG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

struct Shape {
  int T, NVB, epc, smem;
};

constexpr int kMaxSmem = 227 * 1024;
// threads per CTA of the step kernels (launch bound 512 x 1: 128 registers)
constexpr int kMaxBlock = 512;

int choose_shape(const braxg_model* m, const braxg_options* opt, int n_env, Shape* s) {
  int nv = m->dims.nv;
  s->NVB = nv <= 16 ? 16 : (nv <= 32 ? 32 : 64);
  // default lanes per env: 16 for small models (nv <= 8: two envs per warp),
  // else 32 (measured on the packaged models, one CTA per SM)
  int T = (opt && opt->threads_per_env) ? opt->threads_per_env : (nv <= 8 ? 16 : 32);
  if (T != 16 && T != 32) return fail(BRAXG_ERR_INVALID, "threads_per_env must be 0, 16 or 32 (got %d)", T);
  if (T == 16 && s->NVB == 64) T = 32;
  s->T = T;
  int model_bytes = (braxg::al4(m->words) + braxg::kLayoutWords) * 4;
  int env_bytes = m->L.total * 4;
  int max_epc = kMaxBlock / T;
  int fit = (kMaxSmem - model_bytes) / env_bytes;
  if (fit < 1)
    return fail(BRAXG_ERR_UNSUPPORTED, "model needs %d bytes of shared memory per env; at most %d fit",
                env_bytes, kMaxSmem - model_bytes);
  int epc = (opt && opt->envs_per_cta) ? opt->envs_per_cta : 0;
  if (epc == 0) {
    // default: one CTA per SM holding as many envs as its shared memory and
    // 512 threads allow, so that every warp of the SM runs the same stage's
    // code (the instruction working set of one stage); a batch too small to
    // fill every SM that way is spread over all of them instead
    epc = (kMaxSmem - model_bytes) / env_bytes;
    if (n_env > 0 && m->sms > 0) epc = std::min(epc, (n_env + m->sms - 1) / m->sms);
    if (epc < 1) epc = 1;
    if (epc > max_epc) epc = max_epc;
  }
  if (epc > max_epc || epc > fit || epc < 1)
    return fail(BRAXG_ERR_INVALID, "envs_per_cta %d out of range [1, %d]", epc, fit < max_epc ? fit : max_epc);
  s->epc = epc;
  s->smem = model_bytes + epc * env_bytes;
  return BRAXG_OK;
}

int launch(const braxg_model* m, const braxg_options* opt, braxg::StepArgs& a, cudaStream_t st) {
  g_launches = 0;
  Shape s;
  int rc = choose_shape(m, opt, a.n_env, &s);
  if (rc) return rc;
  if (a.n_env == 0) return BRAXG_OK;
  a.envs_per_cta = s.epc;
  a.prof = opt ? opt->stage_cycles : nullptr;
  a.relax = opt ? opt->relax_barriers : 0;
  int grid = (a.n_env + s.epc - 1) / s.epc;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != m->device) {
    cudaError_t e = cudaSetDevice(m->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  }
  cudaError_t e;
  if (s.T == 16 && s.NVB == 16) e = braxg::launch_step<16, 16>(a, grid, s.smem, st);
  else if (s.T == 16) e = braxg::launch_step<16, 32>(a, grid, s.smem, st);
  else if (s.NVB == 16) e = braxg::launch_step<32, 16>(a, grid, s.smem, st);
  else if (s.NVB == 32) e = braxg::launch_step<32, 32>(a, grid, s.smem, st);
  else e = braxg::launch_step<32, 64>(a, grid, s.smem, st);
  if (cur != m->device) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
  g_launches = 1;
  return BRAXG_OK;
}

int check_common(const braxg_model* m, int n_env, const braxg_options* opt) {
  if (m == nullptr) return fail(BRAXG_ERR_INVALID, "model is NULL");
  if (n_env < 0) return fail(BRAXG_ERR_INVALID, "n_env must be >= 0 (got %d)", n_env);
  if (opt && opt->inverse_mode != BRAXG_INV_NEWTON_SCHULZ && opt->inverse_mode != BRAXG_INV_CHOLESKY)
    return fail(BRAXG_ERR_INVALID, "unknown inverse_mode %d", opt->inverse_mode);
  return BRAXG_OK;
}

}  // namespace

extern "C" {

const char* braxg_last_error(void) { return g_err.c_str(); }

int braxg_last_launch_count(void) { return g_launches; }

int braxg_model_create(const void* desc, size_t desc_bytes, int device, braxg_model** out) {
  if (desc == nullptr || out == nullptr) return fail(BRAXG_ERR_INVALID, "NULL descriptor or output");
  if (desc_bytes < BXM_HEADER_WORDS * 4 || desc_bytes % 4 != 0)
    return fail(BRAXG_ERR_INVALID, "descriptor size %zu is not a whole header", desc_bytes);
  const int* w = static_cast<const int*>(desc);
  if ((unsigned)w[BXM_H_MAGIC] != (unsigned)BXM_MAGIC || w[BXM_H_VERSION] != BXM_VERSION)
    return fail(BRAXG_ERR_INVALID, "bad descriptor magic/version");
  int words = w[BXM_H_WORDS];
  if ((size_t)words * 4 != desc_bytes) return fail(BRAXG_ERR_INVALID, "descriptor length mismatch");
  for (int k = BXM_O_LINK_PARENT; k <= BXM_O_CON_SOLP; ++k)
    if (w[k] < BXM_HEADER_WORDS || w[k] > words) return fail(BRAXG_ERR_INVALID, "descriptor offset %d out of range", k);
  braxg_dims d{w[BXM_H_NL], w[BXM_H_NQ], w[BXM_H_NV], w[BXM_H_NU], w[BXM_H_NCON], w[BXM_H_NLIM], w[BXM_H_M]};
  if (d.nl < 1 || d.nv < 1 || d.nv > 64 || d.nq < 1 || d.nu < 0 || d.ncon < 0 || d.nlim < 0 || d.nl > 64)
    return fail(BRAXG_ERR_UNSUPPORTED, "model dims out of the supported envelope (nl %d, nv %d)", d.nl, d.nv);
  if (d.m != 4 * d.ncon + d.nlim) return fail(BRAXG_ERR_INVALID, "inconsistent constraint row count");
  auto* m = new braxg_model();
  m->device = device;
  m->words = words;
  m->h.assign(w, w + words);
  m->dims = d;
  m->ns_iters = w[BXM_H_NS_ITERS];
  m->L = braxg::layout_of(w);
  int cur = 0;
  cudaGetDevice(&cur);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_desc, (size_t)words * 4);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_desc, w, (size_t)words * 4, cudaMemcpyHostToDevice);
  cudaSetDevice(cur);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "braxg_model_create");
  }
  *out = m;
  return BRAXG_OK;
}

int braxg_model_destroy(braxg_model* m) {
  if (m == nullptr) return BRAXG_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(m->device);
  cudaFree(m->d_desc);
  cudaSetDevice(cur);
  delete m;
  return BRAXG_OK;
}

int braxg_model_dims(const braxg_model* m, braxg_dims* out) {
  if (m == nullptr || out == nullptr) return fail(BRAXG_ERR_INVALID, "NULL argument");
  *out = m->dims;
  return BRAXG_OK;
}

int braxg_launch_shape(const braxg_model* m, const braxg_options* opt, int32_t* tpe, int32_t* epc, int32_t* smem) {
  if (m == nullptr) return fail(BRAXG_ERR_INVALID, "model is NULL");
  Shape s;
  int rc = choose_shape(m, opt, 0, &s);
  if (rc) return rc;
  if (tpe) *tpe = s.T;
  if (epc) *epc = s.epc;
  if (smem) *smem = s.smem;
  return BRAXG_OK;
}

int braxg_init(const braxg_model* m, void* stream, int n_env, const float* q, const float* qd, braxg_state* out,
               const braxg_options* opt) {
  int rc = check_common(m, n_env, opt);
  if (rc) return rc;
  if (out == nullptr || (n_env > 0 && (q == nullptr || qd == nullptr)))
    return fail(BRAXG_ERR_INVALID, "q, qd and out are required");
  braxg::StepArgs a{};
  a.model = m->d_desc;
  a.model_words = m->words;
  a.n_env = n_env;
  a.n_steps = 0;
  a.n_frames = 0;
  a.exact_inverse = 1;
  a.init = 1;
  a.q_in = q;
  a.qd_in = qd;
  a.out = *out;
  return launch(m, opt, a, static_cast<cudaStream_t>(stream));
}

static int run_steps(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, const float* act,
                     long long act_stride, const braxg_state* in, braxg_state* out, float* tq, float* tqd,
                     const braxg_options* opt, const braxg_task* task = nullptr,
                     const braxg_env_io* io = nullptr) {
  int rc = check_common(m, n_env, opt);
  if (rc) return rc;
  if (in == nullptr || out == nullptr) return fail(BRAXG_ERR_INVALID, "in and out states are required");
  if (n_frames < 1 || n_steps < 0) return fail(BRAXG_ERR_INVALID, "n_frames must be >= 1 and n_steps >= 0");
  bool ns = !(opt && opt->inverse_mode == BRAXG_INV_CHOLESKY) && m->ns_iters > 0;
  if (n_env > 0 && (in->q == nullptr || in->qd == nullptr || (ns && in->mass_mx_inv == nullptr)))
    return fail(BRAXG_ERR_INVALID, "in->q, in->qd and (Newton-Schulz mode) in->mass_mx_inv are required");
  braxg::StepArgs a{};
  a.model = m->d_desc;
  a.model_words = m->words;
  a.n_env = n_env;
  a.n_steps = n_steps;
  a.n_frames = n_frames;
  a.exact_inverse = ns ? 0 : 1;
  a.init = 0;
  a.q_in = in->q;
  a.qd_in = in->qd;
  a.minv_in = in->mass_mx_inv;
  a.act = act;
  a.act_step_stride = act_stride;
  a.out = *out;
  a.traj_q = tq;
  a.traj_qd = tqd;
  a.traj_q_stride = (long long)n_env * m->dims.nq;
  a.traj_qd_stride = (long long)n_env * m->dims.nv;
  a.env_step_stride = n_env;
  if (task != nullptr) {
    a.has_task = 1;
    a.task = *task;
    a.io = *io;
  }
  return launch(m, opt, a, static_cast<cudaStream_t>(stream));
}

// Words of one frame snapshot: the forward arena plus the projected-gradient tape.
static int vjp_snap_words(const braxg_model* m) {
  return m->L.total + braxg::al4(braxg::kTapeHeadWords + m->h[BXM_H_PG_ITERS] * braxg::kTapeIterWords);
}

// Workspace of braxg_rollout_vjp: checkpoints [n_ckpt, n, nq + nv], then the
// frame input states [frames, n, nq + nv] and frame snapshots
// [frames, n, snap_words] of the snapshot blocks: the last `resident` segments
// as the checkpoint pass leaves them, and the first block reused by every
// recomputed segment; each part starts on a 256-byte boundary.
static int vjp_n_ckpt(int n_steps, int ckpt_every) { return (n_steps + ckpt_every - 1) / ckpt_every; }

static void vjp_sizes(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every, int resident,
                      size_t* ckpt_floats, size_t* seg_floats, size_t* snap_floats) {
  size_t S = (size_t)m->dims.nq + m->dims.nv;
  const int n_ckpt = vjp_n_ckpt(n_steps, ckpt_every);
  const int first_res = n_ckpt - resident;
  const int steps = std::max(n_steps - first_res * ckpt_every, first_res > 0 ? ckpt_every : 0);
  size_t frames = (size_t)steps * n_frames;
  *ckpt_floats = ((size_t)n_ckpt * n_env * S + 63) / 64 * 64;
  *seg_floats = (frames * n_env * S + 63) / 64 * 64;
  *snap_floats = frames * n_env * (size_t)vjp_snap_words(m);
}

static size_t vjp_bytes(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every, int resident) {
  size_t c, sg, sn;
  vjp_sizes(m, n_env, n_steps, n_frames, ckpt_every, resident, &c, &sg, &sn);
  return (c + sg + sn) * sizeof(float);
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

int braxg_rollout_vjp(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, int ckpt_every,
                      const float* act_seq, const float* q0, const float* qd0, const float* q_bar,
                      const float* qd_bar, float* act_bar, float* q0_bar, float* qd0_bar, float* traj_q,
                      float* traj_qd, void* workspace, size_t workspace_bytes, int32_t* status,
                      const braxg_options* opt) {
  g_launches = 0;
  size_t need = 0;
  int rc = braxg_rollout_vjp_workspace(m, n_env, n_steps, n_frames, ckpt_every, &need);
  if (rc) return rc;
  if (n_env == 0) return BRAXG_OK;
  if (q0 == nullptr || qd0 == nullptr) return fail(BRAXG_ERR_INVALID, "q0 and qd0 are required");
  if (workspace == nullptr || workspace_bytes < need)
    return fail(BRAXG_ERR_INVALID, "workspace of %zu bytes required (got %zu)", need, workspace_bytes);
  if (m->dims.nv > 32) return fail(BRAXG_ERR_UNSUPPORTED, "gradients support nv <= 32");
  for (int k = 0; k < m->dims.ncon; ++k) {
    int kind = m->h[m->h[BXM_O_CON_KIND] + k], la = m->h[m->h[BXM_O_CON_LA] + k];
    if ((kind != BXM_CON_PLANE_SPHERE && kind != BXM_CON_PLANE_CAPSULE) || la >= 0)
      return fail(BRAXG_ERR_UNSUPPORTED, "gradients support world-plane sphere/capsule contacts only");
  }
  // as many trailing segments resident as the workspace holds
  const int n_ckpt = vjp_n_ckpt(n_steps, ckpt_every);
  int resident = 1;
  while (resident < n_ckpt &&
         vjp_bytes(m, n_env, n_steps, n_frames, ckpt_every, resident + 1) <= workspace_bytes)
    ++resident;
  size_t c, sg, sn;
  vjp_sizes(m, n_env, n_steps, n_frames, ckpt_every, resident, &c, &sg, &sn);
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
  a.ckpt = static_cast<float*>(workspace);
  a.seg = static_cast<float*>(workspace) + c;
  a.snap = static_cast<float*>(workspace) + c + sg;
  a.snap_words = vjp_snap_words(m);
  a.resident = resident;
  a.traj_q = traj_q;
  a.traj_qd = traj_qd;
  a.status = status;
  a.prof = opt ? opt->stage_cycles : nullptr;
  braxg::AdjLayout A = braxg::make_adj_layout(m->dims.nl, m->dims.nq, m->dims.nv, m->dims.nu, m->dims.ncon,
                                              m->dims.nlim, m->h[BXM_H_PG_ITERS]);
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
  cudaGetDevice(&cur);
  if (cur != m->device) cudaSetDevice(m->device);
  cudaError_t e = m->dims.nv <= 16 ? braxg::launch_vjp<32, 16>(a, grid, smem, static_cast<cudaStream_t>(stream))
                                   : braxg::launch_vjp<32, 32>(a, grid, smem, static_cast<cudaStream_t>(stream));
  if (cur != m->device) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "gradient kernel launch");
  g_launches = 1;
  return BRAXG_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free rollout gradient.  The checkpoint / segment workspace of
// braxg_rollout_vjp lives in one fixed device array of this library, so the
// caller passes only its inputs and outputs and nothing here allocates.  Each
// device that loads the library holds the array until the process exits.
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
  int rc = braxg_rollout_vjp_workspace(m, n_env, n_steps, n_frames, ckpt_every, &need);
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
      cudaGetDevice(&cur);
      cudaError_t e = cudaSetDevice(m->device);
      void* addr = nullptr;
      if (e == cudaSuccess) e = cudaGetSymbolAddress(&addr, g_vjp_scratch);
      cudaSetDevice(cur);
      if (e != cudaSuccess) return cuda_fail(e, "braxg_rollout_vjp_noalloc: cudaGetSymbolAddress");
      g_scratch_addr[m->device] = addr;
    }
    scratch = g_scratch_addr[m->device];
  }
  // Every word of the checkpoint / segment workspace is written before it is
  // read, so the array's previous contents need no clearing.
  return braxg_rollout_vjp(m, stream, n_env, n_steps, n_frames, ckpt_every, act_seq, q0, qd0, q_bar, qd_bar,
                           act_bar, q0_bar, qd0_bar, traj_q, traj_qd, scratch, kNoAllocScratchBytes, status, opt);
}

// ---------------------------------------------------------------------------
// Uneven batches: several models, each a group of envs, in one persistent
// launch of batch_kernel.  State arrays are flat: group g's envs occupy one
// contiguous run of every field, starting at that group's offsets.
// ---------------------------------------------------------------------------
struct braxg_batch {
  int device;
  int n_models;
  std::vector<braxg::BatchGroup> groups;
  std::vector<braxg::BatchItem> items;
  std::vector<braxg_batch_offsets> offs;  // n_models + 1 (the last is the totals)
  std::vector<int> ns_iters;
  braxg::BatchGroup* d_groups = nullptr;
  braxg::BatchItem* d_items = nullptr;
  int* d_counter = nullptr;
  int block = 0, smem = 0, grid = 0;
};

static void batch_free(braxg_batch* b) {
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(b->device);
  if (b->d_groups) cudaFree(b->d_groups);
  if (b->d_items) cudaFree(b->d_items);
  if (b->d_counter) cudaFree(b->d_counter);
  cudaSetDevice(cur);
  delete b;
}

int braxg_batch_create(const braxg_model* const* models, const int32_t* n_env, const int32_t* n_frames, int n_models,
                       const braxg_bucket_shape* shapes, int n_shapes, int32_t smem_per_cta, braxg_batch** out) {
  if (models == nullptr || n_env == nullptr || out == nullptr || n_models < 1)
    return fail(BRAXG_ERR_INVALID, "models, n_env and out are required and n_models >= 1");
  if (n_shapes < 0 || (n_shapes > 0 && shapes == nullptr)) return fail(BRAXG_ERR_INVALID, "bad shape list");
  // the batch kernel keeps one work-item index in static shared memory
  const int max_smem = kMaxSmem - 16;
  if (smem_per_cta < 0 || smem_per_cta > max_smem)
    return fail(BRAXG_ERR_INVALID, "smem_per_cta must be in [0, %d]", max_smem);
  const int device = models[0] ? models[0]->device : 0;
  struct Plan {
    int T, epc, head, env_bytes;
    double cost;
  };
  std::vector<Plan> plan(n_models);
  int budget = smem_per_cta > 0 ? smem_per_cta : max_smem;
  for (int g = 0; g < n_models; ++g) {
    const braxg_model* m = models[g];
    if (m == nullptr) return fail(BRAXG_ERR_INVALID, "model %d is NULL", g);
    if (m->device != device) return fail(BRAXG_ERR_INVALID, "model %d lives on device %d, not %d", g, m->device, device);
    if (n_env[g] < 0) return fail(BRAXG_ERR_INVALID, "n_env[%d] = %d < 0", g, n_env[g]);
    if (n_frames != nullptr && n_frames[g] < 1) return fail(BRAXG_ERR_INVALID, "n_frames[%d] must be >= 1", g);
    const int nv = m->dims.nv;
    int T = nv <= 8 ? 16 : 32, epc = 0;  // as the single-model default
    for (int k = 0; k < n_shapes; ++k) {
      if (nv <= shapes[k].nv_max) {
        T = shapes[k].threads_per_env;
        epc = shapes[k].envs_per_cta;
        break;
      }
    }
    if (T != 16 && T != 32) return fail(BRAXG_ERR_INVALID, "threads_per_env must be 16 or 32 (got %d)", T);
    if (T == 16 && nv > 32) return fail(BRAXG_ERR_INVALID, "16 lanes per env support nv <= 32 (model %d has %d)", g, nv);
    if (epc < 0 || epc > kMaxBlock / T)
      return fail(BRAXG_ERR_INVALID, "envs_per_cta %d out of range [0, %d]", epc, kMaxBlock / T);
    Plan& p = plan[g];
    p.T = T;
    p.epc = epc;
    p.head = (braxg::al4(m->words) + braxg::kLayoutWords) * 4;
    p.env_bytes = m->L.total * 4;
    const int need = p.head + p.env_bytes * (epc > 0 ? epc : 1);
    if (need > max_smem)
      return fail(BRAXG_ERR_UNSUPPORTED, "model %d needs %d bytes of shared memory for %d envs; at most %d fit", g,
                  need, epc > 0 ? epc : 1, max_smem);
    if (smem_per_cta > 0 && need > smem_per_cta)  // an explicit budget is a limit, not a hint
      return fail(BRAXG_ERR_INVALID, "model %d needs %d bytes of shared memory for %d envs; smem_per_cta is %d", g,
                  need, epc > 0 ? epc : 1, smem_per_cta);
    budget = std::max(budget, p.head + p.env_bytes * (epc > 0 ? epc : 1));
    // per-env latency estimate (lockstep CTAs run about as long as one env)
    const double nl = m->dims.nl, v = nv, rows = m->dims.m;
    p.cost = (n_frames ? n_frames[g] : 1) * (400 * nl + 150 * v + 11 * v * v + v * v * v / 3 + rows * v * v);
  }
  auto* b = new braxg_batch();
  b->device = device;
  b->n_models = n_models;
  b->groups.resize(n_models);
  b->offs.resize(n_models + 1);
  b->ns_iters.resize(n_models);
  braxg_batch_offsets acc{0, 0, 0, 0, 0, 0, 0, 0};
  int block = 32, smem = 0;
  for (int g = 0; g < n_models; ++g) {
    const braxg_model* m = models[g];
    Plan& p = plan[g];
    if (p.epc == 0) p.epc = std::max(1, std::min(kMaxBlock / p.T, (budget - p.head) / p.env_bytes));
    block = std::max(block, (p.epc * p.T + 31) / 32 * 32);
    smem = std::max(smem, p.head + p.epc * p.env_bytes);
    braxg::BatchGroup& G = b->groups[g];
    G.model = m->d_desc;
    G.model_words = m->words;
    G.threads_per_env = p.T;
    G.nvb = m->dims.nv <= 16 ? 16 : (m->dims.nv <= 32 ? 32 : 64);
    G.n_frames = n_frames ? n_frames[g] : 1;
    G.base = braxg::EnvBase{acc.env, acc.q, acc.qd, acc.mass_mx, acc.link, acc.act, acc.row, acc.jac};
    b->offs[g] = acc;
    b->ns_iters[g] = m->ns_iters;
    const long long n = n_env[g];
    const braxg_dims& d = m->dims;
    acc.env += n;
    acc.q += n * d.nq;
    acc.qd += n * d.nv;
    acc.mass_mx += n * d.nv * d.nv;
    acc.link += n * d.nl;
    acc.act += n * d.nu;
    acc.row += n * d.m;
    acc.jac += n * d.m * d.nv;
    for (int e0 = 0; e0 < n_env[g]; e0 += p.epc)
      b->items.push_back(braxg::BatchItem{g, e0, std::min(p.epc, n_env[g] - e0), 0});
  }
  b->offs[n_models] = acc;
  std::stable_sort(b->items.begin(), b->items.end(), [&](const braxg::BatchItem& x, const braxg::BatchItem& y) {
    return plan[x.group].cost > plan[y.group].cost;
  });
  b->block = block;
  b->smem = smem;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaError_t e = cudaSetDevice(device);
  int sms = 0, per_sm = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = braxg::batch_kernel_occupancy(block, smem, &per_sm);
  if (e == cudaSuccess && per_sm < 1) e = cudaErrorInvalidConfiguration;
  const size_t ni = std::max<size_t>(b->items.size(), 1);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_groups, sizeof(braxg::BatchGroup) * n_models);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_items, sizeof(braxg::BatchItem) * ni);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, sizeof(int));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_groups, b->groups.data(), sizeof(braxg::BatchGroup) * n_models, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !b->items.empty())
    e = cudaMemcpy(b->d_items, b->items.data(), sizeof(braxg::BatchItem) * b->items.size(), cudaMemcpyHostToDevice);
  cudaSetDevice(cur);
  if (e != cudaSuccess) {
    batch_free(b);
    return cuda_fail(e, "braxg_batch_create");
  }
  b->grid = (int)std::min<long long>((long long)sms * per_sm, (long long)b->items.size());
  *out = b;
  return BRAXG_OK;
}

int braxg_batch_destroy(braxg_batch* b) {
  if (b != nullptr) batch_free(b);
  return BRAXG_OK;
}

int braxg_batch_get_offsets(const braxg_batch* b, int index, braxg_batch_offsets* out) {
  if (b == nullptr || out == nullptr) return fail(BRAXG_ERR_INVALID, "NULL argument");
  if (index < 0 || index > b->n_models) return fail(BRAXG_ERR_INVALID, "index %d out of [0, %d]", index, b->n_models);
  *out = b->offs[index];
  return BRAXG_OK;
}

int braxg_batch_launch_info(const braxg_batch* b, int32_t* grid, int32_t* block, int32_t* smem, int32_t* n_items) {
  if (b == nullptr) return fail(BRAXG_ERR_INVALID, "batch is NULL");
  if (grid) *grid = b->grid;
  if (block) *block = b->block;
  if (smem) *smem = b->smem;
  if (n_items) *n_items = (int32_t)b->items.size();
  return BRAXG_OK;
}

static int batch_launch(const braxg_batch* b, void* stream, braxg::StepArgs& s, const braxg_options* opt) {
  g_launches = 0;
  if (b->items.empty()) return BRAXG_OK;
  braxg::BatchArgs ba{};
  s.prof = opt ? opt->stage_cycles : nullptr;
  s.relax = opt ? opt->relax_barriers : 0;
  ba.s = s;
  ba.groups = b->d_groups;
  ba.items = b->d_items;
  ba.n_items = (int)b->items.size();
  ba.counter = b->d_counter;
  ba.smem_bytes = b->smem;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != b->device) cudaSetDevice(b->device);
  cudaError_t e = braxg::launch_batch_kernel(ba, b->grid, b->block, b->smem, static_cast<cudaStream_t>(stream));
  if (cur != b->device) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "batch kernel launch");
  g_launches = 1;
  return BRAXG_OK;
}

int braxg_batch_init(const braxg_batch* b, void* stream, const float* q, const float* qd, braxg_state* out,
                     const braxg_options* opt) {
  if (b == nullptr) return fail(BRAXG_ERR_INVALID, "batch is NULL");
  if (opt && opt->inverse_mode != BRAXG_INV_NEWTON_SCHULZ && opt->inverse_mode != BRAXG_INV_CHOLESKY)
    return fail(BRAXG_ERR_INVALID, "unknown inverse_mode %d", opt->inverse_mode);
  if (out == nullptr || (b->offs.back().env > 0 && (q == nullptr || qd == nullptr)))
    return fail(BRAXG_ERR_INVALID, "q, qd and out are required");
  braxg::StepArgs s{};
  s.exact_inverse = 1;
  s.init = 1;
  s.q_in = q;
  s.qd_in = qd;
  s.out = *out;
  return batch_launch(b, stream, s, opt);
}

int braxg_batch_rollout(const braxg_batch* b, void* stream, int n_steps, const float* act_seq, const braxg_state* in,
                        braxg_state* out, float* traj_q, float* traj_qd, const braxg_options* opt) {
  if (b == nullptr) return fail(BRAXG_ERR_INVALID, "batch is NULL");
  if (opt && opt->inverse_mode != BRAXG_INV_NEWTON_SCHULZ && opt->inverse_mode != BRAXG_INV_CHOLESKY)
    return fail(BRAXG_ERR_INVALID, "unknown inverse_mode %d", opt->inverse_mode);
  if (in == nullptr || out == nullptr) return fail(BRAXG_ERR_INVALID, "in and out states are required");
  if (n_steps < 0) return fail(BRAXG_ERR_INVALID, "n_steps must be >= 0");
  const bool ns_mode = !(opt && opt->inverse_mode == BRAXG_INV_CHOLESKY);
  bool needs_minv = false;
  for (int it : b->ns_iters) needs_minv = needs_minv || (ns_mode && it > 0);
  if (b->offs.back().env > 0 && (in->q == nullptr || in->qd == nullptr || (needs_minv && in->mass_mx_inv == nullptr)))
    return fail(BRAXG_ERR_INVALID, "in->q, in->qd and (Newton-Schulz mode) in->mass_mx_inv are required");
  const braxg_batch_offsets& tot = b->offs.back();
  braxg::StepArgs s{};
  s.n_steps = n_steps;
  s.exact_inverse = ns_mode ? 0 : 1;
  s.q_in = in->q;
  s.qd_in = in->qd;
  s.minv_in = in->mass_mx_inv;
  s.act = act_seq;
  s.act_step_stride = tot.act;
  s.out = *out;
  s.traj_q = traj_q;
  s.traj_qd = traj_qd;
  s.traj_q_stride = tot.q;
  s.traj_qd_stride = tot.qd;
  return batch_launch(b, stream, s, opt);
}

int braxg_env_rollout(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, const float* act_seq,
                      const braxg_state* in, braxg_state* out, const braxg_task* task, const braxg_env_io* io,
                      const braxg_options* opt) {
  if (m == nullptr || task == nullptr || io == nullptr) return fail(BRAXG_ERR_INVALID, "model, task and io are required");
  if (task->episode_length < 1 || task->action_repeat < 1)
    return fail(BRAXG_ERR_INVALID, "episode_length and action_repeat must be >= 1");
  if (task->exclude_current_positions && m->dims.nq < 2)
    return fail(BRAXG_ERR_INVALID, "exclude_current_positions needs nq >= 2");
  const bool ns = !(opt && opt->inverse_mode == BRAXG_INV_CHOLESKY) && m->ns_iters > 0;
  if (n_env > 0 && (io->obs == nullptr || io->reward == nullptr || io->steps == nullptr || io->truncation == nullptr ||
                    io->last_done == nullptr || io->first_q == nullptr || io->first_qd == nullptr ||
                    (ns && task->auto_reset && io->first_mass_mx_inv == nullptr)))
    return fail(BRAXG_ERR_INVALID,
                "io.obs, reward, steps, truncation, last_done, first_q, first_qd (and, Newton-Schulz mode with "
                "auto_reset, first_mass_mx_inv) are required");
  long long stride = (long long)n_env * m->dims.nu;
  return run_steps(m, stream, n_env, n_steps, n_frames, act_seq, stride, in, out, nullptr, nullptr, opt, task, io);
}

int braxg_step(const braxg_model* m, void* stream, int n_env, int n_frames, const float* act, const braxg_state* in,
               braxg_state* out, const braxg_options* opt) {
  return run_steps(m, stream, n_env, 1, n_frames, act, 0, in, out, nullptr, nullptr, opt);
}

int braxg_rollout(const braxg_model* m, void* stream, int n_env, int n_steps, int n_frames, const float* act_seq,
                  const braxg_state* in, braxg_state* out, float* traj_q, float* traj_qd, const braxg_options* opt) {
  long long stride = m ? (long long)n_env * m->dims.nu : 0;
  return run_steps(m, stream, n_env, n_steps, n_frames, act_seq, stride, in, out, traj_q, traj_qd, opt);
}

}  // extern "C"
