// C ABI (include/braxg.h): models, steps, rollouts and env steps.  Rollout
// gradients are in braxg_grad.cu, uneven batches in braxg_batch.cu.
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
#include "braxg_host.h"
#include "braxg_step.cuh"


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {
thread_local std::string g_err;
thread_local int g_launches = 0;
}  // namespace

namespace braxg {
namespace host {

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

void set_launches(int n) { g_launches = n; }

}  // namespace host
}  // namespace braxg

using braxg::host::cuda_fail;
using braxg::host::fail;
using braxg::host::kMaxBlock;
using braxg::host::kMaxSmem;

namespace {

struct Shape {
  int T, NVB, epc, smem;
};


int choose_shape(const braxg_model* m, const braxg_options* opt, int n_env, Shape* s, bool ovf_global = false,
                 bool dyn_dr = false) {
  int nv = m->dims.nv;
  s->NVB = nv <= 16 ? 16 : (nv <= 32 ? 32 : 64);
  // default lanes per env: 16 for small models (nv <= 8: two envs per warp),
  // else 32 (measured on the packaged models, one CTA per SM)
  int T = (opt && opt->threads_per_env) ? opt->threads_per_env : (nv <= 8 ? 16 : 32);
  if (T != 16 && T != 32) return fail(BRAXG_ERR_INVALID, "threads_per_env must be 0, 16 or 32 (got %d)", T);
  if (T == 16 && s->NVB == 64) T = 32;
  s->T = T;
  int model_bytes = (braxg::al4(m->words) + braxg::kLayoutWords) * 4;
  int env_bytes = (dyn_dr ? braxg::layout_of(m->h.data(), ovf_global ? 1 : 0, 1).total
                           : (ovf_global ? m->Lg.total : m->L.total)) * 4;
  int max_epc = kMaxBlock / T;
  int fit = (kMaxSmem - model_bytes) / env_bytes;
  if (fit < 1)
    return fail(BRAXG_ERR_UNSUPPORTED, "model needs %d bytes of shared memory per env; at most %d fit",
                env_bytes, kMaxSmem - model_bytes);
  int epc = (opt && opt->envs_per_cta) ? opt->envs_per_cta : 0;
  if (epc == 0) {
    // default: one CTA per SM holding as many envs as its shared memory and
    // 512 threads allow, so that every warp of the SM runs the same stage's
    // code (the instruction working set of one stage); the batch then takes
    // the fewest waves of such CTAs with its envs spread evenly over every
    // SM of each wave (4096 quadrupeds: 2 waves of 152 CTAs of at most 14
    // envs, not 256 CTAs of 16 whose second wave leaves 48 SMs idle; a batch
    // smaller than one wave is spread over all SMs)
    epc = std::min(fit, max_epc);
    if (n_env > 0 && m->sms > 0) {
      const long long per_wave = (long long)m->sms * epc;
      const long long waves = (n_env + per_wave - 1) / per_wave;
      epc = (int)((n_env + (long long)m->sms * waves - 1) / ((long long)m->sms * waves));
    }
    if (epc < 1) epc = 1;
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
  // Jacobian rows beyond the first 32 go to the output state's cache slots
  // when it has them and that layout fits more envs per CTA
  a.ovf_global = (m->ovf_ok && a.out.cache != nullptr) ? 1 : 0;
  a.cache_stride = m->cache_words;
  if (opt && opt->randomization) {
    const braxg_randomization& r = *opt->randomization;
    a.dyn_dr = (r.link_mass || r.link_inertia || r.dof_armature || r.dof_damping || r.dof_stiffness) ? 1 : 0;
  }
  int rc = choose_shape(m, opt, a.n_env, &s, a.ovf_global != 0, a.dyn_dr != 0);
  if (rc) return rc;
  if (a.n_env == 0) return BRAXG_OK;
  a.envs_per_cta = s.epc;
  a.prof = opt ? opt->stage_cycles : nullptr;
  a.relax = opt ? opt->relax_barriers : 0;
  if (opt && opt->randomization) a.dr = *opt->randomization;
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
  for (int k = BXM_O_LINK_PARENT; k <= BXM_O_LI_BOX; ++k)
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
  m->Lg = braxg::layout_of(w, 1);
  {
    const int model_bytes = (braxg::al4(words) + braxg::kLayoutWords) * 4;
    const int fit_s = (kMaxSmem - model_bytes) / (m->L.total * 4);
    const int fit_g = (kMaxSmem - model_bytes) / (m->Lg.total * 4);
    m->ovf_ok = fit_g > fit_s && m->Lg.total < m->L.total;
    const int ovf_words = (d.m - m->L.jcap) * m->L.ldj;
    m->cache_words = m->ovf_ok ? std::max(m->L.total, braxg::al4(m->Lg.total + ovf_words)) : m->L.total;
    // calls with per-env dynamics parameters lay out a larger arena
    const braxg::Layout Ld = braxg::layout_of(w, 0, 1), Lgd = braxg::layout_of(w, 1, 1);
    m->cache_words = std::max(m->cache_words, Ld.total);
    if (m->ovf_ok) m->cache_words = std::max(m->cache_words, braxg::al4(Lgd.total + ovf_words));
  }
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

int braxg_model_cache_words(const braxg_model* m, int32_t* words) {
  if (m == nullptr || words == nullptr) return fail(BRAXG_ERR_INVALID, "NULL argument");
  *words = m->cache_words;  // the env's arena (and its overflow Jacobian rows)
  return BRAXG_OK;
}

int braxg_model_cache_span(const braxg_model* m, int32_t* fixed_words, int32_t* row_words, int32_t* rows_in_fixed) {
  if (m == nullptr || fixed_words == nullptr || row_words == nullptr || rows_in_fixed == nullptr)
    return fail(BRAXG_ERR_INVALID, "NULL argument");
  const braxg::Layout& L = m->ovf_ok ? m->Lg : m->L;  // the spans copy_position_terms copies (cached calls)
  *fixed_words = L.scr + (L.M >= L.scr ? braxg::al4(m->dims.nv * L.ldm) : 0);
  *row_words = L.ldj;
  *rows_in_fixed = L.jcap;
  return BRAXG_OK;
}

int braxg_launch_shape(const braxg_model* m, const braxg_options* opt, int n_env, int32_t* tpe, int32_t* epc,
                       int32_t* smem) {
  if (m == nullptr) return fail(BRAXG_ERR_INVALID, "model is NULL");
  if (n_env < 0) return fail(BRAXG_ERR_INVALID, "n_env must be >= 0");
  Shape s;
  int rc = choose_shape(m, opt, n_env, &s, m->ovf_ok);  // as for output states with a cache
  if (rc) return rc;
  if (tpe) *tpe = s.T;
  if (epc) *epc = s.epc;
  if (smem) *smem = s.smem;
  return BRAXG_OK;
}

// The caches are read and written with 16-byte vector accesses.
static int check_caches(const braxg_state* in, const braxg_state* out) {
  auto misaligned = [](const float* p) { return p != nullptr && (reinterpret_cast<uintptr_t>(p) & 15) != 0; };
  if ((in && misaligned(in->cache)) || (out && misaligned(out->cache)))
    return fail(BRAXG_ERR_INVALID, "state cache must be 16-byte aligned");
  return BRAXG_OK;
}

int braxg_init(const braxg_model* m, void* stream, int n_env, const float* q, const float* qd, braxg_state* out,
               const braxg_options* opt) {
  int rc = check_common(m, n_env, opt);
  if (rc) return rc;
  if (out == nullptr || (n_env > 0 && (q == nullptr || qd == nullptr)))
    return fail(BRAXG_ERR_INVALID, "q, qd and out are required");
  if ((rc = check_caches(nullptr, out))) return rc;
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
  if ((rc = check_caches(in, out))) return rc;
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
  a.cache_in = in->cache;
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
