// C ABI: uneven batches (several models in one persistent launch).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "braxg.h"
#include "braxg_host.h"
#include "braxg_launch.h"

using braxg::host::cuda_fail;
using braxg::host::fail;
using braxg::host::kMaxBlock;
using braxg::host::kMaxSmem;

extern "C" {

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
  braxg::host::set_launches(0);
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
  braxg::host::set_launches(1);
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
  s.out.cache = nullptr;  // per-model arena sizes differ: batches keep no cache
  s.out.contact_dist = s.out.contact_pos = s.out.contact_frame = nullptr;  // no per-slot offsets in batches
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
  s.out.cache = nullptr;
  s.out.contact_dist = s.out.contact_pos = s.out.contact_frame = nullptr;
  s.traj_q = traj_q;
  s.traj_qd = traj_qd;
  s.traj_q_stride = tot.q;
  s.traj_qd_stride = tot.qd;
  return batch_launch(b, stream, s, opt);
}

}  // extern "C"
