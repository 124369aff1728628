// The persistent uneven-batch kernel (one definition, in this unit only).
#include "braxg_kernel.cuh"

namespace braxg {

// Persistent kernel over the work items of an uneven batch (several models,
// each a group of envs): every CTA takes the next item from a global counter
// (items are ordered by decreasing estimated cost), copies that model into
// shared memory and runs its envs with the group's lanes per env.
__device__ __forceinline__ void batch_item(const BatchArgs& ba, const BatchItem& it, int* smem) {
  const BatchGroup& g = ba.groups[it.group];
  for (int i = threadIdx.x; i < g.model_words; i += blockDim.x) smem[i] = g.model[i];
  Layout* sl = reinterpret_cast<Layout*>(smem + al4(g.model_words));
  if (threadIdx.x == 0) {
    const int* w0 = g.model;
    *sl = layout_of(w0);
  }
  __syncthreads();
  float* arena = reinterpret_cast<float*>(smem + al4(g.model_words) + kLayoutWords);
  const int T = g.threads_per_env;
  // the item's arenas must fit the launch's dynamic shared memory and its
  // teams the block; otherwise flag its envs and skip it (host and device
  // compute the same layout, so this never fires when they agree)
  const long long need = 4ll * (al4(g.model_words) + kLayoutWords + (long long)it.count * sl->total);
  if (need > ba.smem_bytes || it.count * T > (int)blockDim.x) {
    int* st = ba.s.out.status;
    for (int e = threadIdx.x; st != nullptr && e < it.count; e += blockDim.x)
      st[g.base.env + it.env0 + e] = BRAXG_ENV_SKIPPED;
    return;
  }
  const int team = threadIdx.x / T;
  const bool active = team < it.count;
  const long long env = active ? (long long)it.env0 + team : it.env0;
  const int nf = g.n_frames;
  if (T == 16) {
    if (g.nvb == 16) run_team<16, 16>(ba.s, g.base, smem, sl, arena, team, env, active, nf);
    else run_team<16, 32>(ba.s, g.base, smem, sl, arena, team, env, active, nf);
  } else {
    if (g.nvb == 16) run_team<32, 16>(ba.s, g.base, smem, sl, arena, team, env, active, nf);
    else if (g.nvb == 32) run_team<32, 32>(ba.s, g.base, smem, sl, arena, team, env, active, nf);
    else run_team<32, 64>(ba.s, g.base, smem, sl, arena, team, env, active, nf);
  }
}

__global__ void __launch_bounds__(512, 1) batch_kernel(const BatchArgs ba) {
  extern __shared__ __align__(16) int smem[];
  __shared__ int next;
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(ba.counter, 1);
    __syncthreads();
    const int item = next;
    if (item >= ba.n_items) return;  // uniform over the CTA
    batch_item(ba, ba.items[item], smem);
    __syncthreads();  // every team is done with this model before the next copy
  }
}

// Largest dynamic shared memory batch_kernel may take: the per-CTA limit less
// its static shared variables.
static cudaError_t batch_smem_limit(int* limit) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, batch_kernel);
  if (e != cudaSuccess) return e;
  *limit = kMaxSmemBytes - (int)fa.sharedSizeBytes;
  return cudaSuccess;
}

cudaError_t launch_batch_kernel(const BatchArgs& a, int grid, int block, int smem, cudaStream_t st) {
  static SmemOptIn opt_in;
  cudaError_t e = opt_in.ensure(batch_kernel, batch_smem_limit);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(a.counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  batch_kernel<<<grid, block, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t batch_kernel_occupancy(int block, int smem, int* ctas_per_sm) {
  int limit = 0;
  cudaError_t e = batch_smem_limit(&limit);
  if (e != cudaSuccess) return e;
  if (smem > limit) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, batch_kernel, block, smem);
}

}  // namespace braxg
