// Declarations shared by the C ABI translation unit and the kernel
// instantiation units (each instantiation compiles in its own unit).
#pragma once
#include <cuda_runtime.h>

#include <mutex>

#include "braxg.h"

namespace braxg {

// Device ordinals a kernel's one-time attribute set-up tracks.
constexpr int kMaxDevices = 64;

// One kernel's opt-in to more than 48 KB of dynamic shared memory, set once
// per device (the attribute is per device context) under a lock, so that
// first launches from several host threads do not race.  A device ordinal at
// or above kMaxDevices is refused with cudaErrorInvalidDevice rather than
// launched without the attribute.
class SmemOptIn {
 public:
  // `bytes(int*)` computes the attribute's value (called once per device).
  template <class K, class F>
  cudaError_t ensure(K kernel, F bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu_);
    if (done_[dev]) return cudaSuccess;
    int b = 0;
    e = bytes(&b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) done_[dev] = true;
    return e;
  }

 private:
  std::mutex mu_;
  bool done_[kMaxDevices] = {};
};

// Element offsets of a model group's first env inside flat (concatenated)
// batch arrays, one per per-env size class (q: nq, v: nv, vv: nv^2, l: nl,
// u: nu, m: constraint rows, mv: rows x nv); all zero for a single model.
struct EnvBase {
  long long env, q, v, vv, l, u, m, mv;
};

struct StepArgs {
  const int* model;
  int model_words;
  int n_env;
  int n_steps;
  int n_frames;
  int envs_per_cta;
  int exact_inverse;  // Cholesky mode
  int init;
  const float* q_in;
  const float* qd_in;
  const float* minv_in;
  const float* cache_in;   // position-level cache of the input state (or null)
  long long cache_stride;  // words per env of the cache buffers
  int ovf_global;          // Jacobian rows beyond the first 32 in the output cache (Layout::ovf_g)
  const float* act;
  long long act_step_stride;
  braxg_state out;
  float* traj_q;
  float* traj_qd;
  long long traj_q_stride;   // elements between env steps of traj_q
  long long traj_qd_stride;  // and of traj_qd
  unsigned long long* prof;
  int relax;                 // braxg_options.relax_barriers
  braxg_randomization dr;    // per-env System parameters (NULL fields: the model's)
  int dyn_dr;                // the arena holds per-env dynamics parameters (Layout::dprm)
  int has_task;              // fused env step (task, io) after every env step
  long long env_step_stride; // envs between env steps of io.reward / io.done
  braxg_task task;
  braxg_env_io io;
};

// One model group of an uneven batch.
struct BatchGroup {
  const int* model;  // device descriptor
  int model_words;
  int threads_per_env;  // 16 or 32
  int nvb;              // matmul tile bucket: 16, 32 or 64
  int n_frames;         // pipeline steps per env step for this model
  EnvBase base;
};

// A CTA's worth of envs of one group.
struct BatchItem {
  int group, env0, count, pad;
};

struct BatchArgs {
  StepArgs s;  // flat state arrays, flags and strides (model fields unused)
  const BatchGroup* groups;
  const BatchItem* items;
  int n_items;
  int* counter;    // next item; zeroed before each launch
  int smem_bytes;  // dynamic shared memory of the launch
};

struct VjpArgs {
  const int* model;
  int model_words;
  int n_env, n_steps, n_frames, ckpt_every, envs_per_cta;
  const float* act;     // [n_steps, n, nu]
  const float* q0;      // [n, nq]
  const float* qd0;     // [n, nv]
  const float* q_bar;   // [n_steps, n, nq] or null
  const float* qd_bar;  // [n_steps, n, nv] or null
  float* act_bar;       // [n_steps, n, nu]
  float* q0_bar;        // [n, nq]
  float* qd0_bar;       // [n, nv]
  float* ckpt;          // [n_ckpt, n, nq + nv]
  float* seg;           // [ckpt_every * n_frames, n, nq + nv] frame input states
  float* snap;          // [ckpt_every * n_frames, n, snap_words] frame snapshots
  int snap_words;       // forward arena + PG tape words (multiple of 4)
  int resident;         // trailing segments snapshotted by the checkpoint pass (>= 1)
  float* traj_q;        // optional forward trajectory [n_steps, n, nq]
  float* traj_qd;       // [n_steps, n, nv]
  int* status;          // [n]
  unsigned long long* prof;  // optional per-phase cycle counters
  int phases;           // 1: the forward (checkpoints, snapshots, trajectory) only; 2: the
                        // reverse only, from a workspace a phase-1 launch filled; 3: both
  int ckpt_words;       // floats per env of a checkpoint: nq + nv (+ nv * nv in Newton-Schulz mode)
  int ns_iters;         // > 0: Newton-Schulz mode (the carried inverse updated every frame after the first)
  float* nsrec;         // [frames of the snapshot blocks, n, ns_rec_words]: per frame, M and the
                        // carried inverse its update started from
  int ns_rec_words;
  float* nsscr;         // [n, ns_scr_words]: per env, the Newton-Schulz reverse's scratch
  int ns_scr_words;
};

// Launches vjp_kernel<T, NVB> (defined in braxg_vjp_kernel.cuh, instantiated
// in inst_vjp_*.cu).
template <int T, int NVB>
cudaError_t launch_vjp(const VjpArgs& a, int grid, int smem, cudaStream_t st);

// Launches step_kernel<T, NVB> (defined in braxg_kernel.cuh, instantiated in
// inst_*.cu).
template <int T, int NVB>
cudaError_t launch_step(const StepArgs& a, int grid, int smem, cudaStream_t st);

// Launches the persistent batch_kernel (instantiated in inst_batch.cu) after
// zeroing the item counter on the same stream.
cudaError_t launch_batch_kernel(const BatchArgs& a, int grid, int block, int smem, cudaStream_t st);
// Occupancy of batch_kernel: CTAs per SM at this block size and shared memory.
cudaError_t batch_kernel_occupancy(int block, int smem, int* ctas_per_sm);

}  // namespace braxg
