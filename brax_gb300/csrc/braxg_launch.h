// Declarations shared by the C ABI translation unit and the kernel
// instantiation units (each instantiation compiles in its own unit).
#pragma once
#include <cuda_runtime.h>

#include "braxg.h"

namespace braxg {

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
  const float* act;
  long long act_step_stride;
  braxg_state out;
  float* traj_q;
  float* traj_qd;
  unsigned long long* prof;
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
  float* seg;           // [ckpt_every * n_frames, n, nq + nv]
  float* traj_q;        // optional forward trajectory [n_steps, n, nq]
  float* traj_qd;       // [n_steps, n, nv]
  int* status;          // [n]
};

// Launches vjp_kernel<T, NVB> (defined in braxg_vjp_kernel.cuh, instantiated
// in inst_vjp_*.cu).
template <int T, int NVB>
cudaError_t launch_vjp(const VjpArgs& a, int grid, int smem, cudaStream_t st);

// Launches step_kernel<T, NVB> (defined in braxg_kernel.cuh, instantiated in
// inst_*.cu).
template <int T, int NVB>
cudaError_t launch_step(const StepArgs& a, int grid, int smem, cudaStream_t st);

}  // namespace braxg
