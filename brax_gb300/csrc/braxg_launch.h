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

// Launches step_kernel<T, NVB> (defined in braxg_kernel.cuh, instantiated in
// inst_*.cu).
template <int T, int NVB>
cudaError_t launch_step(const StepArgs& a, int grid, int smem, cudaStream_t st);

}  // namespace braxg
