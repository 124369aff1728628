// Host-side pieces shared by the C ABI translation units (braxg.cu: models,
// steps, env steps; braxg_grad.cu: rollout gradients; braxg_batch.cu: uneven
// batches): the model handle, launch limits and error reporting.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "braxg.h"
#include "braxg_step.cuh"

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

namespace braxg {
namespace host {

// dynamic shared memory a CTA may take, and threads per CTA of the step
// kernels (launch bound 512 x 1: 128 registers)
constexpr int kMaxSmem = 227 * 1024;
constexpr int kMaxBlock = 512;

// Records the message of a failing call for braxg_last_error (per thread)
// and returns `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
// Kernel launches issued by the calling thread's last call.
void set_launches(int n);

}  // namespace host
}  // namespace braxg
