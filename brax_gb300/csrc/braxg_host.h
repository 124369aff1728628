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
  braxg::Layout L;   // arena with every Jacobian row in shared memory
  // arena whose Jacobian rows beyond the first 32 live in the output state's
  // cache slot; used by the single-model calls whose output carries a cache
  // when it fits more envs per CTA than L (ovf_ok)
  braxg::Layout Lg;
  bool ovf_ok;
  int cache_words;   // floats per env of a cache buffer (either layout)
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
