// Instantiation of the rollout gradient kernel for nv <= 16.
#include "braxg_vjp_kernel.cuh"

template cudaError_t braxg::launch_vjp<32, 16>(const braxg::VjpArgs&, int, int, cudaStream_t);
