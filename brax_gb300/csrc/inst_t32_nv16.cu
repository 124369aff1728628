// Instantiation of the step kernel for 32 lanes per env, nv <= 16.
#include "braxg_kernel.cuh"

template cudaError_t braxg::launch_step<32, 16>(const braxg::StepArgs&, int, int, cudaStream_t);
