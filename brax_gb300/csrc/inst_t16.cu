// Instantiations of the step kernel for 16 lanes per env, nv <= 16 and nv <= 32.
#include "braxg_kernel.cuh"

template cudaError_t braxg::launch_step<16, 16>(const braxg::StepArgs&, int, int, cudaStream_t);
template cudaError_t braxg::launch_step<16, 32>(const braxg::StepArgs&, int, int, cudaStream_t);
