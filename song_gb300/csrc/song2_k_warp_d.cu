/* song2_k_warp_d.cu - one instantiation of the evolver kernel (evolver_kernel<double, MODE_WARP, 0>). */
#include "song2_evolver.cuh"

void *song2_kernel_warp_d() { return (void *)evolver_kernel<double, MODE_WARP, 0>; }
