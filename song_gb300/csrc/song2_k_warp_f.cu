/* song2_k_warp_f.cu - one instantiation of the evolver kernel (evolver_kernel<float, MODE_WARP, 0>). */
#include "song2_evolver.cuh"

void *song2_kernel_warp_f() { return (void *)evolver_kernel<float, MODE_WARP, 0>; }
