/* song2_k_block_d.cu - one instantiation of the evolver kernel (evolver_kernel<double, MODE_BLOCK, 0>). */
#include "song2_evolver.cuh"

void *song2_kernel_block_d() { return (void *)evolver_kernel<double, MODE_BLOCK, 0>; }
