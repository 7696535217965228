/* song2_k_block_f.cu - one instantiation of the evolver kernel (evolver_kernel<float, MODE_BLOCK, 0>). */
#include "song2_evolver.cuh"

void *song2_kernel_block_f() { return (void *)evolver_kernel<float, MODE_BLOCK, 0>; }
