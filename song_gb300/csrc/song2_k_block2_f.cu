/* song2_k_block2_f.cu - one instantiation of the evolver kernel (evolver_kernel<float, MODE_BLOCK, 0, 2>:
   one hierarchy for all triplets, registers for two CTAs per SM). */
#include "song2_evolver.cuh"

void *song2_kernel_block2_f() { return (void *)evolver_kernel<float, MODE_BLOCK, 0, 2>; }
