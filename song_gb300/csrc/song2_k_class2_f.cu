/* song2_k_class2_f.cu - one instantiation of the evolver kernel (evolver_kernel<float, MODE_BLOCK, 1, 2>:
   hierarchy classes, registers for two CTAs per SM). */
#include "song2_evolver.cuh"

void *song2_kernel_class2_f() { return (void *)evolver_kernel<float, MODE_BLOCK, 1, 2>; }
