/* song2_k_class2_d.cu - one instantiation of the evolver kernel (evolver_kernel<double, MODE_BLOCK, 1, 2>:
   hierarchy classes, registers for two CTAs per SM). */
#include "song2_evolver.cuh"

void *song2_kernel_class2_d() { return (void *)evolver_kernel<double, MODE_BLOCK, 1, 2>; }
