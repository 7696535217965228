/* song2_k_class_d.cu - one instantiation of the evolver kernel (evolver_kernel<double, MODE_BLOCK, 1>). */
#include "song2_evolver.cuh"

void *song2_kernel_class_d() { return (void *)evolver_kernel<double, MODE_BLOCK, 1>; }
