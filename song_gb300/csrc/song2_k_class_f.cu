/* song2_k_class_f.cu - one instantiation of the evolver kernel (evolver_kernel<float, MODE_BLOCK, 1>). */
#include "song2_evolver.cuh"

void *song2_kernel_class_f() { return (void *)evolver_kernel<float, MODE_BLOCK, 1>; }
