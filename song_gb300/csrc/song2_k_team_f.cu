/* song2_k_team_f.cu - one instantiation of the evolver kernel (team_kernel<float>). */
#include "song2_evolver.cuh"

void *song2_kernel_team_f() { return (void *)team_kernel<float>; }
