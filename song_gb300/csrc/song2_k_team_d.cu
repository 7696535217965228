/* song2_k_team_d.cu - one instantiation of the evolver kernel (team_kernel<double>). */
#include "song2_evolver.cuh"

void *song2_kernel_team_d() { return (void *)team_kernel<double>; }
