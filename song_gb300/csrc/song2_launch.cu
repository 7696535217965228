/*
 * song2_launch.cu - host side of the evolver kernels: shared-memory plans,
 * occupancy and the launch itself.  The kernels are instantiated in the
 * song2_k_*.cu translation units.
 */
#include "song2_evolver.cuh"

void *song2_kernel_block_f();
void *song2_kernel_block_d();
void *song2_kernel_warp_f();
void *song2_kernel_warp_d();
void *song2_kernel_class_f();
void *song2_kernel_class_d();
void *song2_kernel_class2_f();
void *song2_kernel_class2_d();
void *song2_kernel_block2_f();
void *song2_kernel_block2_d();
void *song2_kernel_team_f();
void *song2_kernel_team_d();

size_t song2_smem_bytes(const DevSpec &spec, int precision, int block, int lu_in_smem) {
  (void)block;
  return make_plan(spec, precision, lu_in_smem).total;
}

size_t song2_class_spec_bytes() { return al(sizeof(DevSpec)); }

size_t song2_team_smem_bytes(const DevSpec &spec, int teams_per_cta) {
  return team_tables_bytes(spec) + sizeof(Shared) * (size_t)teams_per_cta;
}

int song2_team_slab_doubles(const DevSpec &spec) { return make_team_plan(spec).total; }

namespace {
/* mode 0: CTA per triplet; 1: warp per triplet; 2: lane teams; 3: CTA per triplet
   with hierarchy classes; 4: the same with registers for two CTAs per SM; 5: CTA
   per triplet (one hierarchy) with registers for two CTAs per SM */
void *pick_kernel(int precision, int mode) {
  int f = precision == SONG2_PREC_MIXED;
  switch (mode) {
  case 1: return f ? song2_kernel_warp_f() : song2_kernel_warp_d();
  case 2: return f ? song2_kernel_team_f() : song2_kernel_team_d();
  case 3: return f ? song2_kernel_class_f() : song2_kernel_class_d();
  case 4: return f ? song2_kernel_class2_f() : song2_kernel_class2_d();
  case 5: return f ? song2_kernel_block2_f() : song2_kernel_block2_d();
  default: return f ? song2_kernel_block_f() : song2_kernel_block_d();
  }
}
} // namespace

int song2_max_ctas_per_sm(int precision, int mode, int block, size_t smem) {
  int nb = 0;
  const void *f = pick_kernel(precision, mode);
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, block, smem);
  return e == cudaSuccess ? nb : 0;
}

int song2_launch_evolver(const DevSpec &spec, const DevPtrs &ptrs, int precision, int mode, int grid, int block,
                         size_t smem, cudaStream_t stream) {
  if (ptrs.class_spec && mode < 3) mode = 3;
  const void *f = pick_kernel(precision, mode);
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  DevSpec sp = spec;
  DevPtrs pp = ptrs;
  void *args[] = {(void *)&sp, (void *)&pp};
  cudaError_t e = cudaLaunchKernel(f, dim3(grid), dim3(block), args, smem, stream);
  return e == cudaSuccess ? 0 : 1;
}
