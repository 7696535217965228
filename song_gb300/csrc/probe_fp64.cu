// FP64 pipe probe: cycles per DFMA for dependent and independent chains, full and partial warps (one SM).
#include <cstdio>
#include <cuda_runtime.h>
template <int CH>
__global__ void k(double *out, long long *cyc, int iters, int active_lanes, double a, double b) {
  int lane = threadIdx.x & 31;
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = 1.0 + threadIdx.x * 1e-3 + c;
  __syncthreads();
  long long t0 = clock64();
  if (lane < active_lanes) {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < CH; ++c) x[c] = fma(x[c], a, b);
    }
  }
  __syncwarp();
  long long t1 = clock64();
  double s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}
template <int CH> void run(int warps, int lanes, int iters) {
  double *o; long long *c;
  cudaMalloc(&o, sizeof(double) * 32 * warps);
  cudaMalloc(&c, sizeof(long long));
  k<CH><<<1, 32 * warps>>>(o, c, iters, lanes, 0.999999, 1e-9);
  k<CH><<<1, 32 * warps>>>(o, c, iters, lanes, 0.999999, 1e-9);
  long long h = 0;
  cudaMemcpy(&h, c, sizeof(h), cudaMemcpyDeviceToHost);
  cudaError_t e = cudaGetLastError();
  printf("warps=%d lanes=%2d chains=%d: %.2f cycles per DFMA per warp-chain-step; SM DFMA instr/cycle=%.4f (%s)\n", warps, lanes, CH,
         (double)h / iters / CH, (double)warps * CH * iters / h, cudaGetErrorString(e));
  cudaFree(o); cudaFree(c);
}
int main() {
  int it = 4096;
  run<1>(1, 32, it); run<1>(1, 1, it);
  run<8>(1, 32, it); run<8>(1, 1, it); run<8>(1, 8, it);
  run<8>(4, 32, it); run<8>(4, 1, it); run<8>(4, 8, it);
  run<8>(8, 32, it); run<8>(8, 1, it);
  run<8>(16, 32, it); run<8>(16, 1, it);
  return 0;
}
