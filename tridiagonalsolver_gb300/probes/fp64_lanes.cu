// FP64 issue cost per warp instruction with 32, 16, 8 or 4 active lanes and
// 1, 2 or 4 warps per SM sub-partition (eight independent DFMA chains per
// thread).  Result on GB300: 80 cycles per FP64 warp instruction per
// sub-partition regardless of the active lanes.
#include <cstdio>
#include <cuda_runtime.h>
__global__ void dfma_lanes(double* out, int iters, int active) {
  const int lane = threadIdx.x & 31;
  if (lane >= active) return;
  double a0 = lane, a1 = lane + 1, a2 = lane + 2, a3 = lane + 3, a4 = 1, a5 = 2, a6 = 3, a7 = 4;
  const double x = 0.999999, y = 1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, x, y); a1 = fma(a1, x, y); a2 = fma(a2, x, y); a3 = fma(a3, x, y);
    a4 = fma(a4, x, y); a5 = fma(a5, x, y); a6 = fma(a6, x, y); a7 = fma(a7, x, y);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
int main() {
  int sms = 0; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  double* out; cudaMalloc(&out, 1 << 24);
  const int iters = 20000;
  for (int wps : {1, 2, 4}) {           // warps per SM sub-partition
    for (int active : {32, 16, 8, 4}) {
      const int blocks = sms * 4 * wps;  // one-warp CTAs
      dfma_lanes<<<blocks, 32>>>(out, 100, active);
      cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
      cudaEventRecord(e0);
      dfma_lanes<<<blocks, 32>>>(out, iters, active);
      cudaEventRecord(e1); cudaEventSynchronize(e1);
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      const double warp_instr = (double)blocks * iters * 8;
      const double lane_ops = warp_instr * active;
      printf("warps/SMSP %d active %2d: %.3f ms  %.1f Gwarp-instr/s  %.1f Glane-op/s  cycles/warp-instr/SMSP %.1f\n",
             wps, active, ms, warp_instr / ms / 1e6, lane_ops / ms / 1e6,
             2.07e9 * ms * 1e-3 / (iters * 8.0 * wps));
    }
  }
  cudaError_t e = cudaGetLastError();
  printf("%s\n", cudaGetErrorString(e));
  return e != cudaSuccess;
}
