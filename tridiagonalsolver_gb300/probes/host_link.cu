// Microbenchmark: how fast the SMs read and write page-locked host memory
// (mapped, through the host link), by kernels streaming 16-byte vectors;
// the copy engines' rate is measured by host_link.py.
#include <cstdio>
#include <cuda_runtime.h>
__global__ void rd(const float4* __restrict__ p, size_t n, float* out) {
  float4 acc = make_float4(0, 0, 0, 0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float4 v = __ldcs(p + i);
    acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
  }
  if (acc.x + acc.y + acc.z + acc.w == 1234.5f) out[0] = acc.x;
}
__global__ void wr(float4* __restrict__ p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    __stcs(p + i, make_float4(1, 2, 3, 4));
}
int main() {
  const size_t bytes = 1ull << 30, n = bytes / 16;
  float4 *h, *hd; float* o;
  cudaHostAlloc(&h, bytes, cudaHostAllocMapped);
  cudaHostGetDevicePointer((void**)&hd, h, 0);
  cudaMalloc(&o, 4);
  for (size_t i = 0; i < n; ++i) h[i] = make_float4(1, 1, 1, 1);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  for (int blocks : {152, 304, 608, 1216, 2432}) {
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0); rd<<<blocks, 512>>>(hd, n, o); cudaEventRecord(e1); cudaEventSynchronize(e1);
    }
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    float msw;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0); wr<<<blocks, 512>>>(hd, n); cudaEventRecord(e1); cudaEventSynchronize(e1);
    }
    cudaEventElapsedTime(&msw, e0, e1);
    printf("blocks %5d: SM read of pinned host %.0f GB/s, SM write %.0f GB/s  (%s)\n", blocks, bytes / ms / 1e6,
           bytes / msw / 1e6, cudaGetErrorString(cudaGetLastError()));
  }
  return 0;
}
