// Microbenchmark: per-SM throughput of FP64/FP32 ops, conversions and HBM streaming.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("ERR %s line %d: %s\n", #x, __LINE__, cudaGetErrorString(e)); return 1; } } while (0)

constexpr int ITERS = 1024;
constexpr int CH = 8;

__device__ unsigned long long g_cycles[4096];

template <int OP>
__global__ void kern(double *out, float *outf, double seed) {
  double x[CH];
  float xf[CH];
  for (int k = 0; k < CH; ++k) { x[k] = seed + threadIdx.x * 1e-3 + k; xf[k] = (float)x[k]; }
  __syncthreads();
  long long t0 = clock64();
  double y = 1.0000001, z = 1e-9;
  float yf = 1.0000001f, zf = 1e-9f;
#pragma unroll 1
  for (int it = 0; it < ITERS; ++it) {
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      if (OP == 0) x[k] = fma(x[k], y, z);                 // DFMA
      else if (OP == 1) xf[k] = fmaf(xf[k], yf, zf);       // FFMA
      else if (OP == 2) x[k] = x[k] * y;                   // DMUL
      else if (OP == 3) { double r; asm volatile("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x[k])); x[k] = r; }
      else if (OP == 4) { float r; asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(xf[k])); xf[k] = r; }
      else if (OP == 5) { float r; asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(x[k])); x[k] = (double)(r + 1.0f) ; }
      else if (OP == 6) { x[k] = __drcp_rn(x[k]); }
      else if (OP == 7) { x[k] = 1.5 / x[k]; }
      else if (OP == 8) { float r; asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(x[k])); xf[k] += r; }
      else if (OP == 9) { double r; asm volatile("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(xf[k])); x[k] += 0.0; xf[k] = xf[k] * 1.0000001f; x[k] = r; }
      else if (OP == 10) { float r; asm volatile("div.approx.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(zf), "f"(xf[k])); xf[k] = r + 1.0f; }
      else if (OP == 11) { x[k] = x[k] + y; }              // DADD
    }
  }
  long long t1 = clock64();
  double s = 0; float sf = 0;
  for (int k = 0; k < CH; ++k) { s += x[k]; sf += xf[k]; }
  if (s == 12345.678) out[0] = s;
  if (sf == 12345.678f) outf[0] = sf;
  if (threadIdx.x == 0) {
    unsigned smid; asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    g_cycles[blockIdx.x] = (unsigned long long)(t1 - t0);
  }
}

__global__ void read_kern(const float4 *__restrict__ p, size_t n, float *out) {
  float4 acc = make_float4(0, 0, 0, 0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float4 v = __ldcs(p + i);
    acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
  }
  if (acc.x + acc.y + acc.z + acc.w == 1234.5f) out[0] = acc.x;
}

__global__ void copy_kern(const float4 *__restrict__ p, float4 *__restrict__ q, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    __stcs(q + i, __ldcs(p + i));
  }
}

template <int OP>
int run(const char *name, int nsm, double *out, float *outf, int ops_per_inner) {
  int threads = 512, blocks = nsm * 4;
  kern<OP><<<blocks, threads>>>(out, outf, 1.0);
  CK(cudaDeviceSynchronize());
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  cudaEventRecord(e0);
  kern<OP><<<blocks, threads>>>(out, outf, 1.0);
  cudaEventRecord(e1);
  CK(cudaEventSynchronize(e1));
  float ms; cudaEventElapsedTime(&ms, e0, e1);
  unsigned long long cyc[4096];
  CK(cudaMemcpyFromSymbol(cyc, g_cycles, sizeof(unsigned long long) * blocks));
  double avgcyc = 0; for (int i = 0; i < blocks; ++i) avgcyc += cyc[i]; avgcyc /= blocks;
  double ops = (double)blocks * threads * ITERS * CH * ops_per_inner;
  // 4 blocks resident per SM (512 threads each = 2048 threads): per-SM ops / block-cycles
  double per_sm_clk = (double)threads * 4 * ITERS * CH * ops_per_inner / avgcyc;
  printf("%-28s %9.3f ms  %10.3f Gop/s  %8.2f op/clk/SM (avg block cycles %.0f)\n", name, ms, ops / ms / 1e6, per_sm_clk, avgcyc);
  return 0;
}

int main() {
  int dev = 0; cudaDeviceProp prop; CK(cudaGetDeviceProperties(&prop, dev));
  printf("device %s SMs %d smem/block optin %zu L2 %d MB\n", prop.name, prop.multiProcessorCount,
         prop.sharedMemPerBlockOptin, prop.l2CacheSize >> 20);
  int nsm = prop.multiProcessorCount;
  double *out; float *outf; CK(cudaMalloc(&out, 64)); CK(cudaMalloc(&outf, 64));
  run<0>("DFMA", nsm, out, outf, 1);
  run<1>("FFMA", nsm, out, outf, 1);
  run<2>("DMUL", nsm, out, outf, 1);
  run<11>("DADD", nsm, out, outf, 1);
  run<3>("rcp.approx.ftz.f64", nsm, out, outf, 1);
  run<4>("rcp.approx.ftz.f32", nsm, out, outf, 1);
  run<10>("div.approx.ftz.f32(+fadd)", nsm, out, outf, 1);
  run<5>("cvt f64->f32 (+f32->f64 +fadd)", nsm, out, outf, 1);
  run<8>("cvt f64->f32 (+fadd)", nsm, out, outf, 1);
  run<9>("cvt f32->f64 (+fmul)", nsm, out, outf, 1);
  run<6>("__drcp_rn", nsm, out, outf, 1);
  run<7>("double div 1.5/x", nsm, out, outf, 1);

  size_t bytes = (size_t)4 << 30;  // 4 GiB
  float4 *p, *q; CK(cudaMalloc(&p, bytes)); CK(cudaMalloc(&q, bytes));
  CK(cudaMemset(p, 0, bytes)); CK(cudaMemset(q, 0, bytes));
  size_t n = bytes / 16;
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    read_kern<<<nsm * 8, 512>>>(p, n, outf);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    printf("read  4 GiB: %.3f ms -> %.1f GB/s\n", ms, bytes / ms / 1e6);
  }
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    copy_kern<<<nsm * 8, 512>>>(p, q, n / 2);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    printf("copy  2 GiB: %.3f ms -> %.1f GB/s (r+w)\n", ms, bytes / ms / 1e6);
  }
  CK(cudaFree(p)); CK(cudaFree(q));
  return 0;
}
