// PCR-pThomas, one warp per system, everything on chip.
//
// Five PCR steps with strides 1, 2, 4, 8, 16 couple each row to the rows 32
// above and below it, which splits the system into 32 independent chains
// (rows congruent mod 32); the Thomas algorithm then solves each chain.
//
// Placement.  Lane l holds the Q consecutive rows l*Q .. l*Q+Q-1 (rows past
// n are identity rows), so a PCR step of stride s < Q finds most neighbours
// in the lane's own registers: only the s rows at each end of the chunk
// exchange their three normalised values (a/b, c/b, d/b) with the adjacent
// lane, 6 s shuffles per step instead of 6 Q; strides s >= Q are a plain
// shift by s/Q lanes.  At n = 512 (Q = 16) that is 186 shuffles per system
// instead of the 480 a row-interleaved placement needs -- shuffles run on the
// LSU pipe, one warp instruction per clock per SM, and bounded the kernel.
// After the PCR steps the rows go through shared memory (an XOR-swizzled
// index, conflict-free for the chunk-wise writes and the chain-wise reads)
// and lane c runs Thomas on chain c (rows c, c+32, ...), whose solution it
// stores with coalesced 32-row writes.  The step and chain code is in
// pcr.cuh; the steps are shared with the persistent TMA-fed kernel of wm.cu,
// which serves n = 512 (FP32) / 256 (FP64) in the contiguous layout with the
// half variant (four steps, each stride-16 chain solved by two lanes).
//
// Reference: PCR5_{reg,shmem}_kernel, Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:
// 886-1282 (5 PCR steps over streamed 32-row chunks, then a per-lane Thomas
// on the stride-32 chains), and the CPU versions
// Tridiagonal_AVX512/tridiagonal_d_avx512.cpp:419-646.  The "half" variants
// (4 steps, chains shared by two lanes, PCR4_reg_kernel at :1020-1158) are
// served by the same kernels.
#include "common.cuh"
#include "kernels.h"
#include "pcr.cuh"
#include "tw.cuh"

namespace tdg {

constexpr int PCR_WARPS = 4;

template <typename T>
struct PcrVec;
template <>
struct PcrVec<float> {
  using V = float4;
  static constexpr int N = 4;
  __device__ static __forceinline__ float get(const V& v, int k) {
    return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
  }
};
template <>
struct PcrVec<double> {
  using V = double2;
  static constexpr int N = 2;
  __device__ static __forceinline__ double get(const V& v, int k) { return k == 0 ? v.x : v.y; }
};

// Rows [r0, r0 + Q) of one array into registers; rows past n get `fill`, and
// rows 0 / n-1 of a / c are not read (zero).  VEC: whole chunks inside the
// system load as 16-byte vectors.
template <typename T, int Q, bool VEC>
__device__ __forceinline__ void pcr_load(const T* p, int r0, int n, int skip, T fill, T (&v)[Q]) {
  constexpr int NV = PcrVec<T>::N;
  if (VEC && Q % NV == 0 && r0 + Q <= n) {
#pragma unroll
    for (int u = 0; u < Q / NV; ++u) {
      const typename PcrVec<T>::V w = __ldg(reinterpret_cast<const typename PcrVec<T>::V*>(p + r0) + u);
#pragma unroll
      for (int k = 0; k < NV; ++k) v[u * NV + k] = PcrVec<T>::get(w, k);
    }
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = r0 + q < n ? __ldg(p + r0 + q) : fill;
  }
  if (skip >= 0) {
#pragma unroll
    for (int q = 0; q < Q; ++q)
      if (r0 + q == skip) v[q] = T(0);
  }
}

template <typename T, int Q, bool VEC>
__global__ void __launch_bounds__(32 * PCR_WARPS) pcr_warp_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                                  const T* __restrict__ c, const T* d, T* x, int n,
                                                                  int batch, size_t sys_stride) {
  __shared__ T sh[PCR_WARPS][32 * Q];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * PCR_WARPS + w;
  if (j >= batch) return;
  const size_t base = (size_t)j * sys_stride;
  const int r0 = lane * Q;
  T A[Q], B[Q], C[Q], D[Q], X[Q];
  pcr_load<T, Q, VEC>(a + base, r0, n, 0, T(0), A);
  pcr_load<T, Q, VEC>(b + base, r0, n, -1, T(1), B);
  pcr_load<T, Q, VEC>(c + base, r0, n, n - 1, T(0), C);
  pcr_load<T, Q, VEC>(d + base, r0, n, -1, T(0), D);
  pcr_chunk_steps<T, Q>(A, B, C, D, lane);
  pcr_chain_thomas<T, Q>(A, B, C, D, X, lane, sh[w]);
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const int r = lane + 32 * k;
    if (r < n) x[base + r] = X[k];
  }
}

template <typename T, int Q>
static cudaError_t launch_pcr_q(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                                size_t stride, cudaStream_t st) {
  constexpr int WARPS = PCR_WARPS;
  dim3 grid((batch + WARPS - 1) / WARPS);
  constexpr int NV = PcrVec<T>::N;
  const bool vec = Q % NV == 0 && stride % NV == 0 &&
                   ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c) |
                     reinterpret_cast<uintptr_t>(d)) &
                    15u) == 0;
  if (vec)
    pcr_warp_kernel<T, Q, true><<<grid, 32 * WARPS, 0, st>>>(a, b, c, d, x, n, batch, stride);
  else
    pcr_warp_kernel<T, Q, false><<<grid, 32 * WARPS, 0, st>>>(a, b, c, d, x, n, batch, stride);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pcr_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                            cudaStream_t st, bool* used) {
  *used = false;
  if (layout != CONTIG && layout != PACKED) return cudaSuccess;
  cudaError_t e = launch_pcr_tma<T>(layout, a, b, c, d, x, n, batch, st, used);
  if (e != cudaSuccess || *used) return e;
  const size_t stride = layout == PACKED ? 4 * (size_t)n : (size_t)n;
  const int q = (n + 31) / 32;
  const int qmax = sizeof(T) == 4 ? 32 : 16;
  if (q > qmax) return cudaSuccess;
  *used = true;
  if (q <= 1) return launch_pcr_q<T, 1>(a, b, c, d, x, n, batch, stride, st);
  if (q <= 2) return launch_pcr_q<T, 2>(a, b, c, d, x, n, batch, stride, st);
  if (q <= 4) return launch_pcr_q<T, 4>(a, b, c, d, x, n, batch, stride, st);
  if (q <= 8) return launch_pcr_q<T, 8>(a, b, c, d, x, n, batch, stride, st);
  if (q <= 16) return launch_pcr_q<T, 16>(a, b, c, d, x, n, batch, stride, st);
  if constexpr (sizeof(T) == 4) return launch_pcr_q<T, 32>(a, b, c, d, x, n, batch, stride, st);
  *used = false;
  return cudaSuccess;
}

#define INST(T)                                                                                                   \
  template cudaError_t launch_pcr_warp<T>(int, const T*, const T*, const T*, const T*, T*, int, int, cudaStream_t, \
                                          bool*);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
