// PCR-pThomas, one warp per system, everything on chip.
//
// Lane l holds rows l, l+32, l+64, ... (Q rows per lane, rows past n are
// identity rows), so every global load and store of the warp is one
// coalesced row of 32 consecutive elements.  Five PCR steps with strides
// 1, 2, 4, 8, 16 couple each row to the rows 32 above and below it, which
// splits the system into 32 independent chains -- chain l is exactly the
// rows lane l holds -- and each lane then runs the Thomas algorithm on its
// chain in registers.  A PCR step needs, from the rows s above and below,
// a/b, c/b and d/b (three warp shuffles each way per row); a row that is s
// above or below wraps into the neighbouring block of 32 rows, which one
// shuffle of a per-lane selected block handles.
//
// Reference: PCR5_{reg,shmem}_kernel, Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:
// 886-1282 (5 PCR steps over streamed 32-row chunks, then a per-lane Thomas
// on the stride-32 chains, spilling c', d' to global memory), and the CPU
// versions Tridiagonal_AVX512/tridiagonal_d_avx512.cpp:419-646.  The "half"
// variants (4 steps, chains shared by two lanes) are served by the same
// 5-step kernel.
#include "common.cuh"
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

template <typename T, int Q>
__global__ void __launch_bounds__(128) pcr_warp_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                       const T* __restrict__ c, const T* d, T* x, int n, int batch,
                                                       size_t sys_stride) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= batch) return;
  const size_t base = (size_t)j * sys_stride;
  T A[Q], B[Q], C[Q], D[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int r = q * 32 + lane;
    const bool in = r < n;
    A[q] = (in && r > 0) ? __ldg(a + base + r) : T(0);
    B[q] = in ? __ldg(b + base + r) : T(1);
    C[q] = (in && r < n - 1) ? __ldg(c + base + r) : T(0);
    D[q] = in ? d[base + r] : T(0);
  }
  // PCR steps
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    T al[Q], ga[Q], de[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const Div<T> q_(B[q]);
      al[q] = q_.div(A[q]);
      ga[q] = q_.div(C[q]);
      de[q] = q_.div(D[q]);
    }
    const int srcL = (lane - s) & 31, srcR = (lane + s) & 31;
    const bool lowL = lane < 32 - s;  // as a sender: my block feeds the same block on the left side
    const bool lowR = lane >= s;      // as a sender: my block feeds the same block on the right side
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      // row s above: sender lane srcL gives block q if it lies in the same
      // 32-row block, else block q-1 (identity above row 0)
      const T sa = lowL ? al[q] : (q > 0 ? al[q - 1] : T(0));
      const T sg = lowL ? ga[q] : (q > 0 ? ga[q - 1] : T(0));
      const T sd = lowL ? de[q] : (q > 0 ? de[q - 1] : T(0));
      const T aL = shfl(sa, srcL), gL = shfl(sg, srcL), dL = shfl(sd, srcL);
      // row s below: block q, or block q+1 (identity past the last block)
      const T ra = lowR ? al[q] : (q + 1 < Q ? al[q + 1] : T(0));
      const T rg = lowR ? ga[q] : (q + 1 < Q ? ga[q + 1] : T(0));
      const T rd = lowR ? de[q] : (q + 1 < Q ? de[q + 1] : T(0));
      const T aR = shfl(ra, srcR), gR = shfl(rg, srcR), dR = shfl(rd, srcR);
      const T a0 = A[q], c0 = C[q];
      A[q] = -a0 * aL;
      B[q] = fma(-c0, aR, fma(-a0, gL, B[q]));
      C[q] = -c0 * gR;
      D[q] = fma(-c0, dR, fma(-a0, dL, D[q]));
    }
  }
  // Thomas on the lane's chain (rows lane, lane+32, ...)
  T cp = T(0), dp = T(0);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const Div<T> k(fma(-A[q], cp, B[q]));
    cp = k.div(C[q]);
    dp = k.div(fma(-A[q], dp, D[q]));
    C[q] = cp;
    D[q] = dp;
  }
  T xv = T(0);
#pragma unroll
  for (int qq = 0; qq < Q; ++qq) {
    const int q = Q - 1 - qq;
    xv = fma(-C[q], xv, D[q]);
    const int r = q * 32 + lane;
    if (r < n) x[base + r] = xv;
  }
}

template <typename T, int Q>
static cudaError_t launch_pcr_q(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                                size_t stride, cudaStream_t st) {
  const int wpb = 4;
  dim3 grid((batch + wpb - 1) / wpb);
  pcr_warp_kernel<T, Q><<<grid, 32 * wpb, 0, st>>>(a, b, c, d, x, n, batch, stride);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pcr_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                            cudaStream_t st, bool* used) {
  *used = false;
  if (layout != CONTIG && layout != PACKED) return cudaSuccess;
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
