// Layout conversion of whole batches (a, b, c, d together) in one pass over
// HBM: contiguous (system-major, the reference's layout 0), packed
// ([batch][a|b|c|d][n], the reference's layout 1) and interleaved
// (batch-fastest).  A CTA moves a 32-row x 32-system tile of each array
// through shared memory, reading along the source's unit-stride index and
// writing along the destination's, so both sides are coalesced (128-byte
// rows for FP32, two 128-byte segments for FP64); the tile is padded to 33
// columns so the transposed reads are free of bank conflicts.
#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"

namespace tdg {

struct LayoutPtrs {
  const void* src[4];
  void* dst[4];
};

// element offset of (row i, system j) of array k in layout L
template <int L>
__device__ __forceinline__ size_t lay_idx(int i, int j, int k, int n, int batch) {
  if (L == INTERLEAVED) return (size_t)i * (size_t)batch + (size_t)j;
  if (L == PACKED) return (size_t)j * 4u * (size_t)n + (size_t)k * (size_t)n + (size_t)i;
  return (size_t)j * (size_t)n + (size_t)i;
}

template <typename T, int FROM, int TO>
__global__ void __launch_bounds__(256) relayout_kernel(const LayoutPtrs p, int n, int batch) {
  __shared__ T tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  constexpr bool SRC_ROWS_FAST = FROM != INTERLEAVED;  // unit stride along rows
  constexpr bool DST_ROWS_FAST = TO != INTERLEAVED;
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    // PACKED keeps the four arrays in one allocation: array k at base + k*n
    const T* src = static_cast<const T*>(p.src[FROM == PACKED ? 0 : k]);
    T* dst = static_cast<T*>(p.dst[TO == PACKED ? 0 : k]);
#pragma unroll
    for (int r = 0; r < 32; r += 8) {
      const int i = SRC_ROWS_FAST ? i0 + tx : i0 + ty + r;
      const int j = SRC_ROWS_FAST ? j0 + ty + r : j0 + tx;
      if (i < n && j < batch) {
        const T v = src[lay_idx<FROM>(i, j, k, n, batch)];
        if (SRC_ROWS_FAST)
          tile[ty + r][tx] = v;  // [system][row]
        else
          tile[tx][ty + r] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 32; r += 8) {
      const int i = DST_ROWS_FAST ? i0 + tx : i0 + ty + r;
      const int j = DST_ROWS_FAST ? j0 + ty + r : j0 + tx;
      if (i < n && j < batch) dst[lay_idx<TO>(i, j, k, n, batch)] = DST_ROWS_FAST ? tile[ty + r][tx] : tile[tx][ty + r];
    }
    __syncthreads();
  }
}

template <typename T, int FROM, int TO>
static cudaError_t relayout_launch(const LayoutPtrs& p, int n, int batch, cudaStream_t s) {
  const dim3 grid((n + 31) / 32, (batch + 31) / 32);
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  relayout_kernel<T, FROM, TO><<<grid, 256, 0, s>>>(p, n, batch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_relayout(int from, int to, const T* const src[4], T* const dst[4], int n, int batch,
                            cudaStream_t s) {
  LayoutPtrs p;
  for (int k = 0; k < 4; ++k) {
    p.src[k] = src[k];
    p.dst[k] = dst[k];
  }
#define TDG_CASE(F, D) \
  if (from == F && to == D) return relayout_launch<T, F, D>(p, n, batch, s);
  TDG_CASE(CONTIG, CONTIG)
  TDG_CASE(CONTIG, PACKED)
  TDG_CASE(CONTIG, INTERLEAVED)
  TDG_CASE(PACKED, CONTIG)
  TDG_CASE(PACKED, PACKED)
  TDG_CASE(PACKED, INTERLEAVED)
  TDG_CASE(INTERLEAVED, CONTIG)
  TDG_CASE(INTERLEAVED, PACKED)
  TDG_CASE(INTERLEAVED, INTERLEAVED)
#undef TDG_CASE
  return cudaErrorInvalidValue;
}

}  // namespace tdg

namespace {

template <typename T>
int relayout_entry(int from, int to, const T* a, const T* b, const T* c, const T* d, T* a2, T* b2, T* c2, T* d2,
                   int n, int batch, cudaStream_t s) {
  auto ok_layout = [](int l) {
    return l == TRIDIAG_LAYOUT_CONTIGUOUS || l == TRIDIAG_LAYOUT_PACKED || l == TRIDIAG_LAYOUT_INTERLEAVED;
  };
  if (n <= 0 || batch <= 0 || !ok_layout(from) || !ok_layout(to)) return TRIDIAG_ERR_INVALID_VALUE;
  if (!a || !a2) return TRIDIAG_ERR_INVALID_VALUE;
  if (from != TRIDIAG_LAYOUT_PACKED && (!b || !c || !d)) return TRIDIAG_ERR_INVALID_VALUE;
  if (to != TRIDIAG_LAYOUT_PACKED && (!b2 || !c2 || !d2)) return TRIDIAG_ERR_INVALID_VALUE;
  if ((batch + 31) / 32 > 65535) return TRIDIAG_ERR_NOT_SUPPORTED;
  const T* src[4] = {a, b, c, d};
  T* dst[4] = {a2, b2, c2, d2};
  const cudaError_t e = tdg::launch_relayout<T>(from, to, src, dst, n, batch, s);
  return e == cudaSuccess ? TRIDIAG_SUCCESS : TRIDIAG_ERR_CUDA;
}

}  // namespace

extern "C" {

int tridiag_relayout_single(int from_layout, int to_layout, const float* a, const float* b, const float* c,
                            const float* d, float* a2, float* b2, float* c2, float* d2, int n, int batch,
                            void* stream) {
  return relayout_entry<float>(from_layout, to_layout, a, b, c, d, a2, b2, c2, d2, n, batch, (cudaStream_t)stream);
}

int tridiag_relayout_double(int from_layout, int to_layout, const double* a, const double* b, const double* c,
                            const double* d, double* a2, double* b2, double* c2, double* d2, int n, int batch,
                            void* stream) {
  return relayout_entry<double>(from_layout, to_layout, a, b, c, d, a2, b2, c2, d2, n, batch, (cudaStream_t)stream);
}

}  // extern "C"
