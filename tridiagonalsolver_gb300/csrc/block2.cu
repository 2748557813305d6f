// Block tridiagonal systems with 2 x 2 blocks, one thread per system:
//   A_i x_{i-1} + B_i x_i + C_i x_{i+1} = d_i,  i = 0..n-1  (x_i, d_i in R^2),
// A_0 and C_{n-1} are never read.  Blocks are row-major 2 x 2.
//
// Layouts (per array):
//   CONTIG       block (i, j) at a[(j*n + i)*4 + k], right-hand side at
//                d[(j*n + i)*2 + r]: a system's rows are contiguous, so a
//                thread reads one 16-byte (FP32) or 32-byte (FP64) block per
//                row with vector loads, and its next rows lie in the same
//                128-byte line: these loads allocate in L1 (ld.global.ca) so
//                the line serves 4 (FP64) or 8 (FP32) rows, which measured
//                1.2-2.2x faster than streaming loads;
//   INTERLEAVED  a[(i*4 + k)*batch + j], d[(i*2 + r)*batch + j]: a warp reads
//                32 consecutive systems per entry, fully coalesced.
//
// Algorithms:
//   PIVOTED  Gaussian elimination with partial pivoting over the scalar band
//            matrix of order 2n (lower and upper bandwidth 3), the algorithm
//            of LAPACK ?gbsv.  A panel of four scalar rows x six columns
//            (+ right-hand side) lives in registers: the two rows carried
//            from block row i and the two rows of block row i+1; columns 2i
//            and 2i+1 are eliminated with a pivot search over the candidate
//            rows (first row of largest magnitude, compared on the integer
//            bit patterns), the two pivot rows become rows of U (upper
//            bandwidth 5), and the two remaining rows carry on.  U (13
//            values per block row: two pivot reciprocals, nine entries, two
//            right-hand-side values) overwrites A_i, B_i, C_i, d_i, and the
//            back substitution reads it in reverse.  About 50 FP64
//            operations per block row.
//   THOMAS   block Thomas without pivoting: M_i = B_i - A_i C'_{i-1},
//            C'_i = M_i^{-1} C_i, d'_i = M_i^{-1}(d_i - A_i d'_{i-1}) with
//            the 2 x 2 inverse from the adjugate and one reciprocal of the
//            determinant; C' overwrites C and d' overwrites d, then
//            x_i = d'_i - C'_i x_{i+1}.  About 37 FP64 operations per block
//            row; stable for block diagonally dominant systems.
// info[j] = 0, or the first zero pivot (PIVOTED: scalar column, 1-based, as
// LAPACK's INFO) / the first singular M_i (THOMAS: block row, 1-based).  The
// solution of a system with info != 0 is not meaningful.
//
// Input rows stream through a register ring PF rows deep, so the loads of
// the next rows are in flight while the current row's arithmetic runs.
#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

template <typename T>
struct B2Row {
  T a[4], b[4], c[4], d[2];
};

template <typename T, int L, bool VEC>
struct B2Mem {
  int n, batch, j;

  __device__ __forceinline__ size_t o4(int i) const {
    return L == INTERLEAVED ? (size_t)i * 4u * (size_t)batch + (size_t)j : ((size_t)j * (size_t)n + (size_t)i) * 4u;
  }
  __device__ __forceinline__ size_t o2(int i) const {
    return L == INTERLEAVED ? (size_t)i * 2u * (size_t)batch + (size_t)j : ((size_t)j * (size_t)n + (size_t)i) * 2u;
  }
  __device__ __forceinline__ void ld4(const T* p, int i, T (&v)[4]) const {
    const size_t o = o4(i);
    if (L == INTERLEAVED) {
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = ld_stream(p + o + (size_t)k * batch);
    } else if (VEC) {
      vec_ld4(p + o, v);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = __ldca(p + o + k);
    }
  }
  __device__ __forceinline__ void st4(T* p, int i, const T (&v)[4]) const {
    const size_t o = o4(i);
    if (L == INTERLEAVED) {
#pragma unroll
      for (int k = 0; k < 4; ++k) p[o + (size_t)k * batch] = v[k];
    } else if (VEC) {
      vec_st4(p + o, v);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) p[o + k] = v[k];
    }
  }
  __device__ __forceinline__ void ld2(const T* p, int i, T (&v)[2]) const {
    const size_t o = o2(i);
    if (L == INTERLEAVED) {
      v[0] = ld_stream(p + o);
      v[1] = ld_stream(p + o + batch);
    } else if (VEC) {
      vec_ld2(p + o, v);
    } else {
      v[0] = __ldca(p + o);
      v[1] = __ldca(p + o + 1);
    }
  }
  __device__ __forceinline__ void st2(T* p, int i, const T (&v)[2]) const {
    const size_t o = o2(i);
    if (L == INTERLEAVED) {
      p[o] = v[0];
      p[o + batch] = v[1];
    } else if (VEC) {
      vec_st2(p + o, v);
    } else {
      p[o] = v[0];
      p[o + 1] = v[1];
    }
  }

  // vector forms (CONTIG, base pointers 16-byte aligned)
  static __device__ __forceinline__ void vec_ld4(const float* p, float (&v)[4]) {
    const float4 q = __ldca(reinterpret_cast<const float4*>(p));
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  }
  static __device__ __forceinline__ void vec_ld4(const double* p, double (&v)[4]) {
    const double2 q0 = __ldca(reinterpret_cast<const double2*>(p));
    const double2 q1 = __ldca(reinterpret_cast<const double2*>(p) + 1);
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
  }
  static __device__ __forceinline__ void vec_st4(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
  static __device__ __forceinline__ void vec_st4(double* p, const double (&v)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
  }
  static __device__ __forceinline__ void vec_ld2(const float* p, float (&v)[2]) {
    const float2 q = __ldca(reinterpret_cast<const float2*>(p));
    v[0] = q.x; v[1] = q.y;
  }
  static __device__ __forceinline__ void vec_ld2(const double* p, double (&v)[2]) {
    const double2 q = __ldca(reinterpret_cast<const double2*>(p));
    v[0] = q.x; v[1] = q.y;
  }
  static __device__ __forceinline__ void vec_st2(float* p, const float (&v)[2]) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  }
  static __device__ __forceinline__ void vec_st2(double* p, const double (&v)[2]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  }
};

// rows [first, first + PF) of the forward stream, zeros past the end
// (A of row 0 and C of the last row are not read: zeros)
template <typename T, int L, bool VEC, int PF>
__device__ __forceinline__ void b2_fill(const B2Mem<T, L, VEC>& m, const T* a, const T* b, const T* c, const T* d,
                                        int first, B2Row<T> (&ring)[PF]) {
#pragma unroll
  for (int u = 0; u < PF; ++u) {
    const int i = first + u;
    if (i < m.n) {
      if (i > 0) {
        m.ld4(a, i, ring[u].a);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) ring[u].a[k] = T(0);
      }
      m.ld4(b, i, ring[u].b);
      if (i + 1 < m.n) {
        m.ld4(c, i, ring[u].c);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) ring[u].c[k] = T(0);
      }
      m.ld2(d, i, ring[u].d);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) ring[u].a[k] = ring[u].b[k] = ring[u].c[k] = T(0);
      ring[u].d[0] = ring[u].d[1] = T(0);
    }
  }
}

// |x| as an unsigned bit pattern: orders like |x| for finite values and
// infinities (NaN above them)
__device__ __forceinline__ unsigned long long b2_mag(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned b2_mag(float x) { return (unsigned)__float_as_int(x) & 0x7fffffffu; }

// Panel row swap R[q] <-> R[p] for columns q..6 (p in q..3), by selects.
template <typename T>
__device__ __forceinline__ void b2_swap(T (&R)[4][7], int q, int p) {
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    if (k < q) continue;
    const T v = R[q][k];
    T pv = v;
#pragma unroll
    for (int r = 1; r < 4; ++r)
      if (r > q) pv = (p == r) ? R[r][k] : pv;
#pragma unroll
    for (int r = 1; r < 4; ++r)
      if (r > q) R[r][k] = (p == r) ? v : R[r][k];
    R[q][k] = pv;
  }
}

template <typename T, int L, bool VEC, int PF>
__global__ void __launch_bounds__(128) block2_pivoted_kernel(T* __restrict__ a, T* __restrict__ b,
                                                             T* __restrict__ c, T* __restrict__ d, int* info,
                                                             int n, int batch) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  const B2Mem<T, L, VEC> m{n, batch, j};
  int bad = 0;
  T R[4][7];
  {
    B2Row<T> r0[1];
    b2_fill<T, L, VEC, 1>(m, a, b, c, d, 0, r0);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      R[r][0] = r0[0].b[2 * r];
      R[r][1] = r0[0].b[2 * r + 1];
      R[r][2] = r0[0].c[2 * r];
      R[r][3] = r0[0].c[2 * r + 1];
      R[r][4] = T(0);
      R[r][5] = T(0);
      R[r][6] = r0[0].d[r];
    }
  }
  // step i takes block row i+1 into the panel: the ring runs one row ahead
  B2Row<T> ring[PF];
  b2_fill<T, L, VEC, PF>(m, a, b, c, d, 1, ring);
  for (int i0 = 0; i0 < n; i0 += PF) {
    B2Row<T> cur[PF];
#pragma unroll
    for (int u = 0; u < PF; ++u) cur[u] = ring[u];
    b2_fill<T, L, VEC, PF>(m, a, b, c, d, i0 + PF + 1, ring);
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int i = i0 + u;
      if (i >= n) break;
      // block row i+1 enters the panel (zeros past the end)
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        R[2 + r][0] = cur[u].a[2 * r];
        R[2 + r][1] = cur[u].a[2 * r + 1];
        R[2 + r][2] = cur[u].b[2 * r];
        R[2 + r][3] = cur[u].b[2 * r + 1];
        R[2 + r][4] = cur[u].c[2 * r];
        R[2 + r][5] = cur[u].c[2 * r + 1];
        R[2 + r][6] = cur[u].d[r];
      }
      T inv[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        // pivot search on the magnitudes' bit patterns (integer pipe); the
        // pivot value itself is read after the interchange
        int p = q;
        auto bk = b2_mag(R[q][q]);
#pragma unroll
        for (int r = q + 1; r < 4; ++r) {
          const auto k = b2_mag(R[r][q]);
          const bool gt = k > bk;
          bk = gt ? k : bk;
          p = gt ? r : p;
        }
        b2_swap(R, q, p);
        if (bk == 0 && !bad) bad = 2 * i + q + 1;
        inv[q] = Div<T>(R[q][q]).inv();
#pragma unroll
        for (int r = q + 1; r < 4; ++r) {
          const T nl = R[r][q] * -inv[q];
#pragma unroll
          for (int k = q + 1; k < 7; ++k) R[r][k] = fma(nl, R[q][k], R[r][k]);
        }
      }
      // the U row pair of block row i overwrites A_i, B_i, C_i, d_i (all
      // read before: row i entered the panel at step i-1)
      const T ua[4] = {inv[0], R[0][1], R[0][2], R[0][3]};
      const T ub[4] = {R[0][4], R[0][5], inv[1], R[1][2]};
      const T uc[4] = {R[1][3], R[1][4], R[1][5], T(0)};
      const T ud[2] = {R[0][6], R[1][6]};
      m.st4(a, i, ua);
      m.st4(b, i, ub);
      m.st4(c, i, uc);
      m.st2(d, i, ud);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
#pragma unroll
        for (int k = 0; k < 4; ++k) R[r][k] = R[2 + r][k + 2];
        R[r][4] = T(0);
        R[r][5] = T(0);
        R[r][6] = R[2 + r][6];
      }
    }
  }
  if (info) info[j] = bad;
  // back substitution, reading U in reverse; x_{2i+2..2i+5} in registers
  T x2 = T(0), x3 = T(0), x4 = T(0), x5 = T(0);
  for (int i = n - 1; i >= 0; --i) {
    T ua[4], ub[4], uc[4], ud[2];
    m.ld4(a, i, ua);
    m.ld4(b, i, ub);
    m.ld4(c, i, uc);
    m.ld2(d, i, ud);
    const T x1 = fma(-uc[2], x5, fma(-uc[1], x4, fma(-uc[0], x3, fma(-ub[3], x2, ud[1])))) * ub[2];
    const T x0 =
        fma(-ub[1], x5, fma(-ub[0], x4, fma(-ua[3], x3, fma(-ua[2], x2, fma(-ua[1], x1, ud[0]))))) * ua[0];
    const T xo[2] = {x0, x1};
    m.st2(d, i, xo);
    x4 = x2;
    x5 = x3;
    x2 = x0;
    x3 = x1;
  }
}

template <typename T, int L, bool VEC, int PF>
__global__ void __launch_bounds__(128) block2_thomas_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                            T* __restrict__ c, T* __restrict__ d, int* info, int n,
                                                            int batch) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  const B2Mem<T, L, VEC> m{n, batch, j};
  int bad = 0;
  T cp[4] = {T(0), T(0), T(0), T(0)}, dp[2] = {T(0), T(0)};
  B2Row<T> ring[PF];
  b2_fill<T, L, VEC, PF>(m, a, b, c, d, 0, ring);
  for (int i0 = 0; i0 < n; i0 += PF) {
    B2Row<T> cur[PF];
#pragma unroll
    for (int u = 0; u < PF; ++u) cur[u] = ring[u];
    b2_fill<T, L, VEC, PF>(m, a, b, c, d, i0 + PF, ring);
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int i = i0 + u;
      if (i >= n) break;
      const B2Row<T>& w = cur[u];
      // M = B - A C', r = d - A d'  (A_0 = 0)
      const T m0 = fma(-w.a[1], cp[2], fma(-w.a[0], cp[0], w.b[0]));
      const T m1 = fma(-w.a[1], cp[3], fma(-w.a[0], cp[1], w.b[1]));
      const T m2 = fma(-w.a[3], cp[2], fma(-w.a[2], cp[0], w.b[2]));
      const T m3 = fma(-w.a[3], cp[3], fma(-w.a[2], cp[1], w.b[3]));
      const T r0 = fma(-w.a[1], dp[1], fma(-w.a[0], dp[0], w.d[0]));
      const T r1 = fma(-w.a[3], dp[1], fma(-w.a[2], dp[0], w.d[1]));
      const T det = fma(m0, m3, -m1 * m2);
      if (is_zero(det) && !bad) bad = i + 1;
      const T id = Div<T>(det).inv();
      const T v0 = m3 * id, v1 = -m1 * id, v2 = -m2 * id, v3 = m0 * id;
      cp[0] = fma(v1, w.c[2], v0 * w.c[0]);
      cp[1] = fma(v1, w.c[3], v0 * w.c[1]);
      cp[2] = fma(v3, w.c[2], v2 * w.c[0]);
      cp[3] = fma(v3, w.c[3], v2 * w.c[1]);
      dp[0] = fma(v1, r1, v0 * r0);
      dp[1] = fma(v3, r1, v2 * r0);
      if (i + 1 < n) m.st4(c, i, cp);
      m.st2(d, i, dp);
    }
  }
  if (info) info[j] = bad;
  // x_{n-1} = d'_{n-1} is already in place
  T y0 = dp[0], y1 = dp[1];
  for (int i = n - 2; i >= 0; --i) {
    T q[4], e[2];
    m.ld4(c, i, q);
    m.ld2(d, i, e);
    const T x0 = fma(-q[1], y1, fma(-q[0], y0, e[0]));
    const T x1 = fma(-q[3], y1, fma(-q[2], y0, e[1]));
    const T xo[2] = {x0, x1};
    m.st2(d, i, xo);
    y0 = x0;
    y1 = x1;
  }
}

// CTA size: 128 threads, halved (down to one warp) while the grid would give
// fewer than two CTAs per SM, so that small batches still spread over the SMs.
static int block2_threads(int batch) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int bs = 128;
  while (bs > 32 && (batch + bs - 1) / bs < 2 * sms) bs /= 2;
  return bs;
}

template <typename T, int L, bool VEC>
static cudaError_t block2_go(int algo, T* a, T* b, T* c, T* d, int* info, int n, int batch, cudaStream_t s) {
  constexpr int PF = sizeof(T) == 8 ? 1 : 2;
  const int bs = block2_threads(batch);
  const int grid = (batch + bs - 1) / bs;
  if (algo == TRIDIAG_BLOCK2_THOMAS)
    block2_thomas_kernel<T, L, VEC, PF><<<grid, bs, 0, s>>>(a, b, c, d, info, n, batch);
  else
    block2_pivoted_kernel<T, L, VEC, PF><<<grid, bs, 0, s>>>(a, b, c, d, info, n, batch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_block2(int algo, int layout, T* a, T* b, T* c, T* d, int* info, int n, int batch,
                          cudaStream_t s) {
  if (layout == INTERLEAVED) return block2_go<T, INTERLEAVED, false>(algo, a, b, c, d, info, n, batch, s);
  const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c) |
                     reinterpret_cast<uintptr_t>(d)) &
                    15u) == 0;
  return vec ? block2_go<T, CONTIG, true>(algo, a, b, c, d, info, n, batch, s)
             : block2_go<T, CONTIG, false>(algo, a, b, c, d, info, n, batch, s);
}

template cudaError_t launch_block2<float>(int, int, float*, float*, float*, float*, int*, int, int, cudaStream_t);
template cudaError_t launch_block2<double>(int, int, double*, double*, double*, double*, int*, int, int,
                                           cudaStream_t);

}  // namespace tdg

namespace {

template <typename T>
int block2_entry(int algo, int layout, T* a, T* b, T* c, T* d, int* info, int n, int batch, cudaStream_t s) {
  if (n <= 0 || batch <= 0 || !a || !b || !c || !d) return TRIDIAG_ERR_INVALID_VALUE;
  if (algo != TRIDIAG_BLOCK2_PIVOTED && algo != TRIDIAG_BLOCK2_THOMAS) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout != TRIDIAG_LAYOUT_CONTIGUOUS && layout != TRIDIAG_LAYOUT_INTERLEAVED) return TRIDIAG_ERR_NOT_SUPPORTED;
  return tdg::launch_block2<T>(algo, layout, a, b, c, d, info, n, batch, s) == cudaSuccess ? TRIDIAG_SUCCESS
                                                                                          : TRIDIAG_ERR_CUDA;
}

}  // namespace

extern "C" {

int tridiag_block2_single(int algo, int layout, float* a, float* b, float* c, float* d, int* info, int n, int batch,
                          void* stream) {
  return block2_entry<float>(algo, layout, a, b, c, d, info, n, batch, (cudaStream_t)stream);
}

int tridiag_block2_double(int algo, int layout, double* a, double* b, double* c, double* d, int* info, int n,
                          int batch, void* stream) {
  return block2_entry<double>(algo, layout, a, b, c, d, info, n, batch, (cudaStream_t)stream);
}

}  // extern "C"
