// Factor once, solve many right-hand sides (and the transposed system):
// Gaussian elimination with partial pivoting, the algorithm of LAPACK
// ?gttrf / ?gttrs, one thread per system.
//
// Factor object (device memory of tridiag_factor_size bytes), all arrays
// batch-interleaved (row i of system j at i*batch + j) so that the threads
// of a warp, each walking its own system, read and write coalesced rows:
//   F0 = 1/u0_i, F1 = u1_i, F2 = u2_i (second superdiagonal, nonzero only
//   after an interchange), FL = l_i (the multiplier of step i), FS = 1 if
//   rows i and i+1 were interchanged at step i.
// Forward elimination of a right-hand side replays the steps E_i:
//   no interchange:  r_{i+1} -= l_i r_i;
//   interchange:     (r_i, r_{i+1}) <- (r_{i+1}, r_i - l_i r_{i+1});
// then U x = r is back-substituted.  The transposed solve A^T z = r solves
// U^T w = r forward, then applies E_{n-2}^T ... E_0^T (E_i^T is E_i with l_i
// moved above the diagonal; the interchange step is symmetric).
#include <cstdint>

#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

template <typename T>
struct Factors {
  T *f0, *f1, *f2, *fl;
  unsigned char* fs;
};

template <typename T>
__host__ __device__ inline size_t factor_bytes(int n, int batch) {
  const size_t e = (size_t)n * (size_t)batch;
  const size_t arr = (e * sizeof(T) + 255) / 256 * 256;
  return 4 * arr + (e + 255) / 256 * 256;
}

template <typename T>
__host__ __device__ inline Factors<T> carve_factors(void* base, int n, int batch) {
  const size_t e = (size_t)n * (size_t)batch;
  const size_t arr = (e * sizeof(T) + 255) / 256 * 256;
  char* p = static_cast<char*>(base);
  Factors<T> f;
  f.f0 = reinterpret_cast<T*>(p);
  f.f1 = reinterpret_cast<T*>(p + arr);
  f.f2 = reinterpret_cast<T*>(p + 2 * arr);
  f.fl = reinterpret_cast<T*>(p + 3 * arr);
  f.fs = reinterpret_cast<unsigned char*>(p + 4 * arr);
  return f;
}

template <typename T, int L>
__global__ void __launch_bounds__(128) factor_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                     const T* __restrict__ c, Factors<T> f, int* info, int n,
                                                     int batch) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  auto at = [&](int i) { return idx<L>(i, j, n, batch); };
  auto fi = [&](int i) { return (size_t)i * (size_t)batch + (size_t)j; };
  int zero = 0;
  T cb = b[at(0)], cc = n > 1 ? c[at(0)] : T(0);
  for (int i = 0; i + 1 < n; ++i) {
    const T na = a[at(i + 1)], nb = b[at(i + 1)];
    const T nc = i + 2 < n ? c[at(i + 1)] : T(0);
    const bool sw = !abs_ge(cb, na);
    const T piv = sw ? na : cb;
    if (is_zero(piv) && !zero) zero = i + 1;
    const T inv = Div<T>(piv).inv();
    const T l = (sw ? cb : na) * inv;
    const T u1 = sw ? nb : cc;
    f.f0[fi(i)] = inv;
    f.f1[fi(i)] = u1;
    f.f2[fi(i)] = sw ? nc : T(0);
    f.fl[fi(i)] = l;
    f.fs[fi(i)] = sw ? 1 : 0;
    cb = fma(-l, u1, sw ? cc : nb);
    cc = fma(-l, sw ? nc : T(0), sw ? T(0) : nc);
  }
  if (is_zero(cb) && !zero) zero = n;
  f.f0[fi(n - 1)] = Div<T>(cb).inv();
  f.f1[fi(n - 1)] = T(0);
  f.f2[fi(n - 1)] = T(0);
  f.fl[fi(n - 1)] = T(0);
  f.fs[fi(n - 1)] = 0;
  if (info) info[j] = zero;
}

// x holds nrhs right-hand sides (block k at k*n*batch, layout L) on entry
// and the solutions on exit.
template <typename T, int L, bool TRANS>
__global__ void __launch_bounds__(128) factored_solve_kernel(const Factors<T> f, T* x, int n, int batch, int nrhs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  auto fi = [&](int i) { return (size_t)i * (size_t)batch + (size_t)j; };
  const size_t block = (size_t)n * (size_t)batch;
  for (int k = 0; k < nrhs; ++k) {
    T* r = x + (size_t)k * block;
    auto at = [&](int i) { return idx<L>(i, j, n, batch); };
    if (!TRANS) {
      // forward: replay the elimination steps
      T cur = r[at(0)];
      for (int i = 0; i + 1 < n; ++i) {
        const T nx = r[at(i + 1)];
        const T l = f.fl[fi(i)];
        const bool sw = f.fs[fi(i)] != 0;
        r[at(i)] = sw ? nx : cur;
        cur = fma(-l, sw ? nx : cur, sw ? cur : nx);
      }
      // back substitution U x = r
      T x1 = cur * f.f0[fi(n - 1)], x2 = T(0);
      r[at(n - 1)] = x1;
      for (int i = n - 2; i >= 0; --i) {
        const T xi = fma(-f.f2[fi(i)], x2, fma(-f.f1[fi(i)], x1, r[at(i)])) * f.f0[fi(i)];
        r[at(i)] = xi;
        x2 = x1;
        x1 = xi;
      }
    } else {
      // U^T w = r (forward)
      T w1 = T(0), w2 = T(0);  // w_{i-1}, w_{i-2}
      T u1p = T(0), u2p = T(0);  // u1_{i-1}, u2_{i-2}
      T u2q = T(0);              // u2_{i-1}
      for (int i = 0; i < n; ++i) {
        const T wi = fma(-u2p, w2, fma(-u1p, w1, r[at(i)])) * f.f0[fi(i)];
        r[at(i)] = wi;
        w2 = w1;
        w1 = wi;
        u2p = u2q;
        u2q = f.f2[fi(i)];
        u1p = f.f1[fi(i)];
      }
      // apply E_{n-2}^T ... E_0^T
      T hi = r[at(n - 1)];  // current value of row i+1
      for (int i = n - 2; i >= 0; --i) {
        const T lo = r[at(i)];
        const T l = f.fl[fi(i)];
        const bool sw = f.fs[fi(i)] != 0;
        // no interchange: lo -= l hi; interchange: (lo, hi) <- (hi, lo - l hi)
        const T nlo = sw ? hi : fma(-l, hi, lo);
        const T nhi = sw ? fma(-l, hi, lo) : hi;
        r[at(i + 1)] = nhi;
        hi = nlo;
      }
      r[at(0)] = hi;
    }
  }
}

template <typename T>
cudaError_t launch_factor(int layout, const T* a, const T* b, const T* c, void* factors, int* info, int n, int batch,
                          cudaStream_t s) {
  const Factors<T> f = carve_factors<T>(factors, n, batch);
  const int grid = (batch + 127) / 128;
  if (layout == INTERLEAVED)
    factor_kernel<T, INTERLEAVED><<<grid, 128, 0, s>>>(a, b, c, f, info, n, batch);
  else if (layout == PACKED)
    factor_kernel<T, PACKED><<<grid, 128, 0, s>>>(a, b, c, f, info, n, batch);
  else
    factor_kernel<T, CONTIG><<<grid, 128, 0, s>>>(a, b, c, f, info, n, batch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_factored_solve(int layout, bool trans, const void* factors, T* x, int n, int batch, int nrhs,
                                  cudaStream_t s) {
  const Factors<T> f = carve_factors<T>(const_cast<void*>(factors), n, batch);
  const int grid = (batch + 127) / 128;
#define TDG_LAUNCH(LAY)                                                                    \
  if (trans)                                                                               \
    factored_solve_kernel<T, LAY, true><<<grid, 128, 0, s>>>(f, x, n, batch, nrhs);       \
  else                                                                                     \
    factored_solve_kernel<T, LAY, false><<<grid, 128, 0, s>>>(f, x, n, batch, nrhs);
  if (layout == INTERLEAVED) {
    TDG_LAUNCH(INTERLEAVED)
  } else if (layout == PACKED) {
    TDG_LAUNCH(PACKED)
  } else {
    TDG_LAUNCH(CONTIG)
  }
#undef TDG_LAUNCH
  return cudaGetLastError();
}

}  // namespace tdg

namespace {

template <typename T>
int factor_entry(int layout, const T* a, const T* b, const T* c, void* factors, size_t bytes, int* info, int n,
                 int batch, cudaStream_t s) {
  if (n <= 0 || batch <= 0 || !a || !factors) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout != TRIDIAG_LAYOUT_CONTIGUOUS && layout != TRIDIAG_LAYOUT_PACKED && layout != TRIDIAG_LAYOUT_INTERLEAVED)
    return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) {
    b = a + n;
    c = a + 2 * (size_t)n;
  } else if (!b || !c) {
    return TRIDIAG_ERR_INVALID_VALUE;
  }
  if (bytes < tdg::factor_bytes<T>(n, batch)) return TRIDIAG_ERR_WORKSPACE;
  return tdg::launch_factor<T>(layout, a, b, c, factors, info, n, batch, s) == cudaSuccess ? TRIDIAG_SUCCESS
                                                                                           : TRIDIAG_ERR_CUDA;
}

template <typename T>
int solve_entry(int layout, int trans, const void* factors, size_t bytes, T* x, int nrhs, int n, int batch,
                cudaStream_t s) {
  if (n <= 0 || batch <= 0 || nrhs <= 0 || !x || !factors) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout != TRIDIAG_LAYOUT_CONTIGUOUS && layout != TRIDIAG_LAYOUT_INTERLEAVED) return TRIDIAG_ERR_NOT_SUPPORTED;
  if (bytes < tdg::factor_bytes<T>(n, batch)) return TRIDIAG_ERR_WORKSPACE;
  return tdg::launch_factored_solve<T>(layout, trans != 0, factors, x, n, batch, nrhs, s) == cudaSuccess
             ? TRIDIAG_SUCCESS
             : TRIDIAG_ERR_CUDA;
}

}  // namespace

extern "C" {

size_t tridiag_factor_size(int precision, int n, int batch) {
  if (n <= 0 || batch <= 0) return 0;
  return precision ? tdg::factor_bytes<double>(n, batch) : tdg::factor_bytes<float>(n, batch);
}
int tridiag_factor_single(int layout, const float* a, const float* b, const float* c, void* factors, size_t bytes,
                          int* info, int n, int batch, void* stream) {
  return factor_entry<float>(layout, a, b, c, factors, bytes, info, n, batch, (cudaStream_t)stream);
}
int tridiag_factor_double(int layout, const double* a, const double* b, const double* c, void* factors, size_t bytes,
                          int* info, int n, int batch, void* stream) {
  return factor_entry<double>(layout, a, b, c, factors, bytes, info, n, batch, (cudaStream_t)stream);
}
int tridiag_factored_solve_single(int layout, int transpose, const void* factors, size_t bytes, float* x, int nrhs,
                                  int n, int batch, void* stream) {
  return solve_entry<float>(layout, transpose, factors, bytes, x, nrhs, n, batch, (cudaStream_t)stream);
}
int tridiag_factored_solve_double(int layout, int transpose, const void* factors, size_t bytes, double* x, int nrhs,
                                  int n, int batch, void* stream) {
  return solve_entry<double>(layout, transpose, factors, bytes, x, nrhs, n, batch, (cudaStream_t)stream);
}

}  // extern "C"
