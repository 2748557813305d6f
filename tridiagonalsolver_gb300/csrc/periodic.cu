// Periodic (cyclic) tridiagonal systems: row 0 couples x_{n-1} through a_0
// and row n-1 couples x_0 through c_{n-1}, i.e. A_p = A' + u v^T with A'
// tridiagonal.  Sherman-Morrison (the classical cyclic reduction of the
// corners, e.g. Press et al., "Numerical Recipes", section 2.7): with
// gamma = -b_0, A' takes b'_0 = b_0 - gamma, b'_{n-1} = b_{n-1} -
// c_{n-1} a_0 / gamma, u = (gamma, 0, ..., 0, c_{n-1}), v = (1, 0, ..., 0,
// a_0 / gamma), and
//     x = y - (v.y / (1 + v.z)) z,   A' y = d,   A' z = u.
// The two tridiagonal solves use this library's batched solvers; the kernels
// here build b' and u (one pass) and combine y and z (one pass).
#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"

namespace tdg {

template <typename T>
__global__ void __launch_bounds__(256) periodic_prep_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                            const T* __restrict__ c, T* bp, T* u, int n, int batch) {
  const size_t total = (size_t)n * (size_t)batch;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % (size_t)n);
    const size_t base = k - i;
    const T gamma = -b[base];
    T bv = b[k], uv = T(0);
    if (i == 0) {
      bv = b[k] - gamma;
      uv = gamma;
    }
    if (i == n - 1) {
      const T alpha = c[base + n - 1], beta = a[base];
      bv = b[k] - alpha * beta / gamma;
      uv = alpha;
    }
    bp[k] = bv;
    u[k] = uv;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) periodic_combine_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                               const T* y, const T* __restrict__ z, T* x, int n,
                                                               int batch) {
  const size_t total = (size_t)n * (size_t)batch;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % (size_t)n);
    const size_t base = k - i;
    const T gamma = -b[base];
    const T bg = a[base] / gamma;  // v_{n-1}
    const T fac = (y[base] + bg * y[base + n - 1]) / (T(1) + z[base] + bg * z[base + n - 1]);
    x[k] = y[k] - fac * z[k];
  }
}

static int grid_for_elems(size_t total) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (total + 255) / 256;
  const size_t cap = (size_t)sms * 16;
  return (int)(want < cap ? (want ? want : 1) : cap);
}

template <typename T>
cudaError_t launch_periodic_prep(const T* a, const T* b, const T* c, T* bp, T* u, int n, int batch, cudaStream_t s) {
  periodic_prep_kernel<T><<<grid_for_elems((size_t)n * batch), 256, 0, s>>>(a, b, c, bp, u, n, batch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_periodic_combine(const T* a, const T* b, const T* y, const T* z, T* x, int n, int batch,
                                    cudaStream_t s) {
  periodic_combine_kernel<T><<<grid_for_elems((size_t)n * batch), 256, 0, s>>>(a, b, y, z, x, n, batch);
  return cudaGetLastError();
}

#define INST(T)                                                                                                   \
  template cudaError_t launch_periodic_prep<T>(const T*, const T*, const T*, T*, T*, int, int, cudaStream_t);     \
  template cudaError_t launch_periodic_combine<T>(const T*, const T*, const T*, const T*, T*, int, int, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
