// The reference's vendor row: cuSPARSE ?gtsv2StridedBatch behind the
// reference's cuSparse_* entry points (Tridiagonal_CUDA/tridiagonal_basic.cu:
// 207-246), kept as the GPU library comparator, with the same init / final
// protocol: init creates the handle and the library's workspace, the solve
// is synchronous, final releases both.  This is NVIDIA's library code, not a
// kernel of this project.
#include <cusparse.h>

#include <mutex>

#include "../../include/tridiagonal.h"

namespace {
std::mutex g_mu;
cusparseHandle_t g_handle = nullptr;
void* g_buffer = nullptr;
thread_local int g_vendor_status = 0;

template <typename T>
int init(T* a, T* b, T* c, T* d, int n, int batch) {
  if (n <= 0 || batch <= 0) return TRIDIAG_ERR_INVALID_VALUE;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_handle && cusparseCreate(&g_handle) != CUSPARSE_STATUS_SUCCESS) return TRIDIAG_ERR_CUDA;
  size_t bytes = 0;
  cusparseStatus_t st;
  if constexpr (sizeof(T) == 4)
    st = cusparseSgtsv2StridedBatch_bufferSizeExt(g_handle, n, a, b, c, d, batch, n, &bytes);
  else
    st = cusparseDgtsv2StridedBatch_bufferSizeExt(g_handle, n, a, b, c, d, batch, n, &bytes);
  if (st != CUSPARSE_STATUS_SUCCESS) return TRIDIAG_ERR_CUDA;
  if (g_buffer) cudaFree(g_buffer);
  g_buffer = nullptr;
  if (cudaMalloc(&g_buffer, bytes ? bytes : 256) != cudaSuccess) return TRIDIAG_ERR_CUDA;
  return TRIDIAG_SUCCESS;
}

template <typename T>
int solve(T* a, T* b, T* c, T* d, int n, int batch) {
  if (!g_handle || !g_buffer) return TRIDIAG_ERR_WORKSPACE;
  cusparseStatus_t st;
  if constexpr (sizeof(T) == 4)
    st = cusparseSgtsv2StridedBatch(g_handle, n, a, b, c, d, batch, n, g_buffer);
  else
    st = cusparseDgtsv2StridedBatch(g_handle, n, a, b, c, d, batch, n, g_buffer);
  if (st != CUSPARSE_STATUS_SUCCESS) return TRIDIAG_ERR_CUDA;
  return cudaDeviceSynchronize() == cudaSuccess ? TRIDIAG_SUCCESS : TRIDIAG_ERR_CUDA;
}
}  // namespace

extern "C" {
int cuSparse_init_single(float* a, float* b, float* c, float* d, int n, int batch) {
  return g_vendor_status = init<float>(a, b, c, d, n, batch);
}
int cuSparse_init_double(double* a, double* b, double* c, double* d, int n, int batch) {
  return g_vendor_status = init<double>(a, b, c, d, n, batch);
}
void cuSparse_final(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_buffer) cudaFree(g_buffer);
  g_buffer = nullptr;
  if (g_handle) cusparseDestroy(g_handle);
  g_handle = nullptr;
  g_vendor_status = TRIDIAG_SUCCESS;
}
void cuSparse_single(float* a, float* b, float* c, float* d, int n, int batch) {
  g_vendor_status = solve<float>(a, b, c, d, n, batch);
}
void cuSparse_double(double* a, double* b, double* c, double* d, int n, int batch) {
  g_vendor_status = solve<double>(a, b, c, d, n, batch);
}
int tridiag_vendor_last_status(void) { return g_vendor_status; }
}
