// Partial-pivoting solve that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they solve:
// a control loop with a hard latency budget (cudaMalloc may synchronise the
// device and block for milliseconds), or a process whose GPU memory is owned
// by another allocator or a fixed quota taken at start-up, where a side
// cudaMalloc either fails or breaks the owner's accounting.  For them this
// entry point takes only the caller's inputs and outputs; the pivoted
// elimination's scratch (the U1 and 1/U0 spills and the pivot bits) lives in
// one file-scope device array of TRIDIAG_NOALLOC_SCRATCH_BYTES.
//
// Properties a caller must know:
//   * every GPU that loads this library holds the array until the process
//     exits;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it with
//     the device's context; make that first call before any stream capture.
//     A later call in another context of the device (after cudaDeviceReset)
//     looks the address up again, so it too belongs outside a capture;
//   * all calls share the one array, which keeps the last call's contents;
//     the kernel writes every scratch entry before it reads it, so nothing
//     has to be cleared between calls, but calls that overlap on the GPU
//     (different streams, or different host threads without ordering) race
//     on the array and must be serialised by the caller;
//   * problems whose scratch exceeds the array are rejected with
//     TRIDIAG_ERR_WORKSPACE before anything is launched.
// The arithmetic is the one-ended pivoted sweep of seq.cu (the algorithm of
// LAPACK ?gtsv), so results match tridiag_gtsv_* to rounding.
#include <cuda.h>

#include <cstdint>
#include <mutex>

#include "../../include/tridiagonal.h"
#include "kernels.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TRIDIAG_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};
CUcontext g_noalloc_ctx[64] = {};

// The calling thread's current driver context (cuCtxGetCurrent through the
// runtime's driver entry point; no link-time dependency on libcuda).
CUcontext current_context() {
  using Fn = CUresult (*)(CUcontext*);
  static Fn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<Fn>(p);
  });
  CUcontext ctx = nullptr;
  if (fn && fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  return ctx;
}

// Device address of g_noalloc_scratch on the current device (the host-side
// symbol itself is not a device address).  Looked up on the first call on a
// device and again whenever that device's context has changed since (after
// cudaDeviceReset the primary context, and with it the array, is new).
cudaError_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  // bind the device's primary context to this thread (a thread that has made
  // no runtime call yet has none current)
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return e;
  const CUcontext ctx = current_context();
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || ctx != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx[dev] = ctx;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

inline size_t up256(size_t x) { return (x + 255) / 256 * 256; }

template <typename T>
int gtsv_noalloc(int layout, const T* a, const T* b, const T* c, T* d, int* info, int n, int batch,
                 cudaStream_t s) {
  if (n <= 0 || batch <= 0 || !a || !d) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout != TRIDIAG_LAYOUT_CONTIGUOUS && layout != TRIDIAG_LAYOUT_PACKED &&
      layout != TRIDIAG_LAYOUT_INTERLEAVED)
    return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) {
    b = a + n;
    c = a + 2 * (size_t)n;
  } else if (!b || !c) {
    return TRIDIAG_ERR_INVALID_VALUE;
  }
  const size_t elems = (size_t)n * (size_t)batch;
  const size_t spill = up256(elems * sizeof(T));
  const size_t need = 2 * spill + up256(tdg::pivot_words(n, batch) * sizeof(unsigned));
  if (need > (size_t)TRIDIAG_NOALLOC_SCRATCH_BYTES) return TRIDIAG_ERR_WORKSPACE;
  void* base = nullptr;
  if (noalloc_scratch(&base) != cudaSuccess) return TRIDIAG_ERR_CUDA;
  char* p = static_cast<char*>(base);
  T* w1 = reinterpret_cast<T*>(p);
  T* w2 = reinterpret_cast<T*>(p + spill);
  unsigned* piv = reinterpret_cast<unsigned*>(p + 2 * spill);
  cudaError_t e = tdg::launch_gtsv_seq<T>(layout, a, b, c, d, w1, w2, piv, info, n, batch, s);
  return e == cudaSuccess ? TRIDIAG_SUCCESS : TRIDIAG_ERR_CUDA;
}

}  // namespace

extern "C" {

int tridiag_gtsv_noalloc_single(int layout, const float* a, const float* b, const float* c, float* d, int* info,
                                int n, int batch, void* stream) {
  return gtsv_noalloc<float>(layout, a, b, c, d, info, n, batch, (cudaStream_t)stream);
}

int tridiag_gtsv_noalloc_double(int layout, const double* a, const double* b, const double* c, double* d,
                                int* info, int n, int batch, void* stream) {
  return gtsv_noalloc<double>(layout, a, b, c, d, info, n, batch, (cudaStream_t)stream);
}

}  // extern "C"
