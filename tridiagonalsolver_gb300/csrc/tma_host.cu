// Host-side tensor-map encoding through the driver entry point obtained from
// the runtime (no link-time dependency on libcuda).
#include <cudaTypedefs.h>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <mutex>

#include "kernels.h"
#include "tma.cuh"

namespace tdg {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool encode_tmap_2d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype, int elem_bytes, uint64_t inner,
                    uint64_t outer, uint64_t outer_stride_bytes, uint32_t box_inner, uint32_t box_outer,
                    CUtensorMapSwizzle swizzle) {
  // cuTensorMapEncodeTiled needs a current context on the calling thread; a
  // thread that has made no runtime call yet (e.g. an autograd worker) has
  // none, so bind the current device's primary context first.
  thread_local bool bound = false;
  if (!bound) {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess) bound = true;
  }
  auto fn = encode_fn();
  if (!fn || !base) {
    if (std::getenv("TRIDIAG_DEBUG")) std::fprintf(stderr, "tridiag: no tensor-map encoder (%p) or null base\n", (void*)fn);
    return false;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (outer_stride_bytes & 15u) != 0) return false;
  if (outer_stride_bytes < inner * (uint64_t)elem_bytes || inner == 0 || outer == 0) return false;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {outer_stride_bytes};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS && std::getenv("TRIDIAG_DEBUG"))
    std::fprintf(stderr, "tridiag: tensor map refused (CUresult %d): base %p dims %llu x %llu stride %llu box %u x %u\n",
                 (int)r, base, (unsigned long long)inner, (unsigned long long)outer,
                 (unsigned long long)outer_stride_bytes, box_inner, box_outer);
  return r == CUDA_SUCCESS;
}

bool encode_tmap_3d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype, int elem_bytes, uint64_t d0,
                    uint64_t d1, uint64_t d2, uint64_t stride1_bytes, uint64_t stride2_bytes, uint32_t box0,
                    uint32_t box1, uint32_t box2, CUtensorMapSwizzle swizzle) {
  thread_local bool bound = false;
  if (!bound) {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess) bound = true;
  }
  auto fn = encode_fn();
  if (!fn || !base) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (stride1_bytes & 15u) != 0 || (stride2_bytes & 15u) != 0)
    return false;
  if (d0 == 0 || d1 == 0 || d2 == 0 || stride1_bytes < d0 * (uint64_t)elem_bytes || stride2_bytes < stride1_bytes)
    return false;
  cuuint64_t dims[3] = {d0, d1, d2};
  cuuint64_t strides[2] = {stride1_bytes, stride2_bytes};
  cuuint32_t box[3] = {box0, box1, box2};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, dtype, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS && std::getenv("TRIDIAG_DEBUG"))
    std::fprintf(stderr, "tridiag: 3-D tensor map refused (CUresult %d)\n", (int)r);
  return r == CUDA_SUCCESS;
}

static std::mutex g_err_mu;
static int* g_err_words[64] = {};

int* error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_err_mu);
  if (!g_err_words[dev]) {
    int* p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return nullptr;
    g_err_words[dev] = p;
  }
  return g_err_words[dev];
}

static int* g_ring_words[64] = {};
static std::atomic<unsigned> g_ring_seq{0};

int* ring_tickets() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  int* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (!g_ring_words[dev]) {
      int* p = nullptr;
      const size_t bytes = 2 * RING_TICKET_SLOTS * sizeof(int);
      if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
      if (cudaMemset(p, 0, bytes) != cudaSuccess) return nullptr;
      g_ring_words[dev] = p;
    }
    base = g_ring_words[dev];
  }
  return base + 2 * (g_ring_seq.fetch_add(1u) % RING_TICKET_SLOTS);
}

cudaError_t read_device_error(int* code, bool reset) {
  *code = 0;
  int* w = error_word();
  if (!w) return cudaErrorMemoryAllocation;
  cudaError_t e = cudaMemcpy(code, w, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset && *code != 0) e = cudaMemset(w, 0, sizeof(int));
  return e;
}

}  // namespace tdg
