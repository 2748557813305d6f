// C ABI of libtridiag.so: argument checking, workspace carving, dispatch to
// the kernel launchers, and the per-thread status of the last call.
// Declarations and contracts: include/tridiagonal.h.
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"

namespace {

thread_local int g_status = TRIDIAG_SUCCESS;

int set_status(int s) {
  g_status = s;
  return s;
}

int cuda_status(cudaError_t e) { return e == cudaSuccess ? TRIDIAG_SUCCESS : TRIDIAG_ERR_CUDA; }

bool valid_dims(int n, int batch) { return n > 0 && batch > 0; }

bool valid_layout(int layout) {
  return layout == TRIDIAG_LAYOUT_CONTIGUOUS || layout == TRIDIAG_LAYOUT_PACKED ||
         layout == TRIDIAG_LAYOUT_INTERLEAVED;
}

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Below this size the thread-per-system sweeps beat the partitioned solve
// (measured on GB300 at batch 2^24 / n: the partitioned solve is faster
// from n = 512 in both precisions, the two-ended sweep below).
constexpr int PGE_MIN_N = 512;
// From this size on FP64 pivoted solves with a workspace run in chunks.
constexpr int PGE_LONG_MIN_FP64 = 12288;

// Expand the four array pointers of a packed (layout 1) base pointer.
template <typename T>
void packed_ptrs(int layout, T*& a, T*& b, T*& c, T*& d, int n) {
  if (layout == TRIDIAG_LAYOUT_PACKED) {
    b = a + n;
    c = a + 2 * (size_t)n;
    d = a + 3 * (size_t)n;
  }
}

// Two arrays of n batch elements, the pivot words, and one int per system
// (the chunked long-system solve's marks).
template <typename T>
size_t gtsv_ws_bytes(int n, int batch) {
  size_t elems = (size_t)n * (size_t)batch;
  return 2 * align_up(elems * sizeof(T)) + align_up(tdg::pivot_words(n, batch) * sizeof(unsigned)) +
         align_up((size_t)batch * sizeof(int));
}

// The workspace tridiag_gtsv_* asks for: FP64 contiguous batches that the
// thread-per-partition solve covers (ppt.cu) get its factor arrays.
template <typename T>
size_t gtsv_ws_query(int layout, int n, int batch) {
  size_t w = gtsv_ws_bytes<T>(n, batch);
  if (sizeof(T) == 8 && tdg::ppt_eligible(layout, n, batch)) w = std::max(w, tdg::ppt_workspace_bytes<T>(n, batch));
  return w;
}

template <typename T>
struct GtsvWs {
  T* w1;
  T* w2;
  unsigned* piv;
  int* flag;
};

template <typename T>
GtsvWs<T> carve_gtsv(void* work, int n, int batch) {
  size_t elems = (size_t)n * (size_t)batch;
  char* p = static_cast<char*>(work);
  GtsvWs<T> w;
  w.w1 = reinterpret_cast<T*>(p);
  p += align_up(elems * sizeof(T));
  w.w2 = reinterpret_cast<T*>(p);
  p += align_up(elems * sizeof(T));
  w.piv = reinterpret_cast<unsigned*>(p);
  p += align_up(tdg::pivot_words(n, batch) * sizeof(unsigned));
  w.flag = reinterpret_cast<int*>(p);
  return w;
}

template <typename T>
int gtsv_impl(int layout, const T* a, const T* b, const T* c, T* d, unsigned* pivots, int* info, void* work,
              size_t work_bytes, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout) || !a || !d) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) {
    b = a + n;
    c = a + 2 * (size_t)n;
  } else if (!b || !c) {
    return TRIDIAG_ERR_INVALID_VALUE;
  }
  if (!work || work_bytes < gtsv_ws_bytes<T>(n, batch)) return TRIDIAG_ERR_WORKSPACE;
  GtsvWs<T> w = carve_gtsv<T>(work, n, batch);
  if (!pivots && sizeof(T) == 8 && tdg::ppt_eligible(layout, n, batch)) {
    // many FP64 systems longer than one CTA holds, up to the clusters'
    // 27648 rows: partitions of a few hundred rows, a thread each, instead of
    // clusters of CTAs or the chunked solve (1.5-2.3x faster, measured on
    // GB300; the systems that miss its acceptance test take the clusters)
    bool used = false;
    cudaError_t e = tdg::launch_ppt<T>(layout, a, b, c, d, d, info, n, batch, work, work_bytes, s, &used);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
    if (used) return TRIDIAG_SUCCESS;
  }
  // Long systems without a pivot record, contiguous: the chunked partitioned
  // solve where the one-CTA and cluster solves do not reach, and for FP64
  // from PGE_LONG_MIN_FP64 rows on (measured on GB300: n = 16384 / 27648 FP64
  // 1.32 / 1.15 ms chunked vs 2.63 / 1.60 ms in clusters; FP32 chunks fail
  // their separator checks too often -- 4-13% of systems -- to replace the
  // clusters).
  const bool chunked_first = sizeof(T) == 8 && n >= PGE_LONG_MIN_FP64;
  if (!pivots && layout == TRIDIAG_LAYOUT_CONTIGUOUS && n >= PGE_MIN_N &&
      (chunked_first || !tdg::pge_eligible<T>(layout, n))) {
    bool used = false;
    cudaError_t e = tdg::launch_pge_long<T>(a, b, c, d, info, n, batch, w.w1, w.w2, w.piv, w.flag, s, &used);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
    if (used) return TRIDIAG_SUCCESS;
  }
  if (!pivots && n >= PGE_MIN_N && tdg::pge_eligible<T>(layout, n)) {
    // no pivot record wanted: the partitioned solve (many chains per system)
    bool used = false;
    cudaError_t e = tdg::launch_pge<T>(layout, a, b, c, d, d, info, n, batch, s, &used);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
    if (used) return TRIDIAG_SUCCESS;
  }
  unsigned* piv = pivots ? pivots : w.piv;
  if (tdg::tw_eligible(layout, n, batch, sizeof(T))) {
    bool used = false;
    cudaError_t e = tdg::launch_gtsv_tw<T>(layout, a, b, c, d, w.w1, w.w2, piv, info, n, batch, s, &used);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
    return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_INVALID_VALUE;  // misaligned base pointer
  }
  return cuda_status(tdg::launch_gtsv_seq<T>(layout, a, b, c, d, w.w1, w.w2, piv, info, n, batch, s));
}

template <typename T>
int adjoint_impl(int layout, const T* a, const T* b, const T* c, const T* x, const unsigned* piv, const T* g,
                 T* ga, T* gb, T* gc, T* gd, void* work, size_t work_bytes, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout)) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) return TRIDIAG_ERR_NOT_SUPPORTED;
  if (!a || !b || !c || !x || !piv || !g || !ga || !gb || !gc || !gd) return TRIDIAG_ERR_INVALID_VALUE;
  if (!work || work_bytes < gtsv_ws_bytes<T>(n, batch)) return TRIDIAG_ERR_WORKSPACE;
  GtsvWs<T> w = carve_gtsv<T>(work, n, batch);
  if (tdg::tw_eligible(layout, n, batch, sizeof(T))) {
    bool used = false;
    cudaError_t e =
        tdg::launch_gtsv_adjoint_tw<T>(layout, a, b, c, x, piv, g, ga, gb, gc, gd, w.w1, w.w2, n, batch, s, &used);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
    return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_INVALID_VALUE;
  }
  return cuda_status(
      tdg::launch_gtsv_adjoint<T>(layout, a, b, c, x, piv, g, ga, gb, gc, gd, w.w1, w.w2, n, batch, s));
}

// Thomas on long contiguous / packed systems in batches too small for one
// thread (two, two-ended) per system to fill the GPU -- every batch in FP32,
// up to 4096 systems in FP64 -- runs as the partition method: one CTA per
// system, the same elimination without pivoting, partition by partition
// (FP64 4096 x 4096: 0.71 ms against 1.07 ms for the two-ended sweep).
template <typename T>
bool thomas_by_partition(int layout, int n, int batch) {
  return layout != TRIDIAG_LAYOUT_INTERLEAVED && n > 1024 && (sizeof(T) == 4 || batch <= 4096);
}

template <typename T>
int solve_impl(int algo, int layout, T* a, T* b, T* c, T* d, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout) || !a) return TRIDIAG_ERR_INVALID_VALUE;
  packed_ptrs(layout, a, b, c, d, n);
  if (!b || !c || !d) return TRIDIAG_ERR_INVALID_VALUE;
  if (algo == TRIDIAG_ALGO_AUTO)
    algo = (n > 1024 && (tdg::wmc_gen_eligible<T>(layout, n) || tdg::wml_eligible<T>(layout, n)))
               ? TRIDIAG_ALGO_PARTITION
               : TRIDIAG_ALGO_THOMAS;
  switch (algo) {
    case TRIDIAG_ALGO_PARTITION: {
      bool used = false;
      cudaError_t e = tdg::launch_wmc<T>(layout, a, b, c, d, d, n, batch, s, &used);
      if (e == cudaSuccess && !used && tdg::wml_eligible<T>(layout, n)) {
        // long systems: the chunked kernels with a stream-ordered workspace
        const size_t bytes = tdg::wml_workspace_bytes<T>(n, batch);
        void* work = nullptr;
        e = cudaMallocAsync(&work, bytes, s);
        if (e == cudaSuccess) {
          e = tdg::launch_wml<T>(a, b, c, d, d, n, batch, work, bytes, s, &used);
          const cudaError_t ef = cudaFreeAsync(work, s);
          if (e == cudaSuccess) e = ef;
        }
      }
      if (e == cudaSuccess && !used) {
        e = tdg::launch_thomas_tw<T>(layout, a, b, c, d, n, batch, s, &used);
        if (e == cudaSuccess && !used) e = tdg::launch_thomas_seq<T>(layout, a, b, c, d, n, batch, s);
      }
      return cuda_status(e);
    }
    case TRIDIAG_ALGO_THOMAS: {
      bool used = false;
      cudaError_t e = cudaSuccess;
      if (thomas_by_partition<T>(layout, n, batch)) e = tdg::launch_wmc<T>(layout, a, b, c, d, d, n, batch, s, &used);
      if (e == cudaSuccess && !used) e = tdg::launch_thomas_tw<T>(layout, a, b, c, d, n, batch, s, &used);
      if (e == cudaSuccess && !used) e = tdg::launch_thomas_seq<T>(layout, a, b, c, d, n, batch, s);
      return cuda_status(e);
    }
    case TRIDIAG_ALGO_CR:
    case TRIDIAG_ALGO_PCR:
    case TRIDIAG_ALGO_WM: {
      bool used = false;
      cudaError_t e = algo == TRIDIAG_ALGO_CR    ? tdg::launch_crpcr_warp<T>(layout, a, b, c, d, d, n, batch, s, &used)
                      : algo == TRIDIAG_ALGO_PCR ? tdg::launch_pcr_warp<T>(layout, a, b, c, d, d, n, batch, s, &used)
                                                 : tdg::launch_wm_warp<T>(layout, a, b, c, d, d, n, batch, s, &used);
      if (e == cudaSuccess && !used && algo == TRIDIAG_ALGO_WM && n >= PGE_MIN_N)
        e = tdg::launch_pge<T>(layout, a, b, c, d, d, nullptr, n, batch, s, &used);
      if (e == cudaSuccess && !used && algo != TRIDIAG_ALGO_WM)
        e = tdg::launch_wmc<T>(layout, a, b, c, d, d, n, batch, s, &used);
      if (e == cudaSuccess && !used) {
        e = tdg::launch_thomas_tw<T>(layout, a, b, c, d, n, batch, s, &used);
        if (e == cudaSuccess && !used) e = tdg::launch_thomas_seq<T>(layout, a, b, c, d, n, batch, s);
      }
      return cuda_status(e);
    }
    case TRIDIAG_ALGO_PGE: {
      bool used = false;
      cudaError_t e = tdg::launch_pge<T>(layout, a, b, c, d, d, nullptr, n, batch, s, &used);
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_NOT_SUPPORTED;
    }
    case TRIDIAG_ALGO_GTSV: {
      size_t bytes = gtsv_ws_query<T>(layout, n, batch);
      void* work = nullptr;
      cudaError_t e = cudaMallocAsync(&work, bytes, s);
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      int st = gtsv_impl<T>(layout == TRIDIAG_LAYOUT_PACKED ? TRIDIAG_LAYOUT_PACKED : layout, a, b, c, d, nullptr,
                            nullptr, work, bytes, n, batch, s);
      e = cudaFreeAsync(work, s);
      if (st == TRIDIAG_SUCCESS && e != cudaSuccess) st = TRIDIAG_ERR_CUDA;
      return st;
    }
    default:
      return TRIDIAG_ERR_INVALID_VALUE;
  }
}

// Out-of-place solve: a, b, c, d untouched, x receives the solution.  The
// on-chip algorithms need no workspace; the sweeps that spill (Thomas) copy
// d into x and use `work` for the c' spill.
// Interleaved Thomas runs the partitioned sweep (ipt.cu), whose factors need
// two n x batch arrays and the partitions' end relations.
template <typename T>
size_t solve_out_ws(int algo, int n, int batch, int layout = TRIDIAG_LAYOUT_CONTIGUOUS) {
  if (algo == TRIDIAG_ALGO_THOMAS) {
    const size_t w = align_up((size_t)n * (size_t)batch * sizeof(T));
    return layout == TRIDIAG_LAYOUT_INTERLEAVED ? std::max(w, tdg::ipt_workspace_bytes<T>(n, batch)) : w;
  }
  if (algo == TRIDIAG_ALGO_GTSV) return gtsv_ws_query<T>(layout, n, batch);
  return 0;
}

template <typename T>
int solve_out_impl(int algo, int layout, const T* a, const T* b, const T* c, const T* d, T* x, void* work,
                   size_t work_bytes, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout) || !a || !b || !c || !d || !x) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) return TRIDIAG_ERR_NOT_SUPPORTED;
  if (algo == TRIDIAG_ALGO_AUTO)
    algo = (n > 1024 && (tdg::wmc_gen_eligible<T>(layout, n) || tdg::wml_eligible<T>(layout, n)))
               ? TRIDIAG_ALGO_PARTITION
               : TRIDIAG_ALGO_WM;
  if (work_bytes < solve_out_ws<T>(algo, n, batch) || (solve_out_ws<T>(algo, n, batch) && !work))
    return TRIDIAG_ERR_WORKSPACE;  // (the interleaved Thomas sweep falls back when given less than it wants)
  switch (algo) {
    case TRIDIAG_ALGO_PARTITION: {
      bool used = false;
      cudaError_t e = tdg::launch_wmc<T>(layout, a, b, c, d, x, n, batch, s, &used);
      if (e == cudaSuccess && !used) e = tdg::launch_wml<T>(a, b, c, d, x, n, batch, work, work_bytes, s, &used);
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      if (used) return TRIDIAG_SUCCESS;
      if (!work || work_bytes < solve_out_ws<T>(TRIDIAG_ALGO_THOMAS, n, batch)) return TRIDIAG_ERR_WORKSPACE;
      return solve_out_impl<T>(TRIDIAG_ALGO_THOMAS, layout, a, b, c, d, x, work, work_bytes, n, batch, s);
    }
    case TRIDIAG_ALGO_CR:
    case TRIDIAG_ALGO_PCR:
    case TRIDIAG_ALGO_WM: {
      bool used = false;
      cudaError_t e = algo == TRIDIAG_ALGO_CR    ? tdg::launch_crpcr_warp<T>(layout, a, b, c, d, x, n, batch, s, &used)
                      : algo == TRIDIAG_ALGO_PCR ? tdg::launch_pcr_warp<T>(layout, a, b, c, d, x, n, batch, s, &used)
                                                 : tdg::launch_wm_warp<T>(layout, a, b, c, d, x, n, batch, s, &used);
      if (e == cudaSuccess && !used && algo == TRIDIAG_ALGO_WM && n >= PGE_MIN_N)
        e = tdg::launch_pge<T>(layout, a, b, c, d, x, nullptr, n, batch, s, &used);
      if (e == cudaSuccess && !used && algo != TRIDIAG_ALGO_WM)
        e = tdg::launch_wmc<T>(layout, a, b, c, d, x, n, batch, s, &used);
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      if (used) return TRIDIAG_SUCCESS;
      if (!work || work_bytes < solve_out_ws<T>(TRIDIAG_ALGO_THOMAS, n, batch)) return TRIDIAG_ERR_WORKSPACE;
      algo = TRIDIAG_ALGO_THOMAS;
    }
      // fall through: shapes beyond the on-chip kernel use the Thomas sweep
    case TRIDIAG_ALGO_THOMAS: {
      if (thomas_by_partition<T>(layout, n, batch)) {
        bool used = false;
        const cudaError_t e = tdg::launch_wmc<T>(layout, a, b, c, d, x, n, batch, s, &used);
        if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
        if (used) return TRIDIAG_SUCCESS;
      }
      if (layout == TRIDIAG_LAYOUT_INTERLEAVED) {
        // partitioned sweep: every SM sub-partition busy for a few thousand systems
        bool used = false;
        const cudaError_t e = tdg::launch_ipt<T>(a, b, c, d, x, n, batch, work, work_bytes, s, &used);
        if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
        if (used) return TRIDIAG_SUCCESS;
      }
      T* cs = static_cast<T*>(work);
      size_t bytes = (size_t)n * (size_t)batch * sizeof(T);
      if (cudaMemcpyAsync(cs, c, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
      if (x != d && cudaMemcpyAsync(x, d, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
      bool used = false;
      cudaError_t e = tdg::launch_thomas_tw<T>(layout, const_cast<T*>(a), const_cast<T*>(b), cs, x, n, batch, s, &used);
      if (e == cudaSuccess && !used)
        e = tdg::launch_thomas_seq<T>(layout, const_cast<T*>(a), const_cast<T*>(b), cs, x, n, batch, s);
      return cuda_status(e);
    }
    case TRIDIAG_ALGO_PGE: {
      bool used = false;
      cudaError_t e = tdg::launch_pge<T>(layout, a, b, c, d, x, nullptr, n, batch, s, &used);
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_NOT_SUPPORTED;
    }
    case TRIDIAG_ALGO_GTSV: {
      bool used = false;
      cudaError_t e = cudaSuccess;
      if (sizeof(T) == 8 && tdg::ppt_eligible(layout, n, batch))
        e = tdg::launch_ppt<T>(layout, a, b, c, d, x, nullptr, n, batch, work, work_bytes, s, &used);
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      if (used) return TRIDIAG_SUCCESS;
      e = n >= PGE_MIN_N ? tdg::launch_pge<T>(layout, a, b, c, d, x, nullptr, n, batch, s, &used) : cudaSuccess;
      if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
      if (used) return TRIDIAG_SUCCESS;
      size_t bytes = (size_t)n * (size_t)batch * sizeof(T);
      if (x != d && cudaMemcpyAsync(x, d, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
      return gtsv_impl<T>(layout, a, b, c, x, nullptr, nullptr, work, work_bytes, n, batch, s);
    }
    default:
      return TRIDIAG_ERR_INVALID_VALUE;
  }
}

// Refined solve workspace: FP32 a, b, c; two FP32 vectors (right-hand side /
// correction, ping-ponged); one FP64 iterate; the FP32 pivoted solve's own
// workspace.
struct RefineWs {
  float *a32, *b32, *c32, *v0, *v1;
  double* w64;
  void* gws;
  size_t gws_bytes;
};

size_t refine_ws_bytes(int n, int batch) {
  const size_t elems = (size_t)n * (size_t)batch;
  return 5 * align_up(elems * sizeof(float)) + align_up(elems * sizeof(double)) + gtsv_ws_bytes<float>(n, batch);
}

RefineWs carve_refine(void* work, int n, int batch) {
  const size_t elems = (size_t)n * (size_t)batch;
  char* p = static_cast<char*>(work);
  RefineWs w;
  float** f[5] = {&w.a32, &w.b32, &w.c32, &w.v0, &w.v1};
  for (float** q : f) {
    *q = reinterpret_cast<float*>(p);
    p += align_up(elems * sizeof(float));
  }
  w.w64 = reinterpret_cast<double*>(p);
  p += align_up(elems * sizeof(double));
  w.gws = p;
  w.gws_bytes = gtsv_ws_bytes<float>(n, batch);
  return w;
}

// The FP32 solve of the refined solve, in place in v: pivoted (GTSV) or the
// unpivoted partition method (PARTITION; the Thomas sweep where neither of
// its kernels covers the shape).
int refine_solve32(int algo, int layout, float* a32, float* b32, float* c32, float* v, int* info, void* gws,
                   size_t gws_bytes, int n, int batch, cudaStream_t s) {
  if (algo != TRIDIAG_ALGO_PARTITION)
    return gtsv_impl<float>(layout, a32, b32, c32, v, nullptr, info, gws, gws_bytes, n, batch, s);
  bool used = false;
  cudaError_t e = tdg::launch_wmc<float>(layout, a32, b32, c32, v, v, n, batch, s, &used);
  if (e == cudaSuccess && !used) e = tdg::launch_wml<float>(a32, b32, c32, v, v, n, batch, gws, gws_bytes, s, &used);
  if (e == cudaSuccess && !used) {
    // Thomas clobbers c: work on a copy (gws holds at least 2 n batch floats)
    float* cs = static_cast<float*>(gws);
    e = cudaMemcpyAsync(cs, c32, (size_t)n * batch * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = tdg::launch_thomas_tw<float>(layout, a32, b32, cs, v, n, batch, s, &used);
    if (e == cudaSuccess && !used) e = tdg::launch_thomas_seq<float>(layout, a32, b32, cs, v, n, batch, s);
  }
  if (info && e == cudaSuccess) e = cudaMemsetAsync(info, 0, (size_t)batch * sizeof(int), s);
  return cuda_status(e);
}

int refine_impl(int algo, int layout, const double* a, const double* b, const double* c, const double* d, double* x,
                int iters, int* info, void* work, size_t work_bytes, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !a || !b || !c || !d || !x || iters < 0 || iters > 8)
    return TRIDIAG_ERR_INVALID_VALUE;
  if (layout != TRIDIAG_LAYOUT_CONTIGUOUS && layout != TRIDIAG_LAYOUT_INTERLEAVED) return TRIDIAG_ERR_NOT_SUPPORTED;
  if (!work || work_bytes < refine_ws_bytes(n, batch)) return TRIDIAG_ERR_WORKSPACE;
  const size_t elems = (size_t)n * (size_t)batch;
  RefineWs w = carve_refine(work, n, batch);
  // FP32 copies; v0 <- d
  if (tdg::launch_narrow4(a, b, c, d, w.a32, w.b32, w.c32, w.v0, elems, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
  // x0: FP32 solve in place in v0
  int st = refine_solve32(algo, layout, w.a32, w.b32, w.c32, w.v0, info, w.gws, w.gws_bytes, n, batch, s);
  if (st != TRIDIAG_SUCCESS) return st;
  // The iterate lives in FP64 (x or w64, alternating so that the last step
  // lands in x); dx holds the latest FP32 solution or correction.
  const double* xcur = nullptr;
  float* dx = w.v0;
  float* spare = w.v1;
  double* xs[2] = {(iters % 2) ? x : w.w64, (iters % 2) ? w.w64 : x};
  for (int it = 0; it < iters; ++it) {
    double* xnew = xs[it % 2];
    if (tdg::launch_residual(layout, a, b, c, d, xcur, dx, xnew, spare, n, batch, s) != cudaSuccess)
      return TRIDIAG_ERR_CUDA;
    st = refine_solve32(algo, layout, w.a32, w.b32, w.c32, spare, nullptr, w.gws, w.gws_bytes, n, batch, s);
    if (st != TRIDIAG_SUCCESS) return st;
    xcur = xnew;
    float* t = dx;
    dx = spare;
    spare = t;
  }
  return cuda_status(tdg::launch_update(xcur, dx, x, elems, s));
}

// Reference-style synchronous wrapper: launch, then wait for the device.
template <typename F>
void sync_call(F&& f) {
  int st = f();
  if (st == TRIDIAG_SUCCESS) st = cuda_status(cudaDeviceSynchronize());
  set_status(st);
}

}  // namespace

extern "C" {

int tridiag_last_status(void) { return g_status; }

const char* tridiag_status_string(int status) {
  switch (status) {
    case TRIDIAG_SUCCESS: return "success";
    case TRIDIAG_ERR_INVALID_VALUE: return "invalid value";
    case TRIDIAG_ERR_NOT_SUPPORTED: return "not supported";
    case TRIDIAG_ERR_CUDA: return "CUDA error";
    case TRIDIAG_ERR_WORKSPACE: return "workspace missing or too small";
    case TRIDIAG_ERR_SINGULAR: return "zero pivot";
    case TRIDIAG_ERR_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

int tridiag_version(void) { return 100; }

int tridiag_device_error(int reset) {
  int code = 0;
  cudaError_t e = tdg::read_device_error(&code, reset != 0);
  if (e != cudaSuccess) return set_status(TRIDIAG_ERR_CUDA);
  return code;
}

// ---- reference entry points ------------------------------------------------

void Thomas_single(float* a, float* b, float* c, float* d, int n, int batch) {
  sync_call([&] { return solve_impl<float>(TRIDIAG_ALGO_THOMAS, TRIDIAG_LAYOUT_CONTIGUOUS, a, b, c, d, n, batch, 0); });
}
void Thomas_double(double* a, double* b, double* c, double* d, int n, int batch) {
  sync_call([&] { return solve_impl<double>(TRIDIAG_ALGO_THOMAS, TRIDIAG_LAYOUT_CONTIGUOUS, a, b, c, d, n, batch, 0); });
}

#define TDG_REF_ENTRY(NAME, T, ALGO)                                                                        \
  void NAME(T* a, T* b, T* c, T* d, int n, int batch) {                                                    \
    sync_call([&] { return solve_impl<T>(ALGO, TRIDIAG_LAYOUT_CONTIGUOUS, a, b, c, d, n, batch, 0); });    \
  }
// WM-pGE -- replace Tridiagonal_CUDA/tridiagonal.h:32,37,42,47 (shmem/reg, 5/4 rounds; kernels
// Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:17-884, wrappers :1437-1569).  All four names run the
// on-chip WM-pGE of wm.cu; the round count of the reference is a tile-shape choice there.
TDG_REF_ENTRY(WM5_shmem_single, float, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM4_shmem_single, float, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM5_reg_single, float, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM4_reg_single, float, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM5_shmem_double, double, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM4_shmem_double, double, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM5_reg_double, double, TRIDIAG_ALGO_WM)
TDG_REF_ENTRY(WM4_reg_double, double, TRIDIAG_ALGO_WM)

// PCR-pThomas -- replace Tridiagonal_CUDA/tridiagonal.h:33-34,38-39,43-44,48-49 (PCR{5,4}_{shmem,reg};
// kernels Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:886-1431).  All run pcr.cu's 5-step PCR-pThomas.
TDG_REF_ENTRY(PCR5_shmem_single, float, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR4_shmem_single, float, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR5_reg_single, float, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR4_reg_single, float, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR5_shmem_double, double, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR4_shmem_double, double, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR5_reg_double, double, TRIDIAG_ALGO_PCR)
TDG_REF_ENTRY(PCR4_reg_double, double, TRIDIAG_ALGO_PCR)

// CR -- replaces Tridiagonal_CUDA/tridiagonal.h:24-28 (kernel Tridiagonal_CUDA/tridiagonal_basic.cu:32-164,
// wrappers :177-204) and the register-packed CR_reg{4,8,16} of tridiagonal.h:50-55 (kernels
// Tridiagonal_CUDA/tridiagonal_onchip.cu:218-820).  All run the on-chip CR-PCR hybrid of wm.cu, which
// needs no scratch: CR_init returns 0 without allocating and CR_final does nothing.
TDG_REF_ENTRY(CR_single, float, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_double, double, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_reg4_single, float, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_reg8_single, float, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_reg16_single, float, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_reg4_double, double, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_reg8_double, double, TRIDIAG_ALGO_CR)
TDG_REF_ENTRY(CR_reg16_double, double, TRIDIAG_ALGO_CR)
int CR_init_single(float*, float*, float*, float*, int n, int batch) {
  return set_status(valid_dims(n, batch) ? TRIDIAG_SUCCESS : TRIDIAG_ERR_INVALID_VALUE);
}
int CR_init_double(double*, double*, double*, double*, int n, int batch) {
  return set_status(valid_dims(n, batch) ? TRIDIAG_SUCCESS : TRIDIAG_ERR_INVALID_VALUE);
}
void CR_final(void) { set_status(TRIDIAG_SUCCESS); }

// BPLG -- replaces Tridiagonal_CUDA/tridiagonal.h:14-17 (the BPLG library's WM / LF / CR / PCR solvers,
// Tridiagonal_CUDA/tridiagonal_third_party.cu:1-41), which take the packed layout 1
// ([batch][a|b|c|d][n], base pointer a; the reference's driver passes a_gbl).  They run this
// library's on-chip kernels on that layout: WM -> WM-pGE, CR and LF -> CR-PCR, PCR -> PCR-pThomas.
#define TDG_BPLG_ENTRY(NAME, ALGO)                                                                          \
  void NAME(float* a, float*, float*, float*, int n, int batch) {                                          \
    sync_call([&] {                                                                                         \
      return solve_impl<float>(ALGO, TRIDIAG_LAYOUT_PACKED, a, nullptr, nullptr, nullptr, n, batch, 0);    \
    });                                                                                                     \
  }
TDG_BPLG_ENTRY(BPLG_WM, TRIDIAG_ALGO_WM)
TDG_BPLG_ENTRY(BPLG_LF, TRIDIAG_ALGO_CR)
TDG_BPLG_ENTRY(BPLG_CR, TRIDIAG_ALGO_CR)
TDG_BPLG_ENTRY(BPLG_PCR, TRIDIAG_ALGO_PCR)

// ---- extensions ---------------------------------------------------------------

int tridiag_solve_single(int algo, int layout, float* a, float* b, float* c, float* d, int n, int batch,
                         void* stream) {
  return set_status(solve_impl<float>(algo, layout, a, b, c, d, n, batch, (cudaStream_t)stream));
}
int tridiag_solve_double(int algo, int layout, double* a, double* b, double* c, double* d, int n, int batch,
                         void* stream) {
  return set_status(solve_impl<double>(algo, layout, a, b, c, d, n, batch, (cudaStream_t)stream));
}

size_t tridiag_solve_out_workspace_size(int precision, int algo, int layout, int n, int batch) {
  if (!valid_dims(n, batch)) return 0;
  if (algo == TRIDIAG_ALGO_AUTO || algo == TRIDIAG_ALGO_WM || algo == TRIDIAG_ALGO_CR || algo == TRIDIAG_ALGO_PCR ||
      algo == TRIDIAG_ALGO_PARTITION)
    algo = TRIDIAG_ALGO_THOMAS;  // possible fallback
  return precision ? solve_out_ws<double>(algo, n, batch, layout) : solve_out_ws<float>(algo, n, batch, layout);
}

int tridiag_solve_out_single(int algo, int layout, const float* a, const float* b, const float* c, const float* d,
                             float* x, void* work, size_t work_bytes, int n, int batch, void* stream) {
  return set_status(solve_out_impl<float>(algo, layout, a, b, c, d, x, work, work_bytes, n, batch, (cudaStream_t)stream));
}
int tridiag_solve_out_double(int algo, int layout, const double* a, const double* b, const double* c,
                             const double* d, double* x, void* work, size_t work_bytes, int n, int batch,
                             void* stream) {
  return set_status(solve_out_impl<double>(algo, layout, a, b, c, d, x, work, work_bytes, n, batch, (cudaStream_t)stream));
}

size_t tridiag_gtsv_workspace_size(int precision, int layout, int n, int batch) {
  if (!valid_dims(n, batch)) return 0;
  return precision ? gtsv_ws_query<double>(layout, n, batch) : gtsv_ws_query<float>(layout, n, batch);
}

size_t tridiag_pivot_record_size(int n, int batch) {
  if (!valid_dims(n, batch)) return 0;
  return tdg::pivot_words(n, batch) * sizeof(unsigned);
}

int tridiag_gtsv_single(int layout, const float* a, const float* b, const float* c, float* d, unsigned* pivots,
                        int* info, void* work, size_t work_bytes, int n, int batch, void* stream) {
  return set_status(gtsv_impl<float>(layout, a, b, c, d, pivots, info, work, work_bytes, n, batch,
                                     (cudaStream_t)stream));
}
int tridiag_gtsv_double(int layout, const double* a, const double* b, const double* c, double* d,
                        unsigned* pivots, int* info, void* work, size_t work_bytes, int n, int batch,
                        void* stream) {
  return set_status(gtsv_impl<double>(layout, a, b, c, d, pivots, info, work, work_bytes, n, batch,
                                      (cudaStream_t)stream));
}

int tridiag_gtsv_adjoint_single(int layout, const float* a, const float* b, const float* c, const float* x,
                                const unsigned* piv, const float* g, float* ga, float* gb, float* gc, float* gd,
                                void* work, size_t work_bytes, int n, int batch, void* stream) {
  return set_status(adjoint_impl<float>(layout, a, b, c, x, piv, g, ga, gb, gc, gd, work, work_bytes, n, batch,
                                        (cudaStream_t)stream));
}
int tridiag_gtsv_adjoint_double(int layout, const double* a, const double* b, const double* c, const double* x,
                                const unsigned* piv, const double* g, double* ga, double* gb, double* gc,
                                double* gd, void* work, size_t work_bytes, int n, int batch, void* stream) {
  return set_status(adjoint_impl<double>(layout, a, b, c, x, piv, g, ga, gb, gc, gd, work, work_bytes, n, batch,
                                         (cudaStream_t)stream));
}

}  // extern "C"

extern "C" {

size_t tridiag_refine_workspace_size(int layout, int n, int batch) {
  (void)layout;
  if (!valid_dims(n, batch)) return 0;
  return refine_ws_bytes(n, batch);
}

int tridiag_refine_double(int layout, const double* a, const double* b, const double* c, const double* d,
                          double* x, int iters, int* info, void* work, size_t work_bytes, int n, int batch,
                          void* stream) {
  return set_status(refine_impl(TRIDIAG_ALGO_GTSV, layout, a, b, c, d, x, iters, info, work, work_bytes, n, batch,
                                (cudaStream_t)stream));
}

int tridiag_refine_ex_double(int algo, int layout, const double* a, const double* b, const double* c,
                             const double* d, double* x, int iters, int* info, void* work, size_t work_bytes, int n,
                             int batch, void* stream) {
  if (algo != TRIDIAG_ALGO_GTSV && algo != TRIDIAG_ALGO_PARTITION && algo != TRIDIAG_ALGO_AUTO)
    return set_status(TRIDIAG_ERR_INVALID_VALUE);
  if (algo == TRIDIAG_ALGO_AUTO) algo = TRIDIAG_ALGO_GTSV;
  return set_status(refine_impl(algo, layout, a, b, c, d, x, iters, info, work, work_bytes, n, batch,
                                (cudaStream_t)stream));
}

int tridiag_convert_check(const double* in, float* out, double* back, size_t count, void* stream) {
  if (!in || !out || !back) return set_status(TRIDIAG_ERR_INVALID_VALUE);
  if (count == 0) return set_status(TRIDIAG_SUCCESS);
  return set_status(cuda_status(tdg::launch_convert_probe(in, out, back, count, (cudaStream_t)stream)));
}

}  // extern "C"

extern "C" long long tridiag_partition_fallbacks(int reset) {
  unsigned long long v = 0;
  if (tdg::pge_fallback_count(&v, reset != 0) != cudaSuccess) return -1;
  return (long long)v;
}

extern "C" int tridiag_partition_path_counts(long long* counts, int reset) {
  if (!counts) return set_status(TRIDIAG_ERR_INVALID_VALUE);
  unsigned long long v[4] = {0ull, 0ull, 0ull, 0ull};
  const cudaError_t e = tdg::pge_path_counts(v, reset != 0);
  if (e != cudaSuccess) return set_status(cuda_status(e));
  for (int k = 0; k < 4; ++k) counts[k] = (long long)v[k];
  return set_status(TRIDIAG_SUCCESS);
}

extern "C" int tridiag_partition_ppt_counts(long long* counts, int reset) {
  if (!counts) return set_status(TRIDIAG_ERR_INVALID_VALUE);
  unsigned long long v[2] = {0ull, 0ull};
  const cudaError_t e = tdg::ppt_counts(v, reset != 0);
  if (e != cudaSuccess) return set_status(cuda_status(e));
  counts[0] = (long long)v[0];
  counts[1] = (long long)v[1];
  return set_status(TRIDIAG_SUCCESS);
}

namespace {
template <typename T>
int pge_entry(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
              cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout) || !a || !x) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) {
    b = a + n;
    c = a + 2 * (size_t)n;
    d = a + 3 * (size_t)n;
  } else if (!b || !c || !d) {
    return TRIDIAG_ERR_INVALID_VALUE;
  }
  bool used = false;
  cudaError_t e = tdg::launch_pge<T>(layout, a, b, c, d, x, info, n, batch, s, &used);
  if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
  return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_NOT_SUPPORTED;
}
}  // namespace

extern "C" int tridiag_pge_single(int layout, const float* a, const float* b, const float* c, const float* d,
                                  float* x, int* info, int n, int batch, void* stream) {
  return set_status(pge_entry<float>(layout, a, b, c, d, x, info, n, batch, (cudaStream_t)stream));
}
extern "C" int tridiag_pge_double(int layout, const double* a, const double* b, const double* c, const double* d,
                                  double* x, int* info, int n, int batch, void* stream) {
  return set_status(pge_entry<double>(layout, a, b, c, d, x, info, n, batch, (cudaStream_t)stream));
}

namespace {
template <typename T>
int pge_adjoint_entry(int layout, const T* a, const T* b, const T* c, const T* x, const T* xbar, T* ga, T* gb, T* gc,
                      T* gd, int* info, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout)) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) return TRIDIAG_ERR_NOT_SUPPORTED;
  if (!a || !b || !c || !x || !xbar || !ga || !gb || !gc || !gd) return TRIDIAG_ERR_INVALID_VALUE;
  bool used = false;
  cudaError_t e = tdg::launch_pge_adjoint<T>(layout, a, b, c, x, xbar, ga, gb, gc, gd, info, n, batch, s, &used);
  if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
  return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_NOT_SUPPORTED;
}
}  // namespace

extern "C" int tridiag_pge_adjoint_single(int layout, const float* a, const float* b, const float* c, const float* x,
                                          const float* xbar, float* ga, float* gb, float* gc, float* gd, int* info,
                                          int n, int batch, void* stream) {
  return set_status(pge_adjoint_entry<float>(layout, a, b, c, x, xbar, ga, gb, gc, gd, info, n, batch,
                                             (cudaStream_t)stream));
}
extern "C" int tridiag_pge_adjoint_double(int layout, const double* a, const double* b, const double* c,
                                          const double* x, const double* xbar, double* ga, double* gb, double* gc,
                                          double* gd, int* info, int n, int batch, void* stream) {
  return set_status(pge_adjoint_entry<double>(layout, a, b, c, x, xbar, ga, gb, gc, gd, info, n, batch,
                                              (cudaStream_t)stream));
}

namespace {
template <typename T>
int partition_adjoint_entry(int layout, const T* a, const T* b, const T* c, const T* x, const T* xbar, T* ga, T* gb,
                            T* gc, T* gd, int n, int batch, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout)) return TRIDIAG_ERR_INVALID_VALUE;
  if (!a || !b || !c || !x || !xbar || !ga || !gb || !gc || !gd) return TRIDIAG_ERR_INVALID_VALUE;
  if (layout != TRIDIAG_LAYOUT_CONTIGUOUS) return TRIDIAG_ERR_NOT_SUPPORTED;
  bool used = false;
  cudaError_t e = tdg::launch_wmc_adjoint<T>(a, b, c, x, xbar, ga, gb, gc, gd, n, batch, s, &used);
  if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
  return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_NOT_SUPPORTED;
}
}  // namespace

extern "C" int tridiag_partition_supported(int precision, int layout, int n) {
  return precision ? (int)tdg::wmc_gen_eligible<double>(layout, n) : (int)tdg::wmc_gen_eligible<float>(layout, n);
}
extern "C" int tridiag_partition_adjoint_single(int layout, const float* a, const float* b, const float* c,
                                                const float* x, const float* xbar, float* ga, float* gb, float* gc,
                                                float* gd, int n, int batch, void* stream) {
  return set_status(
      partition_adjoint_entry<float>(layout, a, b, c, x, xbar, ga, gb, gc, gd, n, batch, (cudaStream_t)stream));
}
extern "C" int tridiag_partition_adjoint_double(int layout, const double* a, const double* b, const double* c,
                                                const double* x, const double* xbar, double* ga, double* gb,
                                                double* gc, double* gd, int n, int batch, void* stream) {
  return set_status(
      partition_adjoint_entry<double>(layout, a, b, c, x, xbar, ga, gb, gc, gd, n, batch, (cudaStream_t)stream));
}

// ---------------------------------------------------------------------------
// cuSPARSE-shaped entry points: the argument lists of cusparse?gtsv2StridedBatch
// and cusparse?gtsvInterleavedBatch (the reference's vendor row,
// Tridiagonal_CUDA/tridiagonal_basic.cu:207-246), served by this library's
// kernels, so code written against those calls switches by renaming them.
namespace {

template <typename T>
size_t gtsv2_strided_ws(int m, int batch, int stride) {
  if (m <= 0 || batch <= 0 || stride < m) return 0;
  return stride == m ? solve_out_ws<T>(TRIDIAG_ALGO_THOMAS, m, batch) : 0;
}

template <typename T>
int gtsv2_strided_impl(int m, const T* dl, const T* d, const T* du, T* x, int batch, int stride, void* buf,
                       cudaStream_t s) {
  if (m <= 0 || batch <= 0 || stride < m || !dl || !d || !du || !x) return TRIDIAG_ERR_INVALID_VALUE;
  if (stride == m)
    return solve_out_impl<T>(TRIDIAG_ALGO_WM, TRIDIAG_LAYOUT_CONTIGUOUS, dl, d, du, x, x, buf,
                             gtsv2_strided_ws<T>(m, batch, stride), m, batch, s);
  bool used = false;
  cudaError_t e = tdg::launch_pge_strided<T>(dl, d, du, x, x, nullptr, m, batch, (size_t)stride, s, &used);
  if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
  return used ? TRIDIAG_SUCCESS : TRIDIAG_ERR_NOT_SUPPORTED;
}

template <typename T>
size_t gtsv_interleaved_ws(int algo, int m, int batch) {
  if (m <= 0 || batch <= 0) return 0;
  return algo == 2 ? 0 : gtsv_ws_bytes<T>(m, batch);
}

template <typename T>
int gtsv_interleaved_impl(int algo, int m, T* dl, T* d, T* du, T* x, int batch, void* buf, cudaStream_t s) {
  if (m <= 0 || batch <= 0 || !dl || !d || !du || !x || algo < 0 || algo > 2) return TRIDIAG_ERR_INVALID_VALUE;
  if (algo == 2) return solve_impl<T>(TRIDIAG_ALGO_THOMAS, TRIDIAG_LAYOUT_INTERLEAVED, dl, d, du, x, m, batch, s);
  return gtsv_impl<T>(TRIDIAG_LAYOUT_INTERLEAVED, dl, d, du, x, nullptr, nullptr, buf,
                      gtsv_interleaved_ws<T>(algo, m, batch), m, batch, s);
}

}  // namespace

extern "C" {

size_t tridiag_gtsv2StridedBatch_bufferSize(int precision, int m, int batchCount, int batchStride) {
  return precision ? gtsv2_strided_ws<double>(m, batchCount, batchStride)
                   : gtsv2_strided_ws<float>(m, batchCount, batchStride);
}
int tridiag_Sgtsv2StridedBatch(int m, const float* dl, const float* d, const float* du, float* x, int batchCount,
                               int batchStride, void* pBuffer, void* stream) {
  return set_status(gtsv2_strided_impl<float>(m, dl, d, du, x, batchCount, batchStride, pBuffer, (cudaStream_t)stream));
}
int tridiag_Dgtsv2StridedBatch(int m, const double* dl, const double* d, const double* du, double* x, int batchCount,
                               int batchStride, void* pBuffer, void* stream) {
  return set_status(
      gtsv2_strided_impl<double>(m, dl, d, du, x, batchCount, batchStride, pBuffer, (cudaStream_t)stream));
}
size_t tridiag_gtsvInterleavedBatch_bufferSize(int precision, int algo, int m, int batchCount) {
  return precision ? gtsv_interleaved_ws<double>(algo, m, batchCount) : gtsv_interleaved_ws<float>(algo, m, batchCount);
}
int tridiag_SgtsvInterleavedBatch(int algo, int m, float* dl, float* d, float* du, float* x, int batchCount,
                                  void* pBuffer, void* stream) {
  return set_status(gtsv_interleaved_impl<float>(algo, m, dl, d, du, x, batchCount, pBuffer, (cudaStream_t)stream));
}
int tridiag_DgtsvInterleavedBatch(int algo, int m, double* dl, double* d, double* du, double* x, int batchCount,
                                  void* pBuffer, void* stream) {
  return set_status(gtsv_interleaved_impl<double>(algo, m, dl, d, du, x, batchCount, pBuffer, (cudaStream_t)stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Periodic systems (Sherman-Morrison over two tridiagonal solves; see
// periodic.cu).
namespace {

template <typename T>
size_t periodic_solver_ws(int algo, int n, int batch) {
  const size_t w = solve_out_ws<T>(algo == TRIDIAG_ALGO_GTSV ? TRIDIAG_ALGO_GTSV : TRIDIAG_ALGO_THOMAS, n, batch);
  return w;
}

template <typename T>
size_t periodic_ws(int algo, int n, int batch) {
  if (n < 3 || batch <= 0) return 0;
  return 3 * align_up((size_t)n * (size_t)batch * sizeof(T)) + periodic_solver_ws<T>(algo, n, batch);
}

template <typename T>
int periodic_impl(int algo, const T* a, const T* b, const T* c, const T* d, T* x, void* work, size_t work_bytes, int n,
                  int batch, cudaStream_t s) {
  if (n < 3 || batch <= 0 || !a || !b || !c || !d || !x) return TRIDIAG_ERR_INVALID_VALUE;
  if (algo == TRIDIAG_ALGO_AUTO) algo = TRIDIAG_ALGO_GTSV;
  if (algo != TRIDIAG_ALGO_GTSV && algo != TRIDIAG_ALGO_WM && algo != TRIDIAG_ALGO_THOMAS) return TRIDIAG_ERR_NOT_SUPPORTED;
  if (!work || work_bytes < periodic_ws<T>(algo, n, batch)) return TRIDIAG_ERR_WORKSPACE;
  const size_t one = align_up((size_t)n * (size_t)batch * sizeof(T));
  char* p = static_cast<char*>(work);
  T* bp = reinterpret_cast<T*>(p);
  T* u = reinterpret_cast<T*>(p + one);
  T* y = reinterpret_cast<T*>(p + 2 * one);
  void* sw = p + 3 * one;
  const size_t sw_bytes = periodic_solver_ws<T>(algo, n, batch);
  if (tdg::launch_periodic_prep<T>(a, b, c, bp, u, n, batch, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
  int st = solve_out_impl<T>(algo, TRIDIAG_LAYOUT_CONTIGUOUS, a, bp, c, d, y, sw, sw_bytes, n, batch, s);
  if (st != TRIDIAG_SUCCESS) return st;
  st = solve_out_impl<T>(algo, TRIDIAG_LAYOUT_CONTIGUOUS, a, bp, c, u, u, sw, sw_bytes, n, batch, s);
  if (st != TRIDIAG_SUCCESS) return st;
  return cuda_status(tdg::launch_periodic_combine<T>(a, b, y, u, x, n, batch, s));
}

}  // namespace

extern "C" {

size_t tridiag_periodic_workspace_size(int precision, int algo, int n, int batch) {
  if (algo == TRIDIAG_ALGO_AUTO) algo = TRIDIAG_ALGO_GTSV;
  return precision ? periodic_ws<double>(algo, n, batch) : periodic_ws<float>(algo, n, batch);
}
int tridiag_periodic_single(int algo, const float* a, const float* b, const float* c, const float* d, float* x,
                            void* work, size_t work_bytes, int n, int batch, void* stream) {
  return set_status(periodic_impl<float>(algo, a, b, c, d, x, work, work_bytes, n, batch, (cudaStream_t)stream));
}
int tridiag_periodic_double(int algo, const double* a, const double* b, const double* c, const double* d, double* x,
                            void* work, size_t work_bytes, int n, int batch, void* stream) {
  return set_status(periodic_impl<double>(algo, a, b, c, d, x, work, work_bytes, n, batch, (cudaStream_t)stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Solves with the arrays in host memory: the batch streams through device
// buffers in chunks, each chunk's host -> device copies, solve and
// device -> host copy of x on three streams of the library's own, so that the
// link carries one chunk while another is solved.  Streams, a ring of chunk
// buffers and its events persist per device and are shared by all such calls
// (enqueued under a lock): a call made while an earlier one is still in
// flight -- from an independent caller stream -- queues its copies behind the
// earlier ones and keeps the link busy across calls.
namespace {

constexpr int HOST_SLOTS = 3;
// Systems per chunk: about 96 MB of coefficient and right-hand-side bytes
// (measured on GB300: each copy adds a fixed gap on the link, so 12 MB chunks
// cost 15% over 96 MB ones; larger chunks lengthen the pipeline's fill).
constexpr size_t HOST_CHUNK_BYTES = 96u << 20;

struct HostPipe {
  cudaStream_t in = nullptr, comp = nullptr, out = nullptr;
  unsigned char* buf = nullptr;
  size_t slot_bytes = 0;
  cudaEvent_t ev_in[HOST_SLOTS] = {}, ev_comp[HOST_SLOTS] = {}, ev_out[HOST_SLOTS] = {};
  bool used[HOST_SLOTS] = {};
  int next = 0;
};

std::mutex g_pipe_mu;
HostPipe g_pipes[64];

cudaError_t host_pipe_init(HostPipe& q) {
  if (q.in) return cudaSuccess;
  cudaError_t e = cudaStreamCreateWithFlags(&q.in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&q.comp, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&q.out, cudaStreamNonBlocking);
  for (int k = 0; k < HOST_SLOTS && e == cudaSuccess; ++k) {
    e = cudaEventCreateWithFlags(&q.ev_in[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&q.ev_comp[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&q.ev_out[k], cudaEventDisableTiming);
  }
  return e;
}

// Grow the ring to slots of at least `bytes` (waits for the pipe's work).
cudaError_t host_pipe_reserve(HostPipe& q, size_t bytes) {
  if (q.slot_bytes >= bytes) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(q.in);
  if (e == cudaSuccess) e = cudaStreamSynchronize(q.comp);
  if (e == cudaSuccess) e = cudaStreamSynchronize(q.out);
  if (e == cudaSuccess && q.buf) e = cudaFree(q.buf);
  q.buf = nullptr;
  q.slot_bytes = 0;
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&q.buf), HOST_SLOTS * bytes);
  if (e == cudaSuccess) q.slot_bytes = bytes;
  for (bool& u : q.used) u = false;
  return e;
}

template <typename T>
int solve_host_impl(int algo, int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                    int chunk, cudaStream_t s) {
  if (!valid_dims(n, batch) || !valid_layout(layout) || !a || !b || !c || !d || !x || chunk < 0)
    return TRIDIAG_ERR_INVALID_VALUE;
  if (layout == TRIDIAG_LAYOUT_PACKED) return TRIDIAG_ERR_NOT_SUPPORTED;
  const size_t row = (size_t)n * sizeof(T);  // one array of one system
  int K = chunk;
  if (K == 0) {
    // interleaved: one contiguous copy per array (chunks of systems are 2-D
    // copies of n short rows, which the copy engines move far below the
    // link's rate: 6 KB rows measured at about half of it on GB300)
    const size_t k = layout == TRIDIAG_LAYOUT_INTERLEAVED ? (size_t)batch : HOST_CHUNK_BYTES / (4 * row);
    K = (int)(k < 1 ? 1 : k > (size_t)batch ? (size_t)batch : k);
  }
  if (K > batch) K = batch;
  const int nchunks = (batch + K - 1) / K;
  const size_t arr = align_up((size_t)K * row);
  const int ws_algo = algo == TRIDIAG_ALGO_AUTO || algo == TRIDIAG_ALGO_WM || algo == TRIDIAG_ALGO_CR ||
                              algo == TRIDIAG_ALGO_PCR || algo == TRIDIAG_ALGO_PARTITION
                          ? TRIDIAG_ALGO_THOMAS  // possible fallback
                          : algo;
  const size_t ws = align_up(solve_out_ws<T>(ws_algo, n, K, layout));
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TRIDIAG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_pipe_mu);
  HostPipe& p = g_pipes[dev];
  cudaError_t e = host_pipe_init(p);
  if (e == cudaSuccess) e = host_pipe_reserve(p, 5 * arr + ws);
  if (e != cudaSuccess) return cuda_status(e);
  cudaEvent_t ev_start = nullptr, ev_end = nullptr;
  e = cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_end, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(ev_start, s);
  for (cudaStream_t q : {p.in, p.comp, p.out})
    if (e == cudaSuccess) e = cudaStreamWaitEvent(q, ev_start, 0);
  const bool inter = layout == TRIDIAG_LAYOUT_INTERLEAVED;
  // one array of the systems [j0, j0 + kc) between host and a device buffer
  auto copy = [&](T* dst, const T* src, int j0, int kc, bool to_dev, cudaStream_t q) {
    if (!inter) {
      const size_t bytes = (size_t)kc * row;
      return to_dev ? cudaMemcpyAsync(dst, src + (size_t)j0 * n, bytes, cudaMemcpyHostToDevice, q)
                    : cudaMemcpyAsync(dst + (size_t)j0 * n, src, bytes, cudaMemcpyDeviceToHost, q);
    }
    const size_t w = (size_t)kc * sizeof(T), hp = (size_t)batch * sizeof(T);
    if (kc == batch)  // the whole batch: one contiguous copy
      return to_dev ? cudaMemcpyAsync(dst, src, w * n, cudaMemcpyHostToDevice, q)
                    : cudaMemcpyAsync(dst, src, w * n, cudaMemcpyDeviceToHost, q);
    return to_dev ? cudaMemcpy2DAsync(dst, w, src + j0, hp, w, n, cudaMemcpyHostToDevice, q)
                  : cudaMemcpy2DAsync(dst + j0, hp, src, w, w, n, cudaMemcpyDeviceToHost, q);
  };
  int st = TRIDIAG_SUCCESS;
  for (int ch = 0; ch < nchunks && e == cudaSuccess && st == TRIDIAG_SUCCESS; ++ch) {
    const int k = p.next, j0 = ch * K, kc = batch - j0 < K ? batch - j0 : K;
    p.next = (p.next + 1) % HOST_SLOTS;
    unsigned char* sb = p.buf + k * p.slot_bytes;
    T* da = reinterpret_cast<T*>(sb);
    T* db = reinterpret_cast<T*>(sb + arr);
    T* dc = reinterpret_cast<T*>(sb + 2 * arr);
    T* dd = reinterpret_cast<T*>(sb + 3 * arr);
    T* dx = reinterpret_cast<T*>(sb + 4 * arr);
    void* dw = ws ? sb + 5 * arr : nullptr;
    // inputs, once the slot's previous solve has read its own
    if (p.used[k]) e = cudaStreamWaitEvent(p.in, p.ev_comp[k], 0);
    const T* src[4] = {a, b, c, d};
    T* dst[4] = {da, db, dc, dd};
    for (int q = 0; q < 4 && e == cudaSuccess; ++q) e = copy(dst[q], src[q], j0, kc, true, p.in);
    if (e == cudaSuccess) e = cudaEventRecord(p.ev_in[k], p.in);
    // solve, once the inputs are in and the slot's previous x is out
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p.comp, p.ev_in[k], 0);
    if (e == cudaSuccess && p.used[k]) e = cudaStreamWaitEvent(p.comp, p.ev_out[k], 0);
    if (e == cudaSuccess) st = solve_out_impl<T>(algo, layout, da, db, dc, dd, dx, dw, ws, n, kc, p.comp);
    if (e == cudaSuccess && st == TRIDIAG_SUCCESS) e = cudaEventRecord(p.ev_comp[k], p.comp);
    // x back to the host
    if (e == cudaSuccess && st == TRIDIAG_SUCCESS) e = cudaStreamWaitEvent(p.out, p.ev_comp[k], 0);
    if (e == cudaSuccess && st == TRIDIAG_SUCCESS) e = copy(x, dx, j0, kc, false, p.out);
    if (e == cudaSuccess && st == TRIDIAG_SUCCESS) e = cudaEventRecord(p.ev_out[k], p.out);
    p.used[k] = true;
  }
  // the copy-out stream has waited for every solve of this call: the
  // caller's stream continues after its last copy
  if (ev_end) {
    const cudaError_t r = cudaEventRecord(ev_end, p.out);
    const cudaError_t w = r == cudaSuccess ? cudaStreamWaitEvent(s, ev_end, 0) : r;
    if (e == cudaSuccess) e = w;
  }
  if (ev_start) cudaEventDestroy(ev_start);
  if (ev_end) cudaEventDestroy(ev_end);
  if (st != TRIDIAG_SUCCESS) return st;
  return cuda_status(e);
}

}  // namespace

extern "C" {

int tridiag_solve_host_single(int algo, int layout, const float* a, const float* b, const float* c, const float* d,
                              float* x, int n, int batch, int chunk, void* stream) {
  return set_status(solve_host_impl<float>(algo, layout, a, b, c, d, x, n, batch, chunk, (cudaStream_t)stream));
}
int tridiag_solve_host_double(int algo, int layout, const double* a, const double* b, const double* c,
                              const double* d, double* x, int n, int batch, int chunk, void* stream) {
  return set_status(solve_host_impl<double>(algo, layout, a, b, c, d, x, n, batch, chunk, (cudaStream_t)stream));
}

}  // extern "C"
