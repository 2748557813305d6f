// Ragged batches: systems of different sizes packed back to back (system s
// = rows [offsets[s], offsets[s+1]) of a, b, c, d), solved -- and
// differentiated -- with partial pivoting in size buckets.
//
// The plan groups the systems by size class (class k: 2^(k-1) < n <= 2^k)
// and gives each class a kernel variant: the thread-per-system sequential
// solve for n < 65 (variant 0), the partitioned solve with 64/128/256
// partitions in one CTA (1-3) or in a cluster of 2/4/8 CTAs (4-6).  A
// variant table (from the autotuner, or the defaults) overrides the choice
// per class.  Systems the caller marks as needing no pivoting (diagonally
// dominant ones, say) form buckets of their own that run the unpivoted
// partition method: one CTA per system up to 128 128-byte rows (variant 7),
// chunks of that size per CTA with the separators' system in between for
// longer ones (variant 8), forward and adjoint.  Within a bucket the systems run longest first.  Solving is one
// launch per non-empty bucket on the caller's stream, so the whole ragged
// solve can be captured in one CUDA graph and replayed.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

constexpr int RAGGED_TINY_MAX = 64;

// Thread-per-system sequential partial-pivoting solve (LAPACK ?gtsv
// elimination) for the short systems of a bucket; U rows in thread-local
// arrays.  MODE 1: the transposed system (the caller passes c - 1 and a + 1)
// with the gradient epilogue.
template <typename T, int MODE>
__global__ void __launch_bounds__(128) ragged_tiny_kernel(const T* a, const T* b, const T* c, const T* d, T* x,
                                                          const T* xf, T* ga, T* gb, T* gc, int* info,
                                                          const long long* offsets, const int* list, int count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int sys = list[k];
  const size_t base = (size_t)offsets[sys];
  const int n = (int)(offsets[sys + 1] - offsets[sys]);
  T inv[RAGGED_TINY_MAX], u1[RAGGED_TINY_MAX], u2[RAGGED_TINY_MAX], y[RAGGED_TINY_MAX];
  int zero = 0;
  T cb = b[base], cc = n > 1 ? c[base] : T(0), cy = d[base];
  for (int i = 0; i + 1 < n; ++i) {
    const T na = a[base + i + 1], nb = b[base + i + 1];
    const T nc = i + 2 < n ? c[base + i + 1] : T(0);
    const T ny = d[base + i + 1];
    const bool sw = !abs_ge(cb, na);
    const T piv = sw ? na : cb;
    if (is_zero(piv) && !zero) zero = i + 1;
    inv[i] = Div<T>(piv).inv();
    const T l = (sw ? cb : na) * inv[i];
    u1[i] = sw ? nb : cc;
    u2[i] = sw ? nc : T(0);
    y[i] = sw ? ny : cy;
    cb = fma(-l, u1[i], sw ? cc : nb);
    cc = fma(-l, sw ? nc : T(0), sw ? T(0) : nc);
    cy = fma(-l, y[i], sw ? cy : ny);
  }
  if (is_zero(cb) && !zero) zero = n;
  if (info) info[sys] = zero;
  if (zero) return;
  T x1 = cy * Div<T>(cb).inv(), x2 = T(0);
  T vals[RAGGED_TINY_MAX];
  vals[n - 1] = x1;
  for (int i = n - 2; i >= 0; --i) {
    const T xi = fma(-u2[i], x2, fma(-u1[i], x1, y[i])) * inv[i];
    vals[i] = xi;
    x2 = x1;
    x1 = xi;
  }
  for (int r = 0; r < n; ++r) {
    const T v = vals[r];
    x[base + r] = v;
    if (MODE == 1) {
      ga[base + r] = r > 0 ? -v * xf[base + r - 1] : T(0);
      gb[base + r] = -v * xf[base + r];
      gc[base + r] = r < n - 1 ? -v * xf[base + r + 1] : T(0);
    }
  }
}

template <typename T>
static cudaError_t launch_tiny(int mode, const T* a, const T* b, const T* c, const T* d, T* x, const T* xf, T* ga,
                               T* gb, T* gc, int* info, const long long* offsets, const int* list, int count,
                               cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int grid = (count + 127) / 128;
  if (mode == 0)
    ragged_tiny_kernel<T, 0><<<grid, 128, 0, s>>>(a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, count);
  else
    ragged_tiny_kernel<T, 1><<<grid, 128, 0, s>>>(c - 1, b, a + 1, d, x, xf, ga, gb, gc, info, offsets, list, count);
  return cudaGetLastError();
}

}  // namespace tdg

// The opaque plan of include/tridiagonal.h.
struct tridiag_ragged_plan {
  struct Bucket {
    int cls;      // size class
    int variant;  // 0 tiny, 1-6 partitioned, 7 unpivoted partition method
    int count;    // systems
    int m_max;    // rows per partition of the longest system
    int max_n;
    long long rows;
    size_t list_off;  // into d_lists
  };
  int precision = 0;
  int batch = 0;
  long long total_rows = 0;
  std::vector<Bucket> buckets;
  int* d_lists = nullptr;
  int device = 0;
  // long systems marked as needing no pivoting (variant 8): chunk lists and
  // the partition workspace, one device allocation
  tdg::WmlRagged lr;
  void* d_lr = nullptr;
  void* lr_work = nullptr;
};

namespace {

int size_class(long long n) {
  int k = 0;
  while ((1ll << k) < n) ++k;
  return k;
}

constexpr int RAGGED_UNPIVOTED = 7;
constexpr int RAGGED_UNPIVOTED_LONG = 8;

template <typename T>
int unpivoted_max_n() {
  return tdg::WML_CHUNK_R * (128 / (int)sizeof(T));  // one chunk-sized CTA (three per SM)
}

// long unpivoted systems: beyond one CTA, their separators' system within one
template <typename T>
bool long_unpivoted_ok(long long n) {
  constexpr int M = 128 / (int)sizeof(T);
  return n > unpivoted_max_n<T>() && (n + M - 1) / M <= (long long)tdg::WMC_GEN_MAX_ROWS * M;
}

template <typename T>
bool variant_serves(int v, int max_n) {
  if (v == 0) return max_n <= tdg::RAGGED_TINY_MAX;
  if (v == RAGGED_UNPIVOTED) return max_n <= unpivoted_max_n<T>();
  return max_n >= 65 && max_n <= tdg::pge_variant_max_n<T>(v);
}

// no_pivoting (may be NULL): systems marked 1 need no pivoting and run the
// unpivoted partition method (variant 7) where their class allows it.
template <typename T>
int plan_create(tridiag_ragged_plan** out, const long long* offsets, int batch, const int* table, int table_len,
                const unsigned char* no_pivoting = nullptr) {
  if (!out || !offsets || batch <= 0) return TRIDIAG_ERR_INVALID_VALUE;
  *out = nullptr;
  // classes 0 .. CLASSES-1 pivoted, CLASSES .. 2 CLASSES-1 unpivoted; long
  // unpivoted systems apart
  std::vector<std::vector<int>> by_class(2 * TRIDIAG_RAGGED_CLASSES);
  std::vector<int> longs;
  for (int s = 0; s < batch; ++s) {
    const long long n = offsets[s + 1] - offsets[s];
    if (n < 1 || n > (1ll << (TRIDIAG_RAGGED_CLASSES - 1))) return TRIDIAG_ERR_INVALID_VALUE;
    const bool unp = no_pivoting && no_pivoting[s] && n <= unpivoted_max_n<T>();
    if (no_pivoting && no_pivoting[s] && !unp && long_unpivoted_ok<T>(n)) {
      longs.push_back(s);
      continue;
    }
    by_class[size_class(n) + (unp ? TRIDIAG_RAGGED_CLASSES : 0)].push_back(s);
  }
  auto* plan = new (std::nothrow) tridiag_ragged_plan;
  if (!plan) return TRIDIAG_ERR_WORKSPACE;
  plan->precision = sizeof(T) == 8 ? 1 : 0;
  plan->batch = batch;
  plan->total_rows = offsets[batch] - offsets[0];
  cudaGetDevice(&plan->device);
  std::vector<int> lists;
  for (int kk = 0; kk < 2 * TRIDIAG_RAGGED_CLASSES; ++kk) {
    auto& sys = by_class[kk];
    if (sys.empty()) continue;
    const bool unp = kk >= TRIDIAG_RAGGED_CLASSES;
    const int k = kk % TRIDIAG_RAGGED_CLASSES;
    std::sort(sys.begin(), sys.end(), [&](int p, int q) {
      const long long np = offsets[p + 1] - offsets[p], nq = offsets[q + 1] - offsets[q];
      return np != nq ? np > nq : p < q;
    });
    const int max_n = (int)(offsets[sys[0] + 1] - offsets[sys[0]]);
    int v = unp ? RAGGED_UNPIVOTED : -1;
    if (!unp && table && k < table_len && table[k] >= 0) {
      if (!variant_serves<T>(table[k], max_n)) {  // an explicit choice that cannot serve the class
        delete plan;
        return TRIDIAG_ERR_NOT_SUPPORTED;
      }
      v = table[k];
    }
    if (v < 0) v = max_n <= tdg::RAGGED_TINY_MAX ? 0 : tdg::pge_default_variant<T>(max_n);
    if (v < 0 || (v == 0 && max_n > tdg::RAGGED_TINY_MAX) || (v > 0 && !variant_serves<T>(v, max_n))) {
      delete plan;
      return TRIDIAG_ERR_NOT_SUPPORTED;
    }
    tridiag_ragged_plan::Bucket bk;
    bk.cls = k;
    bk.variant = v;
    bk.count = (int)sys.size();
    bk.max_n = max_n;
    constexpr int M = 128 / (int)sizeof(T);
    bk.m_max = v == 0                  ? 0
               : v == RAGGED_UNPIVOTED ? (max_n + M - 1) / M  // 128-byte rows of the longest system
                                       : std::max(2, (max_n + tdg::pge_variant_partitions(v) - 1) /
                                                         tdg::pge_variant_partitions(v));
    bk.rows = 0;
    for (int q : sys) bk.rows += offsets[q + 1] - offsets[q];
    bk.list_off = lists.size();
    lists.insert(lists.end(), sys.begin(), sys.end());
    plan->buckets.push_back(bk);
  }
  // longest buckets first: their few, long launches start before the short ones fill the GPU
  std::stable_sort(plan->buckets.begin(), plan->buckets.end(),
                   [](const tridiag_ragged_plan::Bucket& p, const tridiag_ragged_plan::Bucket& q) {
                     return p.cls > q.cls;
                   });
  if (!longs.empty()) {
    constexpr int M = 128 / (int)sizeof(T);
    const long long chunk_rows = (long long)tdg::WML_CHUNK_R * M;
    std::sort(longs.begin(), longs.end(), [&](int p, int q) {
      const long long np = offsets[p + 1] - offsets[p], nq = offsets[q + 1] - offsets[q];
      return np != nq ? np > nq : p < q;
    });
    std::vector<long long> roff(longs.size() + 1, 0);
    std::vector<int> cl_li, cl_ch;
    int pmax = 0;
    long long rows = 0;
    for (size_t i = 0; i < longs.size(); ++i) {
      const long long n = offsets[longs[i] + 1] - offsets[longs[i]];
      const long long P = (n + M - 1) / M;
      roff[i + 1] = roff[i] + P;
      pmax = std::max(pmax, (int)P);
      rows += n;
      for (long long c = 0; c * chunk_rows < n; ++c) {
        cl_li.push_back((int)i);
        cl_ch.push_back((int)c);
      }
    }
    plan->lr.L = (int)longs.size();
    plan->lr.C = (int)cl_li.size();
    plan->lr.P = roff.back();
    plan->lr.Pmax = pmax;
    const size_t b_lsys = longs.size() * sizeof(int), b_roff = roff.size() * sizeof(long long),
                 b_cl = cl_li.size() * sizeof(int);
    const size_t o_roff = (b_lsys + 255) / 256 * 256, o_li = o_roff + (b_roff + 255) / 256 * 256,
                 o_ch = o_li + (b_cl + 255) / 256 * 256, o_end = o_ch + (b_cl + 255) / 256 * 256;
    char* mem = nullptr;
    if (cudaMalloc(&mem, o_end) != cudaSuccess ||
        cudaMalloc(&plan->lr_work, tdg::wml_ragged_workspace_elems<T>(plan->lr.P) * sizeof(T)) != cudaSuccess) {
      cudaFree(mem);
      delete plan;
      return TRIDIAG_ERR_CUDA;
    }
    plan->d_lr = mem;
    cudaMemcpy(mem, longs.data(), b_lsys, cudaMemcpyHostToDevice);
    cudaMemcpy(mem + o_roff, roff.data(), b_roff, cudaMemcpyHostToDevice);
    cudaMemcpy(mem + o_li, cl_li.data(), b_cl, cudaMemcpyHostToDevice);
    cudaMemcpy(mem + o_ch, cl_ch.data(), b_cl, cudaMemcpyHostToDevice);
    plan->lr.l_sys = reinterpret_cast<int*>(mem);
    plan->lr.roff = reinterpret_cast<long long*>(mem + o_roff);
    plan->lr.cl_li = reinterpret_cast<int*>(mem + o_li);
    plan->lr.cl_ch = reinterpret_cast<int*>(mem + o_ch);
    tridiag_ragged_plan::Bucket bk;
    const int max_n = (int)(offsets[longs[0] + 1] - offsets[longs[0]]);
    bk.cls = size_class(max_n);
    bk.variant = RAGGED_UNPIVOTED_LONG;
    bk.count = (int)longs.size();
    bk.max_n = max_n;
    bk.m_max = 0;
    bk.rows = rows;
    bk.list_off = 0;
    plan->buckets.insert(plan->buckets.begin(), bk);  // longest work first
  }
  if (cudaMalloc(&plan->d_lists, std::max<size_t>(lists.size(), 1) * sizeof(int)) != cudaSuccess) {
    cudaFree(plan->d_lr);
    cudaFree(plan->lr_work);
    delete plan;
    return TRIDIAG_ERR_CUDA;
  }
  if (cudaMemcpy(plan->d_lists, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(plan->d_lists);
    delete plan;
    return TRIDIAG_ERR_CUDA;
  }
  *out = plan;
  return TRIDIAG_SUCCESS;
}

template <typename T>
int plan_run(const tridiag_ragged_plan* plan, int mode, const T* a, const T* b, const T* c, const T* d, T* x,
             const T* xf, T* ga, T* gb, T* gc, int* info, const long long* offsets, cudaStream_t s) {
  if (!plan || !a || !b || !c || !d || !x || !offsets) return TRIDIAG_ERR_INVALID_VALUE;
  if (plan->precision != (sizeof(T) == 8 ? 1 : 0)) return TRIDIAG_ERR_INVALID_VALUE;
  if (mode == 1 && (!xf || !ga || !gb || !gc)) return TRIDIAG_ERR_INVALID_VALUE;
  for (const auto& bk : plan->buckets) {
    const int* list = plan->d_lists + bk.list_off;
    cudaError_t e;
    if (bk.variant == RAGGED_UNPIVOTED_LONG)
      e = mode == 0 ? tdg::launch_wml_ragged<T>(0, a, b, c, d, nullptr, x, nullptr, nullptr, nullptr, offsets,
                                                plan->lr, static_cast<T*>(plan->lr_work), info, s)
                    : tdg::launch_wml_ragged<T>(1, a, b, c, d, xf, x, ga, gb, gc, offsets, plan->lr,
                                                static_cast<T*>(plan->lr_work), info, s);
    else if (bk.variant == 0)
      e = tdg::launch_tiny<T>(mode, a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, bk.count, s);
    else if (bk.variant == RAGGED_UNPIVOTED)
      e = mode == 0 ? tdg::launch_wmc_ragged<T>(0, a, b, c, d, nullptr, x, nullptr, nullptr, nullptr, offsets, list,
                                                bk.count, bk.m_max, info, s)
                    : tdg::launch_wmc_ragged<T>(1, a, b, c, d, xf, ga, gb, gc, x, offsets, list, bk.count, bk.m_max,
                                                info, s);
    else
      e = tdg::launch_pge_ragged<T>(bk.variant, mode, a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, bk.count,
                                    bk.m_max, s);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
  }
  return TRIDIAG_SUCCESS;
}

}  // namespace

extern "C" {

int tridiag_ragged_plan_create(tridiag_ragged_plan** plan, int precision, const long long* offsets_host, int batch,
                               const int* variant_by_class, int n_classes) {
  return precision ? plan_create<double>(plan, offsets_host, batch, variant_by_class, n_classes)
                   : plan_create<float>(plan, offsets_host, batch, variant_by_class, n_classes);
}

int tridiag_ragged_plan_create_ex(tridiag_ragged_plan** plan, int precision, const long long* offsets_host,
                                  int batch, const int* variant_by_class, int n_classes,
                                  const unsigned char* no_pivoting_host) {
  return precision ? plan_create<double>(plan, offsets_host, batch, variant_by_class, n_classes, no_pivoting_host)
                   : plan_create<float>(plan, offsets_host, batch, variant_by_class, n_classes, no_pivoting_host);
}

void tridiag_ragged_plan_destroy(tridiag_ragged_plan* plan) {
  if (!plan) return;
  cudaFree(plan->d_lists);
  cudaFree(plan->d_lr);
  cudaFree(plan->lr_work);
  delete plan;
}

int tridiag_ragged_plan_buckets(const tridiag_ragged_plan* plan, int* out, int max_buckets) {
  if (!plan) return -1;
  const int nb = (int)plan->buckets.size();
  if (out)
    for (int i = 0; i < nb && i < max_buckets; ++i) {
      const auto& bk = plan->buckets[i];
      out[4 * i] = bk.cls;
      out[4 * i + 1] = bk.variant;
      out[4 * i + 2] = bk.count;
      out[4 * i + 3] = bk.max_n;
    }
  return nb;
}

int tridiag_ragged_variant_max_n(int precision, int variant) {
  if (variant == 0) return tdg::RAGGED_TINY_MAX;
  if (variant == RAGGED_UNPIVOTED) return precision ? unpivoted_max_n<double>() : unpivoted_max_n<float>();
  if (variant == RAGGED_UNPIVOTED_LONG)
    return precision ? tdg::WMC_GEN_MAX_ROWS * 16 * 16 : tdg::WMC_GEN_MAX_ROWS * 32 * 32;
  return precision ? tdg::pge_variant_max_n<double>(variant) : tdg::pge_variant_max_n<float>(variant);
}

int tridiag_ragged_solve_single(const tridiag_ragged_plan* plan, const float* a, const float* b, const float* c,
                                const float* d, float* x, int* info, const long long* offsets, void* stream) {
  return plan_run<float>(plan, 0, a, b, c, d, x, nullptr, nullptr, nullptr, nullptr, info, offsets,
                         (cudaStream_t)stream);
}
int tridiag_ragged_solve_double(const tridiag_ragged_plan* plan, const double* a, const double* b, const double* c,
                                const double* d, double* x, int* info, const long long* offsets, void* stream) {
  return plan_run<double>(plan, 0, a, b, c, d, x, nullptr, nullptr, nullptr, nullptr, info, offsets,
                          (cudaStream_t)stream);
}
int tridiag_ragged_adjoint_single(const tridiag_ragged_plan* plan, const float* a, const float* b, const float* c,
                                  const float* x, const float* xbar, float* ga, float* gb, float* gc, float* gd,
                                  int* info, const long long* offsets, void* stream) {
  return plan_run<float>(plan, 1, a, b, c, xbar, gd, x, ga, gb, gc, info, offsets, (cudaStream_t)stream);
}
int tridiag_ragged_adjoint_double(const tridiag_ragged_plan* plan, const double* a, const double* b,
                                  const double* c, const double* x, const double* xbar, double* ga, double* gb,
                                  double* gc, double* gd, int* info, const long long* offsets, void* stream) {
  return plan_run<double>(plan, 1, a, b, c, xbar, gd, x, ga, gb, gc, info, offsets, (cudaStream_t)stream);
}

}  // extern "C"
