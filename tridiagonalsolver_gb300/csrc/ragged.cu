// Ragged batches: systems of different sizes packed back to back (system s
// = rows [offsets[s], offsets[s+1]) of a, b, c, d), solved -- and
// differentiated -- with partial pivoting in size buckets.
//
// The plan groups the systems by size class (class k: 2^(k-1) < n <= 2^k)
// and gives each class a kernel variant: the thread-per-system sequential
// solve for n < 65 (variant 0), the partitioned solve with 64/128/256
// partitions in one CTA (1-3) or in a cluster of 2/4/8 CTAs (4-6), and the
// thread-per-system sequential solve with its rows in a workspace for sizes
// beyond every partitioned variant (9), or -- the default there -- the
// partitioned solve in chunks of 4224 rows with the separators' systems in
// between (10: FP64 beyond 27648 rows), which re-solves a system by 9 when
// a chunk misses its accuracy bound.  A
// variant table (from the autotuner, or the defaults) overrides the choice
// per class.  Systems that need no pivoting -- marked by the caller, or
// found by the library itself -- run the unpivoted partition method in
// buckets of their own: one CTA per system up to 128 128-byte rows (variant
// 7), chunks per CTA with the separators' system in between for longer ones
// (variant 8), forward and adjoint.  When the library finds them, each
// solve starts every system of a size the unpivoted method serves as a
// candidate; the unpivoted kernels check the rows they stage (strict
// diagonal dominance) and hand a system that fails to the pivoted bucket of
// its class -- appended to that bucket's list on the device -- before any
// arithmetic, so the classification costs no pass of its own.  A bucket
// whose list a device pass writes, and every bucket of one kind, is served
// by resident CTAs (clusters) that take entries through an atomic ticket.
// Within a class the unpivoted bucket runs before the pivoted one.  Solving
// is a few device-side resets and one launch per non-empty bucket on the
// caller's stream, so the whole ragged solve can be captured in one CUDA
// graph and replayed.
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

// Variant 9: the same elimination for any n, one thread per system, the
// finished rows kept in global memory -- for the classes no partitioned
// variant serves (FP64 beyond the clusters' shared memory).  Forward solve
// (MODE 0): the finished rows' right-hand sides go to x, U1 and 1/U0 to the
// plan's workspace (w1, w2 at the system's workspace row soff[s]), the
// interchange bits to piv (word soff[s] / 32 + i / 32); the back
// substitution reads them back and overwrites x.  MODE 1 (the transposed
// system: the caller passes c - 1 and a + 1 for a and c): U1 and 1/U0 go to
// gb and gc, which the back substitution then overwrites with the
// gradients.  Rows are loaded SEQ_U ahead of the recurrence in both sweeps.
// A kind-0 list grown on the device has its length at *dcount.
constexpr int SEQ_U = 8;

template <typename T, int MODE>
__global__ void __launch_bounds__(32) ragged_seq_kernel(const T* a, const T* b, const T* c, const T* d, T* x,
                                                        const T* xf, T* ga, T* gb, T* gc, int* info,
                                                        const long long* offsets, const int* list, int count,
                                                        const int* dcount, const long long* soff, T* w1, T* w2,
                                                        unsigned* piv, const int* flag) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int live = dcount ? min(*dcount, count) : count;
  if (k >= live) return;
  const int sys = list[k];
  if (flag && !flag[sys]) {  // (variant 10's re-solve: only the systems a chunk failed)
    if (info) info[sys] = 0;
    return;
  }
  const long long base = offsets[sys];
  const int n = (int)(offsets[sys + 1] - base);
  const long long so = soff[sys];
  T* Rs = x + base;
  T* Us = MODE == 0 ? w1 + so : gb + base;
  T* Ws = MODE == 0 ? w2 + so : gc + base;
  unsigned* pv = piv + so / 32;
  T u0 = b[base], u1 = n > 1 ? c[base] : T(0), rhs = d[base];
  int bad = 0;
  unsigned word = 0;
  T na[SEQ_U], nb[SEQ_U], nc[SEQ_U], nd[SEQ_U];
#pragma unroll
  for (int u = 0; u < SEQ_U; ++u) {
    const int i = 1 + u;
    if (i < n) {
      na[u] = a[base + i];
      nb[u] = b[base + i];
      nc[u] = i + 1 < n ? c[base + i] : T(0);
      nd[u] = d[base + i];
    }
  }
  for (int i0 = 0; i0 + 1 < n; i0 += SEQ_U) {
    T ra[SEQ_U], rb[SEQ_U], rc[SEQ_U], rd[SEQ_U];
#pragma unroll
    for (int u = 0; u < SEQ_U; ++u) { ra[u] = na[u]; rb[u] = nb[u]; rc[u] = nc[u]; rd[u] = nd[u]; }
#pragma unroll
    for (int u = 0; u < SEQ_U; ++u) {
      const int i = i0 + 1 + SEQ_U + u;
      if (i < n) {
        na[u] = a[base + i];
        nb[u] = b[base + i];
        nc[u] = i + 1 < n ? c[base + i] : T(0);
        nd[u] = d[base + i];
      }
    }
#pragma unroll
    for (int u = 0; u < SEQ_U; ++u) {
      const int i = i0 + u;  // finishing row i; row i + 1 is (ra, rb, rc, rd)[u]
      if (i + 1 < n) {
        const bool sw = !abs_ge(u0, ra[u]);
        const T p = sw ? ra[u] : u0;
        const T q = sw ? u0 : ra[u];
        if (is_zero(p) && bad == 0) bad = i + 1;
        const T r = Div<T>(p).inv();
        const T m = q * r;
        Rs[i] = sw ? rd[u] : rhs;
        Us[i] = sw ? rb[u] : u1;
        Ws[i] = r;
        const T nu0 = fma(-m, sw ? rb[u] : u1, sw ? u1 : rb[u]);
        const T nu1 = sw ? -m * rc[u] : rc[u];
        const T nrhs = fma(-m, sw ? rd[u] : rhs, sw ? rhs : rd[u]);
        word |= (unsigned)sw << (i & 31);
        if ((i & 31) == 31) {
          pv[i >> 5] = word;
          word = 0;
        }
        u0 = nu0;
        u1 = nu1;
        rhs = nrhs;
      }
    }
  }
  if (n >= 2 && ((n - 2) & 31) != 31) pv[(n - 2) >> 5] = word;
  if (is_zero(u0) && bad == 0) bad = n;
  if (info) info[sys] = bad;
  if (bad) return;
  // back substitution: x_i = (R_i - U1_i x_{i+1} - U2_i x_{i+2}) / U0_i, with
  // U2_i = c_{i+1} where rows i and i+1 were interchanged
  T x1 = rhs * Div<T>(u0).inv();  // x_{n-1}
  T x2 = T(0);
  T fn = T(0), fc = T(0);         // MODE 1: xf of rows i + 1 and i
  if (MODE == 1) {
    fc = xf[base + n - 1];
    const T fp = n > 1 ? xf[base + n - 2] : T(0);
    ga[base + n - 1] = n > 1 ? -x1 * fp : T(0);
    gb[base + n - 1] = -x1 * fc;
    gc[base + n - 1] = T(0);
    fn = fc;
    fc = fp;
  }
  Rs[n - 1] = x1;
  // (every operand of a row, U2's candidate c_{i+1} and the interchange
  // word included, is loaded SEQ_U rows ahead: a load on the recurrence
  // would cost a memory latency per row)
  T qR[SEQ_U], qU[SEQ_U], qW[SEQ_U], qF[SEQ_U], qC[SEQ_U];
#pragma unroll
  for (int u = 0; u < SEQ_U; ++u) {
    const int i = n - 2 - u;
    if (i >= 0) {
      qR[u] = Rs[i];
      qU[u] = Us[i];
      qW[u] = Ws[i];
      qF[u] = MODE == 1 && i > 0 ? xf[base + i - 1] : T(0);
      qC[u] = i + 2 < n ? c[base + i + 1] : T(0);
    }
  }
  int wnext = (n - 2) >> 5;  // word of the next row to finish, and the one after it
  unsigned wcur = n >= 2 ? pv[wnext] : 0u, wpre = wnext > 0 ? pv[wnext - 1] : 0u;
  for (int i0 = n - 2; i0 >= 0; i0 -= SEQ_U) {
    T rR[SEQ_U], rU[SEQ_U], rW[SEQ_U], rF[SEQ_U], rC[SEQ_U];
#pragma unroll
    for (int u = 0; u < SEQ_U; ++u) { rR[u] = qR[u]; rU[u] = qU[u]; rW[u] = qW[u]; rF[u] = qF[u]; rC[u] = qC[u]; }
#pragma unroll
    for (int u = 0; u < SEQ_U; ++u) {
      const int i = i0 - SEQ_U - u;
      if (i >= 0) {
        qR[u] = Rs[i];
        qU[u] = Us[i];
        qW[u] = Ws[i];
        qF[u] = MODE == 1 && i > 0 ? xf[base + i - 1] : T(0);
        qC[u] = i + 2 < n ? c[base + i + 1] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < SEQ_U; ++u) {
      const int i = i0 - u;
      if (i >= 0) {
        if ((i >> 5) != wnext) {  // rows of the next word: it was loaded a word ahead
          wnext = i >> 5;
          wcur = wpre;
          wpre = wnext > 0 ? pv[wnext - 1] : 0u;
        }
        const bool sw = (wcur >> (i & 31)) & 1u;
        const T u2 = sw ? rC[u] : T(0);
        T x0 = fma(-rU[u], x1, rR[u]);
        x0 = fma(-u2, x2, x0) * rW[u];
        Rs[i] = x0;
        if (MODE == 1) {  // lambda_i = x0; rows i - 1, i, i + 1 of the forward solution
          ga[base + i] = -x0 * rF[u];
          gb[base + i] = -x0 * fc;
          gc[base + i] = -x0 * fn;
          fn = fc;
          fc = rF[u];
        }
        x2 = x1;
        x1 = x0;
      }
    }
  }
}

template <typename T>
static cudaError_t launch_ragged_seq(int mode, const T* a, const T* b, const T* c, const T* d, T* x, const T* xf,
                                     T* ga, T* gb, T* gc, int* info, const long long* offsets, const int* list,
                                     int count, const int* dcount, const long long* soff, T* w1, T* w2,
                                     unsigned* piv, const int* flag, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  // one warp per block: the few long systems spread over all SMs
  const int grid = (count + 31) / 32;
  if (mode == 0)
    ragged_seq_kernel<T, 0><<<grid, 32, 0, s>>>(a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, count, dcount,
                                                soff, w1, w2, piv, flag);
  else
    ragged_seq_kernel<T, 1><<<grid, 32, 0, s>>>(c - 1, b, a + 1, d, x, xf, ga, gb, gc, info, offsets, list, count,
                                                dcount, soff, w1, w2, piv, flag);
  return cudaGetLastError();
}

// Gradients of variant 10's adjoint from lambda and the forward solution
// xf, one warp per chunk entry (system cl_sys[k], rows [cl_ch[k] CR,
// (cl_ch[k] + 1) CR)), skipping the systems of the other kind and those a
// chunk failed (re-solved with their gradients by variant 9).
template <typename T>
__global__ void __launch_bounds__(256) ragged_chunk_gradient_kernel(const T* __restrict__ lam,
                                                                    const T* __restrict__ xf, T* __restrict__ ga,
                                                                    T* __restrict__ gb, T* __restrict__ gc,
                                                                    const long long* __restrict__ offsets,
                                                                    const int* __restrict__ cl_sys,
                                                                    const int* __restrict__ cl_ch, int C, int CR,
                                                                    const unsigned char* kinds, int want,
                                                                    const int* flag) {
  const int k = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) / 32);
  const int lane = threadIdx.x & 31;
  if (k >= C) return;
  const int sys = cl_sys[k];
  if ((kinds && kinds[sys] != want) || flag[sys]) return;
  const long long s0 = offsets[sys];
  const long long n = offsets[sys + 1] - s0;
  const long long lo = (long long)cl_ch[k] * CR, hi = min(n, lo + CR);
  for (long long i = lo + lane; i < hi; i += 32) {
    const T l = -lam[s0 + i];
    ga[s0 + i] = i > 0 ? l * xf[s0 + i - 1] : T(0);
    gb[s0 + i] = l * xf[s0 + i];
    gc[s0 + i] = i + 1 < n ? l * xf[s0 + i + 1] : T(0);
  }
}

}  // namespace tdg

// The opaque plan of include/tridiagonal.h.
struct tridiag_ragged_plan {
  struct Bucket {
    int cls;      // size class
    int variant;  // 0 tiny, 1-6 partitioned, 7 unpivoted partition method, 8 its chunked form, 9 sequential
    int count;    // systems (list entries; for kind 0 the room, the length being on the device)
    int m_max;    // rows per partition of the longest system
    int max_n;
    long long rows;
    size_t list_off;  // into d_lists
    int kind;         // -1: every system of the class; 0 / 1: the class's systems of that kind
    int ticket;       // -1: one CTA (cluster) per list entry; else index of its ticket counter
    int klist;        // -1: list in d_lists; else 2 k + kind: the kind list in d_klists
    size_t klist_off;
    // variant 10: the bucket's chunk entries (cl_off .. cl_off + cl_count in
    // d_cl), the separators' systems' variant and rows per partition
    size_t cl_off = 0;
    int cl_count = 0;
    int sep_variant = 0, sep_m_max = 0;
    // its re-solve of the systems a chunk failed (chunks of 31-row
    // partitions: entries cl2_off .. in d_cl2, separators at d_sep_off2)
    size_t cl2_off = 0;
    int cl2_count = 0;
    int sep2_variant = 0, sep2_m_max = 0;
    int ticket2 = -1;  // its separators' solve's ticket counter
  };
  int precision = 0;
  int batch = 0;
  long long total_rows = 0;
  long long row0 = 0;  // offsets[0]
  std::vector<Bucket> buckets;
  int* d_lists = nullptr;
  int device = 0;
  // long systems for the unpivoted chunked method (variant 8): chunk lists
  // and the partition workspace, one device allocation
  tdg::WmlRagged lr;
  void* d_lr = nullptr;
  void* lr_work = nullptr;
  // kinds of the systems (1: solved without pivoting): the caller's mask
  // (mode 1), or found by every solve (mode 2: the unpivoted kernels check
  // the rows they stage and hand the systems that need pivoting over)
  int kinds_mode = 0;  // 0 none, 1 caller's mask, 2 found by the solves
  unsigned char* d_kinds = nullptr;
  bool classified = false;
  int* d_tickets = nullptr;
  int n_tickets = 0;
  int unp_max = 0, long_max = 0;  // rows served by variants 7 and 8
  // variant 9: each system's workspace row (d_soff[s], -1 for the systems of
  // other classes) and the workspace: U1 and 1/U0 (seq_rows values each),
  // then the interchange bits (seq_rows / 32 words)
  long long* d_soff = nullptr;
  void* seq_work = nullptr;
  long long seq_rows = 0;
  // variant 10: chunk entries (system, chunk) of its buckets ([2][n_cl]),
  // each system's first separator row (batch + 1 entries: its separators'
  // system is rows [d_sep_off[s], d_sep_off[s+1])), the separator arrays
  // (4 x sep_total, then x of the separators, then 4 carries per chunk) and
  // per system whether a chunk missed its bound (its systems also have
  // variant 9's workspace, for the re-solve)
  int* d_cl = nullptr;
  size_t n_cl = 0;
  long long* d_sep_off = nullptr;
  long long sep_total = 0;
  void* sep_work = nullptr;
  int* d_flag = nullptr;
  // the re-solve's chunk entries, separator offsets (sep_total2 rows in the
  // same separator arrays) and the systems its chunks fail in turn
  int* d_cl2 = nullptr;
  size_t n_cl2 = 0;
  long long* d_sep_off2 = nullptr;
  long long sep_total2 = 0;
  int* d_flag2 = nullptr;
  // the system holding row k * RAGGED_ROW_CHUNK (the row-parallel passes of
  // the refined solves)
  int* d_chunk_sys = nullptr;
  // per class and kind, the list of the class's systems of that kind: its
  // region in d_klists (d_reg[2 k + kind], -1: none) and its length
  // d_kcount[2 k + kind]
  int* d_klists = nullptr;
  int* d_kcount = nullptr;
  int* d_reg = nullptr;
  // mode 2: the state each forward solve starts from -- every candidate of
  // kind 1 (d_kinds0), the lists' initial lengths (d_kcount0) -- and per
  // system whether a chunk has handed it over (d_claim)
  unsigned char* d_kinds0 = nullptr;
  int* d_kcount0 = nullptr;
  int* d_claim = nullptr;
};

namespace {

int size_class(long long n) {
  int k = 0;
  while ((1ll << k) < n) ++k;
  return k;
}

constexpr int RAGGED_UNPIVOTED = 7;
constexpr int RAGGED_UNPIVOTED_LONG = 8;
constexpr int RAGGED_SEQUENTIAL = 9;
constexpr int RAGGED_CHUNKED = 10;

template <typename T>
int unpivoted_max_n() {
  return tdg::WML_CHUNK_R * (128 / (int)sizeof(T));  // one chunk-sized CTA (three per SM)
}

// long unpivoted systems: beyond one CTA, their separators' system within one
template <typename T>
long long long_unpivoted_max_n() {
  constexpr int M = 128 / (int)sizeof(T);
  return (long long)tdg::WMC_GEN_MAX_ROWS * M * M;
}

// sizes the unpivoted method serves (variant 7 up to unpivoted_max_n, 8 beyond)
template <typename T>
bool unpivoted_capable(long long n) {
  return n > tdg::RAGGED_TINY_MAX && n <= long_unpivoted_max_n<T>();
}

template <typename T>
bool variant_serves(int v, int max_n) {
  if (v == 0) return max_n <= tdg::RAGGED_TINY_MAX;
  if (v == RAGGED_UNPIVOTED) return max_n <= unpivoted_max_n<T>();
  if (v == RAGGED_SEQUENTIAL) return max_n >= 2;
  if (v == RAGGED_CHUNKED) return max_n > 64 && max_n <= tdg::pge_long_ragged_max_n<T>();
  return max_n >= 65 && max_n <= tdg::pge_variant_max_n<T>(v);
}

void free_plan(tridiag_ragged_plan* plan) {
  if (!plan) return;
  cudaFree(plan->d_kinds0);
  cudaFree(plan->d_kcount0);
  cudaFree(plan->d_claim);
  cudaFree(plan->d_klists);
  cudaFree(plan->d_kcount);
  cudaFree(plan->d_reg);
  cudaFree(plan->d_lists);
  cudaFree(plan->d_lr);
  cudaFree(plan->lr_work);
  cudaFree(plan->d_kinds);
  cudaFree(plan->d_tickets);
  cudaFree(plan->d_soff);
  cudaFree(plan->d_cl);
  cudaFree(plan->d_sep_off);
  cudaFree(plan->sep_work);
  cudaFree(plan->d_flag);
  cudaFree(plan->d_cl2);
  cudaFree(plan->d_sep_off2);
  cudaFree(plan->d_flag2);
  cudaFree(plan->seq_work);
  cudaFree(plan->d_chunk_sys);
  delete plan;
}

// The kinds in a pass of their own (an adjoint called before any solve of a
// mode-2 plan): one warp per system, grid-stride; a candidate (cand[s]) whose
// rows are all strictly dominant keeps kind 1, the others get kind 0 and go
// to their class's kind-0 list.
template <typename T>
__global__ void __launch_bounds__(256) ragged_classify_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                              const T* __restrict__ c,
                                                              const long long* __restrict__ offsets, int batch,
                                                              unsigned char* kinds,
                                                              const unsigned char* __restrict__ cand,
                                                              const int* __restrict__ reg, int* kcount, int* klists) {
  const int lane = threadIdx.x & 31;
  const int warps = (int)(gridDim.x * blockDim.x / 32);
  constexpr int U = 4;
  for (int s = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32); s < batch; s += warps) {
    const long long base = offsets[s];
    const long long n = offsets[s + 1] - base;
    bool ok = cand[s] != 0;
    if (ok) {
      for (long long i0 = 0; i0 < n && ok; i0 += 32 * U) {
        T av[U], bv[U], cv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const long long i = i0 + u * 32 + lane;
          av[u] = i > 0 && i < n ? __ldcs(a + base + i) : T(0);
          bv[u] = i < n ? __ldcs(b + base + i) : T(1);
          cv[u] = i < n - 1 ? __ldcs(c + base + i) : T(0);
        }
        bool lane_ok = true;
#pragma unroll
        for (int u = 0; u < U; ++u) lane_ok &= tdg::dominant_row(av[u], bv[u], cv[u]);
        ok = __all_sync(0xffffffffu, lane_ok);
      }
    }
    if (lane == 0) {
      kinds[s] = ok ? 1 : 0;
      if (cand[s] && !ok) {
        int cls = 0;
        while ((1ll << cls) < n) ++cls;
        const int r = reg[2 * cls];
        if (r >= 0) klists[r + atomicAdd(&kcount[2 * cls], 1)] = s;
      }
    }
  }
}

// mode: 0 every system pivoted; 1 the caller's host mask (1: needs no
// pivoting); 2 found by each solve.  unp_table (may be NULL, per class, < 0 =
// default): the variant of the kind-1 systems of a class the one-CTA
// unpivoted method serves (7, or a pivoted variant 1-6); chunk_r: 128-byte
// rows per CTA of variant 8 (0 = default).
template <typename T>
int plan_create(tridiag_ragged_plan** out, const long long* offsets, int batch, const int* table, int table_len,
                int mode, const unsigned char* mask, const int* unp_table, int chunk_r) {
  if (!out || !offsets || batch <= 0 || mode < 0 || mode > 2 || (mode == 1 && !mask)) return TRIDIAG_ERR_INVALID_VALUE;
  if (chunk_r == 0) chunk_r = tdg::WML_CHUNK_R;
  if (chunk_r != 64 && chunk_r != 128 && chunk_r != 256) return TRIDIAG_ERR_INVALID_VALUE;
  *out = nullptr;
  std::vector<std::vector<int>> by_class(TRIDIAG_RAGGED_CLASSES);
  for (int s = 0; s < batch; ++s) {
    const long long n = offsets[s + 1] - offsets[s];
    if (n < 1 || n > (1ll << (TRIDIAG_RAGGED_CLASSES - 1))) return TRIDIAG_ERR_INVALID_VALUE;
    by_class[size_class(n)].push_back(s);
  }
  auto* plan = new (std::nothrow) tridiag_ragged_plan;
  if (!plan) return TRIDIAG_ERR_WORKSPACE;
  plan->precision = sizeof(T) == 8 ? 1 : 0;
  plan->batch = batch;
  plan->total_rows = offsets[batch] - offsets[0];
  plan->row0 = offsets[0];
  plan->kinds_mode = mode;
  plan->unp_max = unpivoted_max_n<T>();
  plan->long_max = (int)long_unpivoted_max_n<T>();
  cudaGetDevice(&plan->device);
  constexpr int M = 128 / (int)sizeof(T);
  std::vector<int> lists;
  std::vector<int> longs;   // systems for variant 8
  std::vector<int> klists;  // the kind lists (kind 0 with room for the whole class)
  std::vector<int> reg(2 * TRIDIAG_RAGGED_CLASSES, -1), kcount(2 * TRIDIAG_RAGGED_CLASSES, 0);
  auto len = [&](int q) { return offsets[q + 1] - offsets[q]; };
  auto candidate = [&](int q) { return mode != 0 && unpivoted_capable<T>(len(q)) && (mode != 1 || mask[q]); };
  std::vector<unsigned char> kinds(batch, 0);  // (1: a candidate of kind 1)
  std::vector<long long> soff(batch, -1);      // variant 9 workspace rows
  long long seq_rows = 0;
  std::vector<int> cl_sys, cl_ch;                 // variant 10 chunk entries
  std::vector<long long> sep_rows(batch, 0);      // variant 10 separator rows per system
  const int CR = tdg::pge_long_chunk_rows();
  std::vector<int> cl2_sys, cl2_ch;               // ... of its re-solve
  std::vector<long long> sep2_rows(batch, 0);
  const int CR2 = tdg::pge_long_retry_rows();
  for (int k = 0; k < TRIDIAG_RAGGED_CLASSES; ++k) {
    auto& sys = by_class[k];
    if (sys.empty()) continue;
    std::sort(sys.begin(), sys.end(), [&](int p, int q) { return len(p) != len(q) ? len(p) > len(q) : p < q; });
    const int max_n = (int)len(sys[0]);
    const bool one_cta_unp = max_n <= unpivoted_max_n<T>();
    int vu = RAGGED_UNPIVOTED;
    if (mode != 0 && one_cta_unp && unp_table && k < table_len && unp_table[k] >= 0) {
      if (unp_table[k] != RAGGED_UNPIVOTED &&
          (unp_table[k] < 1 || unp_table[k] > 6 || !variant_serves<T>(unp_table[k], max_n))) {
        free_plan(plan);
        return TRIDIAG_ERR_NOT_SUPPORTED;
      }
      vu = unp_table[k];
    }
    // a class whose systems that need no pivoting are better served by a
    // pivoted variant (the autotuner's choice) is one pivoted bucket
    std::vector<int> cand, rest;
    for (int q : sys) (candidate(q) && vu == RAGGED_UNPIVOTED ? cand : rest).push_back(q);
    for (int q : cand) kinds[q] = 1;
    const bool capable = !cand.empty();
    int v = -1;
    if (table && k < table_len && table[k] >= 0) {
      if (!variant_serves<T>(table[k], max_n)) {  // an explicit choice that cannot serve the class
        free_plan(plan);
        return TRIDIAG_ERR_NOT_SUPPORTED;
      }
      v = table[k];
    }
    if (v < 0) v = max_n <= tdg::RAGGED_TINY_MAX ? 0 : tdg::pge_default_variant<T>(max_n);
    if (v == 0 && max_n > tdg::RAGGED_TINY_MAX)  // beyond every partitioned variant
      v = variant_serves<T>(RAGGED_CHUNKED, max_n) ? RAGGED_CHUNKED : RAGGED_SEQUENTIAL;
    if (v == RAGGED_SEQUENTIAL || v == RAGGED_CHUNKED)  // (variant 10 re-solves a failing system by 9)
      for (int q : sys) {
        soff[q] = seq_rows;
        seq_rows += (len(q) + 31) / 32 * 32;
      }
    size_t cl_off = cl_sys.size(), cl2_off = cl2_sys.size();
    int sep_variant = 0, sep_m_max = 0, sep2_variant = 0, sep2_m_max = 0;
    if (v == RAGGED_CHUNKED) {
      for (int q : sys) {
        const int nch = (int)((len(q) + CR - 1) / CR), nch2 = (int)((len(q) + CR2 - 1) / CR2);
        sep_rows[q] = (long long)nch * 128;
        sep2_rows[q] = (long long)nch2 * 128;
        for (int c = 0; c < nch; ++c) {
          cl_sys.push_back(q);
          cl_ch.push_back(c);
        }
        for (int c = 0; c < nch2; ++c) {
          cl2_sys.push_back(q);
          cl2_ch.push_back(c);
        }
      }
      const int max_sep = (int)((max_n + CR - 1) / CR) * 128, max_sep2 = (int)((max_n + CR2 - 1) / CR2) * 128;
      sep_variant = tdg::pge_default_variant<T>(max_sep);
      sep2_variant = tdg::pge_default_variant<T>(max_sep2);
      if (sep_variant <= 0 || sep2_variant <= 0) {
        free_plan(plan);
        return TRIDIAG_ERR_NOT_SUPPORTED;
      }
      sep_m_max = std::max(2, (max_sep + tdg::pge_variant_partitions(sep_variant) - 1) /
                                  tdg::pge_variant_partitions(sep_variant));
      sep2_m_max = std::max(2, (max_sep2 + tdg::pge_variant_partitions(sep2_variant) - 1) /
                                   tdg::pge_variant_partitions(sep2_variant));
    }
    const size_t cl_count = cl_sys.size() - cl_off, cl2_count = cl2_sys.size() - cl2_off;
    if (v < 0 || (v == 0 && max_n > tdg::RAGGED_TINY_MAX) || (v > 0 && !variant_serves<T>(v, max_n))) {
      free_plan(plan);
      return TRIDIAG_ERR_NOT_SUPPORTED;
    }
    const size_t list_off = lists.size();
    lists.insert(lists.end(), sys.begin(), sys.end());
    long long rows = 0;
    for (int q : sys) rows += len(q);
    if (capable) {
      // kind 1 (one-CTA classes): the candidates, a fixed list, which each
      // solve checks (mode 2) -- the ones that need pivoting are handed to
      // kind 0.  Kind 0: room for the whole class; its initial entries are
      // the systems without an unpivoted alternative (or the mask's 0s).
      if (one_cta_unp) {
        reg[2 * k + 1] = (int)klists.size();
        klists.insert(klists.end(), cand.begin(), cand.end());
        kcount[2 * k + 1] = (int)cand.size();
      } else {
        longs.insert(longs.end(), cand.begin(), cand.end());
      }
      reg[2 * k] = (int)klists.size();
      klists.insert(klists.end(), rest.begin(), rest.end());
      kcount[2 * k] = (int)rest.size();
      klists.resize(reg[2 * k] + sys.size(), -1);
    }
    auto add = [&](int variant, int kind, int count) {
      tridiag_ragged_plan::Bucket bk;
      bk.cls = k;
      bk.variant = variant;
      bk.count = count;
      bk.max_n = max_n;
      bk.m_max = variant == 0 || variant >= RAGGED_SEQUENTIAL ? 0
                 : variant == RAGGED_UNPIVOTED ? (max_n + M - 1) / M  // 128-byte rows of the longest system
                                               : std::max(2, (max_n + tdg::pge_variant_partitions(variant) - 1) /
                                                                 tdg::pge_variant_partitions(variant));
      bk.rows = rows;
      bk.list_off = list_off;
      bk.kind = kind;
      // resident CTAs with tickets only where the list grows on the device
      bk.ticket = kind == 0 && mode == 2 && variant != 0 && variant != RAGGED_SEQUENTIAL ? plan->n_tickets++ : -1;
      bk.klist = kind >= 0 ? 2 * k + kind : -1;
      bk.klist_off = kind >= 0 ? (size_t)reg[2 * k + kind] : 0;
      if (variant == RAGGED_CHUNKED) {
        bk.cl_off = cl_off;
        bk.cl_count = (int)cl_count;
        bk.sep_variant = sep_variant;
        bk.sep_m_max = sep_m_max;
        bk.cl2_off = cl2_off;
        bk.cl2_count = (int)cl2_count;
        bk.sep2_variant = sep2_variant;
        bk.sep2_m_max = sep2_m_max;
        bk.ticket2 = plan->n_tickets++;
      }
      plan->buckets.push_back(bk);
    };
    if (!capable) {
      add(v, -1, (int)sys.size());
      continue;
    }
    // within a class the unpivoted bucket runs first: its checks fill the pivoted one
    if (one_cta_unp) add(vu, 1, (int)cand.size());
    add(v, 0, mode == 2 ? (int)sys.size() : (int)rest.size());
  }
  // longest buckets first: their few, long launches start before the short ones fill the GPU
  std::stable_sort(plan->buckets.begin(), plan->buckets.end(),
                   [](const tridiag_ragged_plan::Bucket& p, const tridiag_ragged_plan::Bucket& q) {
                     return p.cls > q.cls;
                   });
  if (!longs.empty()) {
    const long long chunk_rows = (long long)chunk_r * M;
    std::sort(longs.begin(), longs.end(), [&](int p, int q) { return len(p) != len(q) ? len(p) > len(q) : p < q; });
    std::vector<long long> roff(longs.size() + 1, 0);
    std::vector<int> cl_li, cl_ch;
    int pmax = 0;
    long long rows = 0;
    for (size_t i = 0; i < longs.size(); ++i) {
      const long long n = len(longs[i]);
      // the chunk kernels put the system's first row after its 16-byte phase
      // in identity rows, so that every chunk starts on a 16-byte boundary
      long long phase = offsets[longs[i]] % (16 / (long long)sizeof(T));
      if ((n + phase + M - 1) / M > (long long)tdg::WMC_GEN_MAX_ROWS * M) phase = 0;  // (as the kernels decide)
      const long long P = (n + phase + M - 1) / M;
      roff[i + 1] = roff[i] + P;
      pmax = std::max(pmax, (int)P);
      rows += n;
      for (long long c = 0; c * chunk_rows < n + phase; ++c) {
        cl_li.push_back((int)i);
        cl_ch.push_back((int)c);
      }
    }
    plan->lr.L = (int)longs.size();
    plan->lr.C = (int)cl_li.size();
    plan->lr.P = roff.back();
    plan->lr.Pmax = pmax;
    plan->lr.R = chunk_r;
    const size_t b_lsys = longs.size() * sizeof(int), b_roff = roff.size() * sizeof(long long),
                 b_cl = cl_li.size() * sizeof(int);
    const size_t o_roff = (b_lsys + 255) / 256 * 256, o_li = o_roff + (b_roff + 255) / 256 * 256,
                 o_ch = o_li + (b_cl + 255) / 256 * 256, o_end = o_ch + (b_cl + 255) / 256 * 256;
    char* mem = nullptr;
    if (cudaMalloc(&mem, o_end) != cudaSuccess ||
        cudaMalloc(&plan->lr_work, tdg::wml_ragged_workspace_elems<T>(plan->lr.P) * sizeof(T)) != cudaSuccess) {
      cudaFree(mem);
      free_plan(plan);
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
    const int max_n = (int)len(longs[0]);
    bk.cls = size_class(max_n);
    bk.variant = RAGGED_UNPIVOTED_LONG;
    bk.count = (int)longs.size();
    bk.max_n = max_n;
    bk.m_max = 0;
    bk.rows = rows;
    bk.list_off = 0;
    bk.kind = 1;
    bk.ticket = -1;
    bk.klist = -1;
    bk.klist_off = 0;
    plan->buckets.insert(plan->buckets.begin(), bk);  // longest work first (and before the pivoted long buckets)
  }
  if (cudaMalloc(&plan->d_lists, std::max<size_t>(lists.size(), 1) * sizeof(int)) != cudaSuccess ||
      cudaMemcpy(plan->d_lists, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    free_plan(plan);
    return TRIDIAG_ERR_CUDA;
  }
  {
    std::vector<int> cs((size_t)((plan->total_rows + tdg::RAGGED_ROW_CHUNK - 1) / tdg::RAGGED_ROW_CHUNK));
    int q = 0;
    for (size_t k = 0; k < cs.size(); ++k) {
      const long long r = (long long)k * tdg::RAGGED_ROW_CHUNK;
      while (offsets[q + 1] <= r) ++q;
      cs[k] = q;
    }
    if (cudaMalloc(&plan->d_chunk_sys, std::max<size_t>(cs.size(), 1) * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(plan->d_chunk_sys, cs.data(), cs.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
      free_plan(plan);
      return TRIDIAG_ERR_CUDA;
    }
  }
  if (!cl_sys.empty()) {
    plan->n_cl = cl_sys.size();
    plan->n_cl2 = cl2_sys.size();
    std::vector<long long> so(batch + 1, 0), so2(batch + 1, 0);
    for (int q = 0; q < batch; ++q) {
      so[q + 1] = so[q] + sep_rows[q];
      so2[q + 1] = so2[q] + sep2_rows[q];
    }
    plan->sep_total = so[batch];
    plan->sep_total2 = so2[batch];
    const size_t st = (size_t)std::max(plan->sep_total, plan->sep_total2);  // (the two passes share the arrays)
    const size_t wbytes = (5 * st + 4 * (st / 128)) * sizeof(T);
    if (cudaMalloc(&plan->d_cl2, 2 * plan->n_cl2 * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(plan->d_cl2, cl2_sys.data(), plan->n_cl2 * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(plan->d_cl2 + plan->n_cl2, cl2_ch.data(), plan->n_cl2 * sizeof(int), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->d_sep_off2, (size_t)(batch + 1) * sizeof(long long)) != cudaSuccess ||
        cudaMemcpy(plan->d_sep_off2, so2.data(), (size_t)(batch + 1) * sizeof(long long), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->d_flag2, (size_t)batch * sizeof(int)) != cudaSuccess) {
      free_plan(plan);
      return TRIDIAG_ERR_CUDA;
    }
    if (cudaMalloc(&plan->d_cl, 2 * plan->n_cl * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(plan->d_cl, cl_sys.data(), plan->n_cl * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(plan->d_cl + plan->n_cl, cl_ch.data(), plan->n_cl * sizeof(int), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->d_sep_off, (size_t)(batch + 1) * sizeof(long long)) != cudaSuccess ||
        cudaMemcpy(plan->d_sep_off, so.data(), (size_t)(batch + 1) * sizeof(long long), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->sep_work, wbytes) != cudaSuccess ||
        cudaMalloc(&plan->d_flag, (size_t)batch * sizeof(int)) != cudaSuccess) {
      free_plan(plan);
      return TRIDIAG_ERR_CUDA;
    }
  }
  if (seq_rows > 0) {
    plan->seq_rows = seq_rows;
    const size_t wbytes = 2 * (size_t)seq_rows * sizeof(T) + (size_t)seq_rows / 32 * sizeof(unsigned);
    if (cudaMalloc(&plan->d_soff, (size_t)batch * sizeof(long long)) != cudaSuccess ||
        cudaMemcpy(plan->d_soff, soff.data(), (size_t)batch * sizeof(long long), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->seq_work, wbytes) != cudaSuccess) {
      free_plan(plan);
      return TRIDIAG_ERR_CUDA;
    }
  }
  if (plan->n_tickets > 0 && cudaMalloc(&plan->d_tickets, plan->n_tickets * sizeof(int)) != cudaSuccess) {
    free_plan(plan);
    return TRIDIAG_ERR_CUDA;
  }
  if (mode != 0) {
    const size_t nk = std::max<size_t>(klists.size(), 1);
    if (cudaMalloc(&plan->d_kinds, (size_t)batch) != cudaSuccess ||
        cudaMemcpy(plan->d_kinds, kinds.data(), (size_t)batch, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc(&plan->d_klists, nk * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(plan->d_klists, klists.data(), klists.size() * sizeof(int), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->d_kcount, kcount.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(plan->d_kcount, kcount.data(), kcount.size() * sizeof(int), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc(&plan->d_reg, reg.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(plan->d_reg, reg.data(), reg.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        (mode == 2 && (cudaMalloc(&plan->d_kinds0, (size_t)batch) != cudaSuccess ||
                       cudaMemcpy(plan->d_kinds0, kinds.data(), (size_t)batch, cudaMemcpyHostToDevice) !=
                           cudaSuccess ||
                       cudaMalloc(&plan->d_kcount0, kcount.size() * sizeof(int)) != cudaSuccess ||
                       cudaMemcpy(plan->d_kcount0, kcount.data(), kcount.size() * sizeof(int),
                                  cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMalloc(&plan->d_claim, (size_t)batch * sizeof(int)) != cudaSuccess))) {
      free_plan(plan);
      return TRIDIAG_ERR_CUDA;
    }
    plan->classified = mode == 1;
  }
  *out = plan;
  return TRIDIAG_SUCCESS;
}

// recheck (forward solves of a mode-2 plan): the unpivoted kernels check
// the rows they stage and the marks follow; false: the solve runs on the
// plan's marks as they stand (marked first, where it has none, by the
// classify pass on ka, kb, kc -- a, b, c when NULL).  pivoted_only: the
// buckets of the systems marked for the unpivoted kernels are skipped (their
// x is left as it is).
template <typename T>
int plan_run(tridiag_ragged_plan* plan, int mode, const T* a, const T* b, const T* c, const T* d, T* x, const T* xf,
             T* ga, T* gb, T* gc, int* info, const long long* offsets, cudaStream_t s, bool recheck = true,
             const T* ka = nullptr, const T* kb = nullptr, const T* kc = nullptr, bool pivoted_only = false) {
  if (!plan || !a || !b || !c || !d || !x || !offsets) return TRIDIAG_ERR_INVALID_VALUE;
  if (plan->precision != (sizeof(T) == 8 ? 1 : 0)) return TRIDIAG_ERR_INVALID_VALUE;
  if (mode == 1 && (!xf || !ga || !gb || !gc)) return TRIDIAG_ERR_INVALID_VALUE;
  if (plan->n_tickets > 0 && cudaMemsetAsync(plan->d_tickets, 0, plan->n_tickets * sizeof(int), s) != cudaSuccess)
    return TRIDIAG_ERR_CUDA;
  const bool check = plan->kinds_mode == 2 && mode == 0 && recheck;
  if (plan->kinds_mode == 2) {
    // every solve starts from the candidates; its unpivoted kernels hand the
    // systems that need pivoting over as they stage them.  (An adjoint with
    // no solve before it sorts the systems in a pass of its own.)
    if (check || !plan->classified) {
      const size_t nk = 2 * TRIDIAG_RAGGED_CLASSES * sizeof(int);
      if (cudaMemcpyAsync(plan->d_kinds, plan->d_kinds0, (size_t)plan->batch, cudaMemcpyDeviceToDevice, s) !=
              cudaSuccess ||
          cudaMemcpyAsync(plan->d_kcount, plan->d_kcount0, nk, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
          cudaMemsetAsync(plan->d_claim, 0, (size_t)plan->batch * sizeof(int), s) != cudaSuccess)
        return TRIDIAG_ERR_CUDA;
    }
    if (!check && !plan->classified) {
      int dev = 0, sms = 152;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      const int grid = std::min((plan->batch + 7) / 8, sms * 8);
      ragged_classify_kernel<T><<<grid, 256, 0, s>>>(ka ? ka : a, kb ? kb : b, kc ? kc : c, offsets, plan->batch,
                                                     plan->d_kinds, plan->d_kinds0, plan->d_reg, plan->d_kcount,
                                                     plan->d_klists);
      if (cudaGetLastError() != cudaSuccess) return TRIDIAG_ERR_CUDA;
    }
    plan->classified = true;
  }
  tdg::RaggedCheck chk;
  if (check) {
    chk.kinds = plan->d_kinds;
    chk.claim = plan->d_claim;
    chk.reg = plan->d_reg;
    chk.kcount = plan->d_kcount;
    chk.klists = plan->d_klists;
  }
  for (const auto& bk : plan->buckets) {
    if (pivoted_only && bk.kind == 1) continue;
    // a bucket of one kind runs through that kind's list of its class
    const int* list = bk.klist >= 0 ? plan->d_klists + bk.klist_off : plan->d_lists + bk.list_off;
    tdg::BucketTicket tk;
    tk.ticket = bk.ticket >= 0 ? plan->d_tickets + bk.ticket : nullptr;
    // kind 0: the list's length on the device (grown by the checks); kind 1:
    // the fixed candidates, of which the adjoint skips those handed over
    tk.dcount = bk.ticket >= 0 ? plan->d_kcount + bk.klist : nullptr;
    tk.kinds = bk.kind == 1 && !check && plan->kinds_mode == 2 ? plan->d_kinds : nullptr;
    tk.want = bk.kind;
    const tdg::BucketTicket* tkp = bk.kind >= 0 ? &tk : nullptr;
    cudaError_t e = cudaErrorInvalidValue;  // (a variant no branch serves is an error)
    if (bk.variant == RAGGED_UNPIVOTED_LONG)
      e = mode == 0 ? tdg::launch_wml_ragged<T>(0, a, b, c, d, nullptr, x, nullptr, nullptr, nullptr, offsets,
                                                plan->lr, static_cast<T*>(plan->lr_work), info, s, plan->d_kinds,
                                                check ? &chk : nullptr)
                    : tdg::launch_wml_ragged<T>(1, a, b, c, d, xf, x, ga, gb, gc, offsets, plan->lr,
                                                static_cast<T*>(plan->lr_work), info, s, plan->d_kinds);
    else if (bk.variant == 0)
      e = tdg::launch_tiny<T>(mode, a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, bk.count, s);
    else if (bk.variant == RAGGED_SEQUENTIAL) {
      T* w1 = static_cast<T*>(plan->seq_work);
      e = tdg::launch_ragged_seq<T>(mode, a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, bk.count,
                                    bk.kind == 0 && plan->kinds_mode == 2 ? plan->d_kcount + bk.klist : nullptr,
                                    plan->d_soff, w1, w1 + plan->seq_rows,
                                    reinterpret_cast<unsigned*>(w1 + 2 * plan->seq_rows), nullptr, s);
    } else if (bk.variant == RAGGED_CHUNKED) {
      // the chunked partitioned solve (of A^T for the adjoint); the systems a
      // chunk fails solved again in chunks of 31-row partitions; the
      // adjoint's gradients; variant 9 for the systems that fail twice
      tdg::BucketTicket tc = tk;
      tc.kinds = bk.kind >= 0 ? plan->d_kinds : nullptr;
      tc.want = bk.kind >= 0 ? bk.kind : 0;
      const int* cls = plan->d_cl + bk.cl_off;
      const int* clc = plan->d_cl + plan->n_cl + bk.cl_off;
      const int* cls2 = plan->d_cl2 + bk.cl2_off;
      const int* clc2 = plan->d_cl2 + plan->n_cl2 + bk.cl2_off;
      const size_t st = (size_t)std::max(plan->sep_total, plan->sep_total2);
      T* sep = static_cast<T*>(plan->sep_work);
      const T* pa = mode == 0 ? a : c - 1;
      const T* pc = mode == 0 ? c : a + 1;
      e = cudaMemsetAsync(plan->d_flag, 0, (size_t)plan->batch * sizeof(int), s);
      if (e == cudaSuccess) e = cudaMemsetAsync(plan->d_flag2, 0, (size_t)plan->batch * sizeof(int), s);
      if (e == cudaSuccess)
        e = tdg::launch_pge_long_ragged<T>(pa, b, pc, d, x, offsets, cls, clc, bk.cl_count, plan->d_sep_off,
                                           (size_t)plan->sep_total, sep, sep + 4 * st, sep + 5 * st, plan->d_flag,
                                           bk.sep_variant, bk.sep_m_max, list, bk.count, &tc, s,
                                           tdg::pge_long_chunk_rows());
      if (e == cudaSuccess) {
        tdg::BucketTicket t2 = tc;  // the re-solve: the systems flagged above, through their own ticket
        t2.ticket = plan->d_tickets + bk.ticket2;
        t2.dcount = bk.kind == 0 && plan->kinds_mode == 2 ? plan->d_kcount + bk.klist : nullptr;
        t2.only = plan->d_flag;
        e = tdg::launch_pge_long_ragged<T>(pa, b, pc, d, x, offsets, cls2, clc2, bk.cl2_count, plan->d_sep_off2,
                                           (size_t)plan->sep_total2, sep, sep + 4 * st, sep + 5 * st,
                                           plan->d_flag2, bk.sep2_variant, bk.sep2_m_max, list, bk.count, &t2, s,
                                           tdg::pge_long_retry_rows());
      }
      if (e == cudaSuccess && mode == 1) {
        tdg::ragged_chunk_gradient_kernel<T><<<(unsigned)(((long long)bk.cl_count * 32 + 255) / 256), 256, 0, s>>>(
            x, xf, ga, gb, gc, offsets, cls, clc, bk.cl_count, tdg::pge_long_chunk_rows(), tc.kinds, tc.want,
            plan->d_flag2);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) {
        T* w1 = static_cast<T*>(plan->seq_work);
        e = tdg::launch_ragged_seq<T>(mode, a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, bk.count,
                                      bk.kind == 0 && plan->kinds_mode == 2 ? plan->d_kcount + bk.klist : nullptr,
                                      plan->d_soff, w1, w1 + plan->seq_rows,
                                      reinterpret_cast<unsigned*>(w1 + 2 * plan->seq_rows), plan->d_flag2, s);
      }
    } else if (bk.variant == RAGGED_UNPIVOTED)
      e = mode == 0 ? tdg::launch_wmc_ragged<T>(0, a, b, c, d, nullptr, x, nullptr, nullptr, nullptr, offsets, list,
                                                bk.count, bk.m_max, info, s, tkp, nullptr, check ? &chk : nullptr)
                    : tdg::launch_wmc_ragged<T>(1, a, b, c, d, xf, ga, gb, gc, x, offsets, list, bk.count, bk.m_max,
                                                info, s, tkp);
    else if (bk.variant >= 1 && bk.variant <= 6)
      e = tdg::launch_pge_ragged<T>(bk.variant, mode, a, b, c, d, x, xf, ga, gb, gc, info, offsets, list, bk.count,
                                    bk.m_max, s, tkp);
    if (e != cudaSuccess) return TRIDIAG_ERR_CUDA;
  }
  return TRIDIAG_SUCCESS;
}

// Mixed-precision refined solve of a ragged FP64 batch through an FP32 plan
// of the same offsets: FP32 copies of A (trans: of A^T) and rhs, an FP32
// solve, then `iters` steps of FP64 residual -> FP32 correction solve, the
// FP64 iterate updated each time; out receives x (trans: lambda = A^{-T}
// rhs).  Then `piv_iters` more steps on the systems the plan solves with
// pivoting only (all of them for a plan without marks): their residual, their
// correction solves, their rows of out updated -- the systems marked for the
// unpivoted kernels are diagonally dominant, and their FP32 solves need fewer
// steps.  Workspace: five FP32 rows-long arrays and one FP64 one.
inline size_t up256(size_t x) { return (x + 255) / 256 * 256; }

size_t ragged_refine_ws(long long rows) {
  return 5 * up256((size_t)rows * sizeof(float)) + up256((size_t)rows * sizeof(double));
}

int ragged_refine_impl(tridiag_ragged_plan* plan32, bool trans, const double* a, const double* b, const double* c,
                       const double* rhs, double* out, int iters, int piv_iters, void* work, size_t work_bytes,
                       const long long* offsets, cudaStream_t s) {
  if (!plan32 || !a || !b || !c || !rhs || !out || !offsets || iters < 0 || iters > 8 || piv_iters < 0 ||
      piv_iters > 8)
    return TRIDIAG_ERR_INVALID_VALUE;
  if (plan32->precision != 0) return TRIDIAG_ERR_INVALID_VALUE;  // the solves run in FP32
  if (plan32->row0 != 0) return TRIDIAG_ERR_INVALID_VALUE;       // rows counted from offsets[0] = 0
  const long long rows = plan32->total_rows;
  if (!work || work_bytes < ragged_refine_ws(rows)) return TRIDIAG_ERR_WORKSPACE;
  char* w = static_cast<char*>(work);
  const size_t f = up256((size_t)rows * sizeof(float));
  float* a32 = reinterpret_cast<float*>(w);
  float* b32 = reinterpret_cast<float*>(w + f);
  float* c32 = reinterpret_cast<float*>(w + 2 * f);
  float* v0 = reinterpret_cast<float*>(w + 3 * f);  // FP32 right-hand side / residual
  float* v1 = reinterpret_cast<float*>(w + 4 * f);  // FP32 solution / correction
  double* w64 = reinterpret_cast<double*>(w + 5 * f);
  const tdg::RaggedRows rr{offsets, plan32->batch, plan32->d_chunk_sys, rows};
  if (tdg::launch_ragged_narrow(trans, a, b, c, rhs, a32, b32, c32, v0, rr, s) != cudaSuccess)
    return TRIDIAG_ERR_CUDA;
  // The FP32 solves of a classifying plan: the first forward solve marks the
  // systems by A's rows and the later ones reuse the marks; the solves of A^T
  // reuse the marks of A as they stand -- A strictly diagonally dominant by
  // rows needs no pivoting for A^T either (a check of A^T's rows would send
  // most long systems to the pivoted kernels) -- marking by A's rows first
  // where the plan has no marks (A's row i = (c32[i-1], b32[i], a32[i+1]) of
  // the transposed copies).
  const float* ka = trans ? c32 - 1 : nullptr;
  const float* kc = trans ? a32 + 1 : nullptr;
  int st = plan_run<float>(plan32, 0, a32, b32, c32, v0, v1, nullptr, nullptr, nullptr, nullptr, nullptr, offsets, s,
                           !trans, ka, b32, kc);
  if (st != TRIDIAG_SUCCESS) return st;
  // the FP64 iterate alternates between w64 and out so that the last step lands in out
  double* xs[2] = {(iters % 2) ? out : w64, (iters % 2) ? w64 : out};
  const double* xcur = nullptr;
  for (int it = 0; it < iters; ++it) {
    double* xnew = xs[it % 2];
    if (tdg::launch_ragged_residual(trans, a, b, c, rhs, xcur, v1, xnew, v0, rr, s) != cudaSuccess)
      return TRIDIAG_ERR_CUDA;
    st = plan_run<float>(plan32, 0, a32, b32, c32, v0, v1, nullptr, nullptr, nullptr, nullptr, nullptr, offsets, s,
                         false, ka, b32, kc);
    if (st != TRIDIAG_SUCCESS) return st;
    xcur = xnew;
  }
  if (tdg::launch_update(xcur, v1, out, (size_t)rows, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
  const unsigned char* sel = plan32->kinds_mode != 0 ? plan32->d_kinds : nullptr;
  for (int it = 0; it < piv_iters; ++it) {
    if (tdg::launch_ragged_residual_sel(trans, a, b, c, rhs, out, v0, sel, rr, s) != cudaSuccess)
      return TRIDIAG_ERR_CUDA;
    st = plan_run<float>(plan32, 0, a32, b32, c32, v0, v1, nullptr, nullptr, nullptr, nullptr, nullptr, offsets, s,
                         false, ka, b32, kc, true);
    if (st != TRIDIAG_SUCCESS) return st;
    if (tdg::launch_ragged_update_sel(out, v1, sel, rr, s) != cudaSuccess) return TRIDIAG_ERR_CUDA;
  }
  return TRIDIAG_SUCCESS;
}

}  // namespace

extern "C" {

int tridiag_ragged_plan_create(tridiag_ragged_plan** plan, int precision, const long long* offsets_host, int batch,
                               const int* variant_by_class, int n_classes) {
  return precision ? plan_create<double>(plan, offsets_host, batch, variant_by_class, n_classes, 0, nullptr, nullptr, 0)
                   : plan_create<float>(plan, offsets_host, batch, variant_by_class, n_classes, 0, nullptr, nullptr, 0);
}

int tridiag_ragged_plan_create_ex(tridiag_ragged_plan** plan, int precision, const long long* offsets_host,
                                  int batch, const int* variant_by_class, int n_classes,
                                  const unsigned char* no_pivoting_host) {
  const int mode = no_pivoting_host ? 1 : 0;
  return precision ? plan_create<double>(plan, offsets_host, batch, variant_by_class, n_classes, mode,
                                         no_pivoting_host, nullptr, 0)
                   : plan_create<float>(plan, offsets_host, batch, variant_by_class, n_classes, mode,
                                        no_pivoting_host, nullptr, 0);
}

int tridiag_ragged_plan_create_classify(tridiag_ragged_plan** plan, int precision, const long long* offsets_host,
                                        int batch, const int* variant_by_class, const int* unpivoted_by_class,
                                        int n_classes, int chunk_rows) {
  return precision ? plan_create<double>(plan, offsets_host, batch, variant_by_class, n_classes, 2, nullptr,
                                         unpivoted_by_class, chunk_rows)
                   : plan_create<float>(plan, offsets_host, batch, variant_by_class, n_classes, 2, nullptr,
                                        unpivoted_by_class, chunk_rows);
}

int tridiag_ragged_plan_kinds(const tridiag_ragged_plan* plan, unsigned char* kinds_host) {
  if (!plan || !kinds_host) return TRIDIAG_ERR_INVALID_VALUE;
  if (!plan->d_kinds || !plan->classified) return TRIDIAG_ERR_NOT_SUPPORTED;
  return cudaMemcpy(kinds_host, plan->d_kinds, (size_t)plan->batch, cudaMemcpyDeviceToHost) == cudaSuccess
             ? TRIDIAG_SUCCESS
             : TRIDIAG_ERR_CUDA;
}

void tridiag_ragged_plan_destroy(tridiag_ragged_plan* plan) { free_plan(plan); }

size_t tridiag_ragged_refine_workspace_size(long long total_rows) {
  return total_rows > 0 ? ragged_refine_ws(total_rows) : 0;
}

int tridiag_ragged_refine_ex_double(tridiag_ragged_plan* plan32, const double* a, const double* b, const double* c,
                                    const double* d, double* x, int iters, int pivoted_iters, void* work,
                                    size_t work_bytes, const long long* offsets, void* stream) {
  return ragged_refine_impl(plan32, false, a, b, c, d, x, iters, pivoted_iters, work, work_bytes, offsets,
                            (cudaStream_t)stream);
}

int tridiag_ragged_refine_double(tridiag_ragged_plan* plan32, const double* a, const double* b, const double* c,
                                 const double* d, double* x, int iters, void* work, size_t work_bytes,
                                 const long long* offsets, void* stream) {
  return tridiag_ragged_refine_ex_double(plan32, a, b, c, d, x, iters, 0, work, work_bytes, offsets, stream);
}

int tridiag_ragged_refine_adjoint_ex_double(tridiag_ragged_plan* plan32, const double* a, const double* b,
                                            const double* c, const double* x, const double* xbar, double* ga,
                                            double* gb, double* gc, double* gd, int iters, int pivoted_iters,
                                            void* work, size_t work_bytes, const long long* offsets, void* stream) {
  if (!x || !ga || !gb || !gc || !gd) return TRIDIAG_ERR_INVALID_VALUE;
  const cudaStream_t s = (cudaStream_t)stream;
  const int st =
      ragged_refine_impl(plan32, true, a, b, c, xbar, gd, iters, pivoted_iters, work, work_bytes, offsets, s);
  if (st != TRIDIAG_SUCCESS) return st;
  const tdg::RaggedRows rr{offsets, plan32->batch, plan32->d_chunk_sys, plan32->total_rows};
  return tdg::launch_ragged_gradient(gd, x, ga, gb, gc, rr, s) == cudaSuccess
             ? TRIDIAG_SUCCESS
             : TRIDIAG_ERR_CUDA;
}

int tridiag_ragged_refine_adjoint_double(tridiag_ragged_plan* plan32, const double* a, const double* b,
                                         const double* c, const double* x, const double* xbar, double* ga,
                                         double* gb, double* gc, double* gd, int iters, void* work,
                                         size_t work_bytes, const long long* offsets, void* stream) {
  return tridiag_ragged_refine_adjoint_ex_double(plan32, a, b, c, x, xbar, ga, gb, gc, gd, iters, 0, work,
                                                 work_bytes, offsets, stream);
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
  if (variant == RAGGED_SEQUENTIAL) return 0x7fffffff;
  if (variant == RAGGED_CHUNKED)
    return precision ? tdg::pge_long_ragged_max_n<double>() : tdg::pge_long_ragged_max_n<float>();
  if (variant == RAGGED_UNPIVOTED_LONG)
    return precision ? tdg::WMC_GEN_MAX_ROWS * 16 * 16 : tdg::WMC_GEN_MAX_ROWS * 32 * 32;
  return precision ? tdg::pge_variant_max_n<double>(variant) : tdg::pge_variant_max_n<float>(variant);
}

int tridiag_ragged_solve_single(tridiag_ragged_plan* plan, const float* a, const float* b, const float* c,
                                const float* d, float* x, int* info, const long long* offsets, void* stream) {
  return plan_run<float>(plan, 0, a, b, c, d, x, nullptr, nullptr, nullptr, nullptr, info, offsets,
                         (cudaStream_t)stream);
}
int tridiag_ragged_solve_double(tridiag_ragged_plan* plan, const double* a, const double* b, const double* c,
                                const double* d, double* x, int* info, const long long* offsets, void* stream) {
  return plan_run<double>(plan, 0, a, b, c, d, x, nullptr, nullptr, nullptr, nullptr, info, offsets,
                          (cudaStream_t)stream);
}
int tridiag_ragged_adjoint_single(tridiag_ragged_plan* plan, const float* a, const float* b, const float* c,
                                  const float* x, const float* xbar, float* ga, float* gb, float* gc, float* gd,
                                  int* info, const long long* offsets, void* stream) {
  return plan_run<float>(plan, 1, a, b, c, xbar, gd, x, ga, gb, gc, info, offsets, (cudaStream_t)stream);
}
int tridiag_ragged_adjoint_double(tridiag_ragged_plan* plan, const double* a, const double* b,
                                  const double* c, const double* x, const double* xbar, double* ga, double* gb,
                                  double* gc, double* gd, int* info, const long long* offsets, void* stream) {
  return plan_run<double>(plan, 1, a, b, c, xbar, gd, x, ga, gb, gc, info, offsets, (cudaStream_t)stream);
}

}  // extern "C"
