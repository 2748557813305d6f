// Partitioned Thomas for batch-interleaved systems (layout 2), out of place.
//
// A thread-per-system sweep has one dependent chain per system (two with the
// two-ended sweep), so a batch of a few thousand systems occupies only a
// fraction of GB300's 608 SM sub-partitions, and FP64 -- one warp
// instruction per ~80 cycles per sub-partition -- needs all of them busy.
// Here every system is cut into P partitions of L rows; thread (j, p) owns
// partition p of system j, and a warp holds 32 adjacent systems at the same
// partition index, so every row access of a warp is one coalesced line of
// the interleaved arrays.  P is chosen for about four warps per
// sub-partition.
//
// Rows: partition p covers [p L, min(n, (p+1) L)); its last row is the
// separator s_p (p < P-1), the others are its interior.
//   * p = 0 sweeps its interior top-down (Thomas: 7 FP64 operations per
//     row), leaving x_last = d'_l - c'_l s_0;
//   * p = P-1 sweeps bottom-up, leaving x_first = d''_f - a''_f s_{P-2};
//   * interior partitions sweep top-down carrying the left spike (the a of
//     their first row times s_{p-1}) and the relation of their first row,
//     x_first = alpha - beta s_{p-1} - gamma x_{i+1}, 12 operations per row;
//     they leave x_first and x_last as functions of s_{p-1} and s_p.
// The separators' tridiagonal system (P-1 unknowns per system) is then
// formed from those relations, row by row in parallel, and solved by one
// thread per system, and a third launch back-substitutes every partition
// with its separators known.
// Factors: d' (d'') in x, c' (a'' of the last partition) and the spike v' in
// two n x batch workspace arrays, the end relations and the separator system
// in two small ones.
//
// Reference: Thomas_kernel (one thread per system, Tridiagonal_CUDA/
// tridiagonal_basic.cu:4-30) and the CPU Thomas (Tridiagonal_AVX512/
// tridiagonal_basic.cpp:6-27): the same elimination without pivoting, for
// the systems the reference's Thomas rows are meant for (diagonally
// dominant ones).
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace tdg {

namespace {

template <typename T>
struct Ipt {
  const T* a;
  const T* b;
  const T* c;
  const T* d;
  T* x;    // d' / d'' during the sweeps, x at the end
  T* cp;   // c' (a'' in the last partition)
  T* vp;   // left spike v' of interior partitions
  T* rel;  // [6][P][batch]: end relations of each partition
  T* sys;  // [2][P][batch]: the separators s in the second half
  int n, batch, P, L;
};

template <typename T>
__device__ __forceinline__ size_t at(const Ipt<T>& g, int i, int j) {
  return (size_t)i * (size_t)g.batch + (size_t)j;
}
template <typename T>
__device__ __forceinline__ T& relv(const Ipt<T>& g, int k, int p, int j) {
  return g.rel[((size_t)k * g.P + p) * g.batch + j];
}

constexpr int IPT_U = 4;  // rows loaded ahead of the recurrence

// ---- forward sweeps -------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(128) ipt_forward_kernel(const Ipt<T> g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (j >= g.batch) return;
  const int lo = p * g.L, hi = min(g.n, lo + g.L);
  if (p == g.P - 1) {
    // bottom-up over [lo, n): x_i = d''_i - a''_i x_{i-1}
    T ap = T(0), dp = T(0);
    T na[IPT_U], nb[IPT_U], nc[IPT_U], nd[IPT_U];
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) {
      const int i = g.n - 1 - u;
      if (i >= lo) {
        const size_t o = at(g, i, j);
        na[u] = ld_stream(g.a + o);
        nb[u] = ld_stream(g.b + o);
        nc[u] = i + 1 < g.n ? ld_stream(g.c + o) : T(0);
        nd[u] = ld_stream(g.d + o);
      }
    }
    for (int i0 = g.n - 1; i0 >= lo; i0 -= IPT_U) {
      T ra[IPT_U], rb[IPT_U], rc[IPT_U], rd[IPT_U];
#pragma unroll
      for (int u = 0; u < IPT_U; ++u) { ra[u] = na[u]; rb[u] = nb[u]; rc[u] = nc[u]; rd[u] = nd[u]; }
#pragma unroll
      for (int u = 0; u < IPT_U; ++u) {
        const int i = i0 - IPT_U - u;
        if (i >= lo) {
          const size_t o = at(g, i, j);
          na[u] = ld_stream(g.a + o);
          nb[u] = ld_stream(g.b + o);
          nc[u] = ld_stream(g.c + o);
          nd[u] = ld_stream(g.d + o);
        }
      }
#pragma unroll
      for (int u = 0; u < IPT_U; ++u) {
        const int i = i0 - u;
        if (i >= lo) {
          const T r = rcp(fma(-rc[u], ap, rb[u]));
          ap = ra[u] * r;
          dp = fma(-rc[u], dp, rd[u]) * r;
          const size_t o = at(g, i, j);
          g.cp[o] = ap;
          g.x[o] = dp;
        }
      }
    }
    relv(g, 0, p, j) = dp;
    relv(g, 1, p, j) = ap;
    return;
  }
  // top-down over the interior [lo, hi - 1)
  const int last = hi - 2;
  const bool first = p == 0;
  T cp = T(0), dp = T(0), vp = T(0);
  T al = T(0), be = T(0), ga = T(0);  // x_first = al - be s_{p-1} - ga x_{i+1}
  T na[IPT_U], nb[IPT_U], nc[IPT_U], nd[IPT_U];
#pragma unroll
  for (int u = 0; u < IPT_U; ++u) {
    const int i = lo + u;
    if (i <= last) {
      const size_t o = at(g, i, j);
      na[u] = i > 0 ? ld_stream(g.a + o) : T(0);
      nb[u] = ld_stream(g.b + o);
      nc[u] = ld_stream(g.c + o);
      nd[u] = ld_stream(g.d + o);
    }
  }
  for (int i0 = lo; i0 <= last; i0 += IPT_U) {
    T ra[IPT_U], rb[IPT_U], rc[IPT_U], rd[IPT_U];
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) { ra[u] = na[u]; rb[u] = nb[u]; rc[u] = nc[u]; rd[u] = nd[u]; }
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) {
      const int i = i0 + IPT_U + u;
      if (i <= last) {
        const size_t o = at(g, i, j);
        na[u] = ld_stream(g.a + o);
        nb[u] = ld_stream(g.b + o);
        nc[u] = ld_stream(g.c + o);
        nd[u] = ld_stream(g.d + o);
      }
    }
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) {
      const int i = i0 + u;
      if (i <= last) {
        const size_t o = at(g, i, j);
        if (first) {
          const T r = rcp(fma(-ra[u], cp, rb[u]));
          cp = rc[u] * r;
          dp = fma(-ra[u], dp, rd[u]) * r;
        } else if (i == lo) {
          // the partition's first row: its a multiplies the previous separator
          const T r = rcp(rb[u]);
          cp = rc[u] * r;
          dp = rd[u] * r;
          vp = ra[u] * r;
          al = dp;
          be = vp;
          ga = cp;
        } else {
          const T r = rcp(fma(-ra[u], cp, rb[u]));
          cp = rc[u] * r;
          dp = fma(-ra[u], dp, rd[u]) * r;
          vp = (-ra[u] * vp) * r;
          al = fma(-ga, dp, al);
          be = fma(-ga, vp, be);
          ga = -ga * cp;
        }
        g.cp[o] = cp;
        g.x[o] = dp;
        if (!first) g.vp[o] = vp;
      }
    }
  }
  relv(g, 0, p, j) = dp;  // x_last = dp - vp s_{p-1} - cp s_p
  relv(g, 1, p, j) = cp;
  relv(g, 2, p, j) = vp;
  relv(g, 3, p, j) = al;  // x_first = al - be s_{p-1} - ga s_p
  relv(g, 4, p, j) = be;
  relv(g, 5, p, j) = ga;
}

// ---- the separators' system ----------------------------------------------
// A block holds 32 systems (lane = system) and 8 warps: the warps first form
// the separator rows of the 32 systems in parallel (warp w forms rows w,
// w + 8, ...; each row reads four inputs and the end relations of the two
// partitions beside it, independent of the others) into shared memory, then
// warp 0 runs Thomas over them, one thread per system, and writes the
// separators.  Dynamic shared memory: 4 (P - 1) 32 values.

constexpr int IPT_SEP_WARPS = 8;

template <typename T>
__global__ void __launch_bounds__(32 * IPT_SEP_WARPS) ipt_separator_kernel(const Ipt<T> g) {
  extern __shared__ __align__(16) unsigned char ipt_sep_smem[];
  const int S = g.P - 1;
  T* sA = reinterpret_cast<T*>(ipt_sep_smem);
  T* sB = sA + (size_t)S * 32;
  T* sC = sB + (size_t)S * 32;
  T* sD = sC + (size_t)S * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  const bool live = j < g.batch;
  for (int q = w; q < S; q += IPT_SEP_WARPS) {
    T A = T(0), B = T(1), C = T(0), D = T(0);
    if (live) {
      const int R = (q + 1) * g.L - 1;
      const size_t o = at(g, R, j);
      const T aR = ld_stream(g.a + o), cR = ld_stream(g.c + o);
      B = ld_stream(g.b + o);
      D = ld_stream(g.d + o);
      // x_{R-1}: the last interior row of partition q
      B = fma(-aR, relv(g, 1, q, j), B);
      D = fma(-aR, relv(g, 0, q, j), D);
      if (q > 0) A = -aR * relv(g, 2, q, j);
      // x_{R+1}: the first interior row of partition q + 1
      if (q + 1 == g.P - 1) {
        B = fma(-cR, relv(g, 1, q + 1, j), B);
        D = fma(-cR, relv(g, 0, q + 1, j), D);
      } else {
        B = fma(-cR, relv(g, 4, q + 1, j), B);
        D = fma(-cR, relv(g, 3, q + 1, j), D);
        C = -cR * relv(g, 5, q + 1, j);
      }
    }
    sA[q * 32 + lane] = A;
    sB[q * 32 + lane] = B;
    sC[q * 32 + lane] = C;
    sD[q * 32 + lane] = D;
  }
  __syncthreads();
  if (w != 0 || !live) return;
  T* sd = g.sys + (size_t)g.P * g.batch;
  T cprev = T(0), dprev = T(0);
  for (int q = 0; q < S; ++q) {
    const T A = sA[q * 32 + lane];
    const T r = rcp(fma(-A, cprev, sB[q * 32 + lane]));
    cprev = sC[q * 32 + lane] * r;
    dprev = fma(-A, dprev, sD[q * 32 + lane]) * r;
    sC[q * 32 + lane] = cprev;
    sD[q * 32 + lane] = dprev;
  }
  T s = dprev;
  sd[(size_t)(S - 1) * g.batch + j] = s;
  for (int q = S - 2; q >= 0; --q) {
    s = fma(-sC[q * 32 + lane], s, sD[q * 32 + lane]);
    sd[(size_t)q * g.batch + j] = s;
  }
}

// ---- back substitution ----------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(128) ipt_back_kernel(const Ipt<T> g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (j >= g.batch) return;
  const int lo = p * g.L, hi = min(g.n, lo + g.L);
  const T* sd = g.sys + (size_t)g.P * g.batch;
  if (p == g.P - 1) {
    T xp = sd[(size_t)(p - 1) * g.batch + j];
    T qa[IPT_U], qd[IPT_U];
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) {
      const int i = lo + u;
      if (i < g.n) {
        qa[u] = ld_stream(g.cp + at(g, i, j));
        qd[u] = g.x[at(g, i, j)];
      }
    }
    for (int i0 = lo; i0 < g.n; i0 += IPT_U) {
      T ra[IPT_U], rd[IPT_U];
#pragma unroll
      for (int u = 0; u < IPT_U; ++u) { ra[u] = qa[u]; rd[u] = qd[u]; }
#pragma unroll
      for (int u = 0; u < IPT_U; ++u) {
        const int i = i0 + IPT_U + u;
        if (i < g.n) {
          qa[u] = ld_stream(g.cp + at(g, i, j));
          qd[u] = g.x[at(g, i, j)];
        }
      }
#pragma unroll
      for (int u = 0; u < IPT_U; ++u) {
        const int i = i0 + u;
        if (i < g.n) {
          xp = fma(-ra[u], xp, rd[u]);
          st_stream(g.x + at(g, i, j), xp);
        }
      }
    }
    return;
  }
  const T so = sd[(size_t)p * g.batch + j];
  const T sp = p > 0 ? sd[(size_t)(p - 1) * g.batch + j] : T(0);
  st_stream(g.x + at(g, hi - 1, j), so);
  T xn = so;
  const bool first = p == 0;
  T qc[IPT_U], qd[IPT_U], qv[IPT_U];
#pragma unroll
  for (int u = 0; u < IPT_U; ++u) {
    const int i = hi - 2 - u;
    if (i >= lo) {
      const size_t o = at(g, i, j);
      qc[u] = ld_stream(g.cp + o);
      qd[u] = g.x[o];
      qv[u] = first ? T(0) : ld_stream(g.vp + o);
    }
  }
  for (int i0 = hi - 2; i0 >= lo; i0 -= IPT_U) {
    T rc[IPT_U], rd[IPT_U], rv[IPT_U];
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) { rc[u] = qc[u]; rd[u] = qd[u]; rv[u] = qv[u]; }
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) {
      const int i = i0 - IPT_U - u;
      if (i >= lo) {
        const size_t o = at(g, i, j);
        qc[u] = ld_stream(g.cp + o);
        qd[u] = g.x[o];
        qv[u] = first ? T(0) : ld_stream(g.vp + o);
      }
    }
#pragma unroll
    for (int u = 0; u < IPT_U; ++u) {
      const int i = i0 - u;
      if (i >= lo) {
        const T r = first ? rd[u] : fma(-rv[u], sp, rd[u]);
        xn = fma(-rc[u], xn, r);
        st_stream(g.x + at(g, i, j), xn);
      }
    }
  }
}

inline size_t ipt_align(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

// Partitions per system: about four warps per SM sub-partition over the
// batch, each partition at least IPT_MIN_ROWS rows, at most 64 partitions.
constexpr int IPT_MIN_ROWS = 32;

int ipt_partitions(int n, int batch) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long groups = (batch + 31) / 32;
  long long P = (4LL * 4 * sms + groups / 2) / std::max(1LL, groups);
  P = std::min<long long>(P, n / IPT_MIN_ROWS);
  P = std::min<long long>(P, 64);
  if (P < 2) return 0;
  // the last partition must not be empty
  const int L = (int)((n + P - 1) / P);
  return (int)((n + L - 1) / L);
}

template <typename T>
size_t ipt_workspace_bytes(int n, int batch) {
  const size_t e = (size_t)n * (size_t)batch * sizeof(T);
  return 2 * ipt_align(e) + ipt_align((size_t)6 * 64 * batch * sizeof(T)) +
         ipt_align((size_t)2 * 64 * batch * sizeof(T));
}

template <typename T>
cudaError_t launch_ipt(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch, void* work,
                       size_t work_bytes, cudaStream_t s, bool* used) {
  *used = false;
  const int P = ipt_partitions(n, batch);
  if (P < 3 || !work || work_bytes < ipt_workspace_bytes<T>(n, batch)) return cudaSuccess;
  Ipt<T> g;
  g.a = a;
  g.b = b;
  g.c = c;
  g.d = d;
  g.x = x;
  char* w = static_cast<char*>(work);
  const size_t e = ipt_align((size_t)n * (size_t)batch * sizeof(T));
  g.cp = reinterpret_cast<T*>(w);
  g.vp = reinterpret_cast<T*>(w + e);
  g.rel = reinterpret_cast<T*>(w + 2 * e);
  g.sys = reinterpret_cast<T*>(w + 2 * e + ipt_align((size_t)6 * 64 * batch * sizeof(T)));
  g.n = n;
  g.batch = batch;
  g.P = P;
  g.L = (n + P - 1) / P;
  const dim3 grid((batch + 127) / 128, P);
  ipt_forward_kernel<T><<<grid, 128, 0, s>>>(g);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const size_t sep_smem = (size_t)4 * (P - 1) * 32 * sizeof(T);
  err = cudaFuncSetAttribute(ipt_separator_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sep_smem);
  if (err != cudaSuccess) return err;
  ipt_separator_kernel<T><<<(batch + 31) / 32, 32 * IPT_SEP_WARPS, sep_smem, s>>>(g);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  ipt_back_kernel<T><<<grid, 128, 0, s>>>(g);
  err = cudaGetLastError();
  if (err == cudaSuccess) *used = true;
  return err;
}

#define INST(T)                                                                                                \
  template size_t ipt_workspace_bytes<T>(int, int);                                                             \
  template cudaError_t launch_ipt<T>(const T*, const T*, const T*, const T*, T*, int, int, void*, size_t,       \
                                     cudaStream_t, bool*);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
