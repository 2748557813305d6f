// Partitioned solve with partial pivoting inside partitions, one thread per
// (system, partition), for contiguous (layout 0) and batch-interleaved
// (layout 2) batches; x may alias d.
//
// The one-CTA-per-system partitioned solve (pge.cu) cuts each system into
// 128 partitions of 32 rows: its separators' system costs ~2.4 FP64
// instructions per row and every partition but none carries the first-row
// relation (5 FP64 instructions per row).  Here each system is cut into P
// partitions of L rows (L a multiple of 32, P chosen for about four warps
// per SM sub-partition over the batch): thread (j, p) owns partition p of
// system j and a warp holds 32 adjacent systems at one partition index.
//   * p = 0 eliminates top-down with partial pivoting (LAPACK ?gtsv's
//     elimination: 7 FP64 instructions per row), leaving its last interior
//     row in terms of the separator s_0;
//   * p = P-1 eliminates bottom-up (the same elimination on the reversed
//     rows), leaving its first row in terms of s_{P-2};
//   * interior partitions eliminate top-down carrying the left spike (a of
//     their first row times s_{p-1}) and the right spike (c of their last
//     interior row times s_p), and the first row of U^{-1} (the omega
//     recurrence omega_i u0_i + omega_{i-1} u1_{i-1} + omega_{i-2} u2_{i-2}
//     = [i = 0]) applied to the eliminated right-hand sides: 12 FP64
//     instructions per row.  They leave their first and last interior rows
//     in terms of s_{p-1} and s_p.
// U rows go to the workspace batch-interleaved (row i of system j at
// i batch + j), so a warp's factor stores and loads are coalesced lines;
// the swap bit of each U row goes to a bit word per 32 rows (L is a multiple
// of 32, so no two partitions share a word).  The separators' system (P-1
// rows per system) is formed from the relations in parallel and solved with
// partial pivoting by one thread per system; the back substitution then
// solves every interior row for its true right-hand side with the
// separators in place (backward stable with partial pivoting).
//
// Acceptance (the one-CTA solve's test): every separator row's residual,
// formed with the back-substituted neighbours, must meet SEP_TOL relative to
// max|A| max|x| + max|d| of its system; a system that misses it (or broke
// down in a partition, or produced a non-finite value) is appended to a
// device list that the one-CTA partitioned solve then drains by ticket from
// the original right-hand side (solving in place, from a copy of it that the
// forward sweep writes while it reads d).
//
// Reference: the pivoting row of the benchmark, MKL ?gtsv
// (Tridiagonal_AVX512/tridiagonal_basic.cpp:131-143), and the partitioned
// GE of WM-pGE (Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:17-884).
#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

namespace {

__device__ __forceinline__ bool ppt_finite(double v) { return ((bits_of(v) >> 52) & 0x7ffull) != 0x7ffull; }
__device__ __forceinline__ bool ppt_finite(float v) { return ((bits_of(v) >> 23) & 0xffu) != 0xffu; }
// magnitude key in 32 bits (FP64: the high word; orders |v| within 2^-20)
__device__ __forceinline__ unsigned ppt_mag(double v) { return (unsigned)(bits_of(v) >> 32) & 0x7fffffffu; }
__device__ __forceinline__ unsigned ppt_mag(float v) { return bits_of(v) & 0x7fffffffu; }
__device__ __forceinline__ double ppt_from_mag(unsigned m, double) { return __longlong_as_double((long long)m << 32); }
__device__ __forceinline__ float ppt_from_mag(unsigned m, float) { return __int_as_float((int)m); }
constexpr unsigned PPT_BAD = 0x7ff80000u;  // a NaN key: a breakdown fails the test

template <typename T>
struct PptTol;
template <>
struct PptTol<double> {
  static constexpr double SEP = 2.5e-13;  // the one-CTA solve's SEP_TOL
};
template <>
struct PptTol<float> {
  static constexpr double SEP = 5e-7;
};

// relation slots per (partition, system)
enum { R_Y0, R_V0, R_W0, R_YL, R_VL, R_WL, R_CW, R_WP, R_AMAX, R_DMAX, R_XMAX, PPT_REL };

template <typename T>
struct Ppt {
  const T* a;
  const T* b;
  const T* c;
  const T* din;  // right-hand sides
  T* x;          // the solution (may be din)
  T* fi;       // [n][batch] 1/u0 of each U row
  T* fu;       // [n][batch] u1
  T* fz;       // [n][batch] z: u2 (swapped row) or the left spike's v' (else)
  T* fy;       // [n][batch] y'
  T* dcopy;    // [batch][n] the right-hand sides as given (in place only; for the fallback)
  unsigned* sw;  // [n / 32][batch] swap bits
  T* rel;      // [PPT_REL][P][batch]
  T* sep;      // [P][batch] separators
  int* info;
  int* list;   // systems for the fallback, count in cnt[0]
  int* cnt;    // [0] fallback count, [1] fallback ticket
  int* flag;   // [batch] (interleaved) systems for the fallback
  int n, batch, P, L;
  bool inter;  // layout 2: row i of system j at i batch + j (else j n + i)
};

template <typename T>
__device__ __forceinline__ T& relv(const Ppt<T>& g, int k, int p, int j) {
  return g.rel[((size_t)k * g.P + p) * g.batch + j];
}
// element (row i, system j) of a, b, c, d, x
template <typename T>
__device__ __forceinline__ size_t ix(const Ppt<T>& g, int i, int j) {
  return g.inter ? (size_t)i * (size_t)g.batch + (size_t)j : (size_t)j * (size_t)g.n + (size_t)i;
}
template <typename T>
__device__ __forceinline__ size_t fat(const Ppt<T>& g, int i, int j) {
  return (size_t)i * (size_t)g.batch + (size_t)j;
}

constexpr int PPT_U = 4;   // rows loaded ahead of the elimination
constexpr int PPT_UB = 6;  // rows loaded ahead of the back substitution (118 registers: four CTAs per SM)

// Rows of partition p: interior [lo, lo + mi), swept top-down (dir +1, row
// lo + k at step k) or, for the last partition, bottom-up (row lo + mi - 1 - k).
__device__ __forceinline__ void ppt_geom(int n, int L, int P, int p, int& lo, int& mi, int& dir) {
  lo = p * L;
  dir = p == P - 1 ? -1 : 1;
  mi = p == P - 1 ? n - lo : L - 1;
}

// ---- forward sweeps --------------------------------------------------------
// INTERIOR: the left spike and the first row's relation are carried.  The
// elimination is the one-CTA solve's (pge.cu), row by row: U row k is
// (1/u0, u1, z, y') with swap bit k; the candidate row is (cb, cc, cy, cv,
// cw) -- its b, c, y', left-spike and right-spike coefficients.
template <typename T, bool INTERIOR>
__device__ __forceinline__ void ppt_sweep(const Ppt<T>& g, int j, int p) {
  int lo, mi, dir;
  ppt_geom(g.n, g.L, g.P, p, lo, mi, dir);
  auto row = [&](int k) { return dir > 0 ? lo + k : lo + mi - 1 - k; };
  // swept row k as (na: toward the eliminated side, nb, cn: toward the
  // rows ahead, ny); the outer coefficient of the first row is the left
  // spike (interior partitions) or absent (a_0, c_{n-1}: not read)
  T qa[PPT_U], qb[PPT_U], qc[PPT_U], qy[PPT_U];
  auto load = [&](int k, int u) {
    if (k < mi) {
      const int i = row(k);
      const T av = (dir > 0 ? k > 0 || INTERIOR : k + 1 < mi || i > 0) ? __ldg(g.a + ix(g, i, j)) : T(0);
      const T cval = (dir > 0 ? k + 1 < mi || i + 1 < g.n : k > 0) ? __ldg(g.c + ix(g, i, j)) : T(0);
      const T dv = __ldg(g.din + ix(g, i, j));
      if (g.dcopy) g.dcopy[ix(g, i, j)] = dv;
      qa[u] = dir > 0 ? av : cval;
      qc[u] = dir > 0 ? cval : av;
      qb[u] = __ldg(g.b + ix(g, i, j));
      qy[u] = dv;
    }
  };
#pragma unroll
  for (int u = 0; u < PPT_U; ++u) load(u, u);
  bool bad = false;
  unsigned amax = 0, dmax = 0, bits = 0;
  T cb, cc, cy, cv, cw, w_prev = T(0);
  T om1 = T(0), om2 = T(0), kro = T(1), pu1 = T(0), pu2a = T(0), pu2b = T(0), Y0 = T(0), V0 = T(0);
  {
    const T a0 = qa[0], b0 = qb[0], c0 = qc[0], d0 = qy[0];
    cb = b0;
    cc = mi > 1 ? c0 : T(0);
    cy = d0;
    cv = INTERIOR ? a0 : T(0);
    cw = mi == 1 ? c0 : T(0);
    amax = max(ppt_mag(a0), max(ppt_mag(b0), ppt_mag(c0)));
    dmax = ppt_mag(d0);
  }
  auto put = [&](int k, T inv, T u1, T z, T y, bool s) {
    const int i = row(k);
    const size_t o = fat(g, i, j);
    st_stream(g.fi + o, inv);
    st_stream(g.fu + o, u1);
    st_stream(g.fz + o, z);
    st_stream(g.fy + o, y);
    bits |= (unsigned)s << (i & 31);
    if ((i & 31) == (dir > 0 ? 31 : 0) || k + 1 == mi) {
      g.sw[fat(g, i >> 5, j)] = bits;
      bits = 0;
    }
  };
  // swept row k+1 (na, nb, cn, ny) against the candidate row: U row k.
  // `last` (row k+1 is the last swept row) only selects: the far spike's
  // product is formed once, after the loop, from the values kept here.
  T l_far = T(0), cn_far = T(0);
  bool s_far = false;
  auto eliminate = [&](int k, T na, T nb, T cn, T ny, bool last) {
    amax = max(amax, max(ppt_mag(na), max(ppt_mag(nb), ppt_mag(cn))));
    dmax = max(dmax, ppt_mag(ny));
    const T nc = last ? T(0) : cn;
    const bool s = !abs_ge(cb, na);
    const T piv = s ? na : cb;
    bad |= is_zero(piv);
    const T inv = Div<T>(piv).inv();
    const T l = (s ? cb : na) * inv;
    const T u1 = s ? nb : cc;
    const T uy = s ? ny : cy;
    const T zs = s ? nc : cv;  // the nonzero one of u2 and v'
    if constexpr (INTERIOR) {
      const T u2 = keep_if(s, nc);
      const T uv = keep_if(!s, cv);
      const T om = fma(-om2, pu2b, fma(-om1, pu1, kro)) * inv;
      kro = T(0);
      Y0 = fma(om, uy, Y0);
      V0 = fma(om, uv, V0);
      om2 = om1;
      om1 = om;
      pu2b = pu2a;
      pu2a = u2;
      pu1 = u1;
    }
    put(k, inv, u1, zs, uy, s);
    cb = fma(-l, u1, s ? cc : nb);
    const T tq = -l * zs;
    cc = s ? tq : nc;
    cy = fma(-l, uy, s ? cy : ny);
    if constexpr (INTERIOR) cv = s ? cv : tq;
    l_far = last ? l : l_far;
    cn_far = last ? cn : cn_far;
    s_far = last ? s : s_far;
  };
  // rows 1 .. mi-1 in groups of PPT_U, the next group loading meanwhile
  for (int k0 = 0; k0 + 1 < mi; k0 += PPT_U) {
    T ra[PPT_U], rb[PPT_U], rc[PPT_U], ry[PPT_U];
#pragma unroll
    for (int u = 0; u < PPT_U; ++u) {
      ra[u] = qa[u];
      rb[u] = qb[u];
      rc[u] = qc[u];
      ry[u] = qy[u];
    }
#pragma unroll
    for (int u = 0; u < PPT_U; ++u) load(k0 + PPT_U + u, u);
    // row k0 + u (u >= 1, or the next group's first) is eliminated against U row k0 + u - 1
#pragma unroll
    for (int u = 1; u <= PPT_U; ++u) {
      const int kk = k0 + u;  // the swept row entering
      if (kk >= mi) break;
      const T na = u < PPT_U ? ra[u] : qa[0], nb = u < PPT_U ? rb[u] : qb[0];
      const T cn = u < PPT_U ? rc[u] : qc[0], ny = u < PPT_U ? ry[u] : qy[0];
      eliminate(kk - 1, na, nb, cn, ny, kk + 1 == mi);
    }
  }
  if (mi >= 2) {  // the far spike enters with the last swept row
    w_prev = s_far ? cn_far : cw;
    cw = fma(-l_far, w_prev, s_far ? cw : cn_far);
  }
  // U row mi-1 is the remaining candidate row (u1 = u2 = 0)
  bad |= is_zero(cb);
  const T inv_last = Div<T>(cb).inv();
  if constexpr (INTERIOR) {
    const T om = fma(-om2, pu2b, fma(-om1, pu1, kro)) * inv_last;
    Y0 = fma(om, cy, Y0);
    V0 = fma(om, cv, V0);
    relv(g, R_Y0, p, j) = Y0;
    relv(g, R_V0, p, j) = V0;
    relv(g, R_W0, p, j) = fma(om1, w_prev, om * cw);
  }
  put(mi - 1, inv_last, T(0), cv, cy, false);
  relv(g, R_YL, p, j) = cy * inv_last;
  relv(g, R_VL, p, j) = cv * inv_last;
  relv(g, R_WL, p, j) = cw * inv_last;
  relv(g, R_CW, p, j) = cw;
  relv(g, R_WP, p, j) = w_prev;
  relv(g, R_AMAX, p, j) = ppt_from_mag(bad ? PPT_BAD : amax, T(0));
  relv(g, R_DMAX, p, j) = ppt_from_mag(dmax, T(0));
}

template <typename T>
__global__ void __launch_bounds__(128) ppt_forward_kernel(const Ppt<T> g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (j >= g.batch) return;
  if (p == 0 || p == g.P - 1)
    ppt_sweep<T, false>(g, j, p);
  else
    ppt_sweep<T, true>(g, j, p);
}

// ---- the separators' system -------------------------------------------------
// 32 systems (lane = system) and 16 warps per block: the warps form the
// separator rows in parallel into shared memory, then warp 0 solves each
// system's P-1 rows with partial pivoting (LAPACK ?gtsv's algorithm) and
// writes the separators.  Dynamic shared memory: 4 (P - 1) 32 values.
constexpr int PPT_SEP_WARPS = 16;

template <typename T>
__global__ void __launch_bounds__(32 * PPT_SEP_WARPS) ppt_separator_kernel(const Ppt<T> g) {
  extern __shared__ __align__(16) unsigned char ppt_sep_smem[];
  const int S = g.P - 1;
  T* sA = reinterpret_cast<T*>(ppt_sep_smem);
  T* sB = sA + (size_t)S * 32;
  T* sC = sB + (size_t)S * 32;
  T* sD = sC + (size_t)S * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  const bool live = j < g.batch;
  for (int q = w; q < S; q += PPT_SEP_WARPS) {
    T A = T(0), B = T(1), C = T(0), D = T(0);
    if (live) {
      const size_t o = ix(g, (q + 1) * g.L - 1, j);
      const T aR = __ldg(g.a + o), cR = __ldg(g.c + o);
      B = __ldg(g.b + o);
      D = __ldg(g.din + o);
      if (g.dcopy) g.dcopy[o] = D;  // (the forward sweeps copied the interior rows)
      // x of the row above: the last interior row of partition q
      B = fma(-aR, relv(g, R_WL, q, j), B);
      D = fma(-aR, relv(g, R_YL, q, j), D);
      if (q > 0) A = -aR * relv(g, R_VL, q, j);
      // x of the row below: the first interior row of partition q + 1
      if (q + 1 == g.P - 1) {  // (bottom-up: its last swept row)
        B = fma(-cR, relv(g, R_WL, q + 1, j), B);
        D = fma(-cR, relv(g, R_YL, q + 1, j), D);
      } else {
        B = fma(-cR, relv(g, R_V0, q + 1, j), B);
        D = fma(-cR, relv(g, R_Y0, q + 1, j), D);
        C = -cR * relv(g, R_W0, q + 1, j);
      }
    }
    sA[q * 32 + lane] = A;
    sB[q * 32 + lane] = B;
    sC[q * 32 + lane] = C;
    sD[q * 32 + lane] = D;
  }
  __syncthreads();
  if (w != 0 || !live) return;
  // partial pivoting: U row q (1/u0 -> sA, u1 -> sB, u2 -> sC, y' -> sD)
  T cb = sB[lane], cc = S > 1 ? sC[lane] : T(0), cy = sD[lane];
  bool bad = false;
  for (int q = 0; q + 1 < S; ++q) {
    const int o = (q + 1) * 32 + lane;
    const T na = sA[o], nb = sB[o], nc = q + 2 < S ? sC[o] : T(0), ny = sD[o];
    const bool s = !abs_ge(cb, na);
    const T piv = s ? na : cb;
    bad |= is_zero(piv);
    const T inv = Div<T>(piv).inv();
    const T l = (s ? cb : na) * inv;
    const T u1 = s ? nb : cc;
    const T uy = s ? ny : cy;
    sA[q * 32 + lane] = inv;
    sB[q * 32 + lane] = u1;
    sC[q * 32 + lane] = keep_if(s, nc);
    sD[q * 32 + lane] = uy;
    cb = fma(-l, u1, s ? cc : nb);
    cc = s ? -l * nc : nc;
    cy = fma(-l, uy, s ? cy : ny);
  }
  bad |= is_zero(cb);
  T x1 = cy * Div<T>(cb).inv(), x2 = T(0);
  T* sp = g.sep;
  sp[(size_t)(S - 1) * g.batch + j] = x1;
  for (int q = S - 2; q >= 0; --q) {
    const T xq = fma(-sC[q * 32 + lane], x2, fma(-sB[q * 32 + lane], x1, sD[q * 32 + lane])) * sA[q * 32 + lane];
    sp[(size_t)q * g.batch + j] = xq;
    x2 = x1;
    x1 = xq;
  }
  if (bad) relv(g, R_AMAX, 0, j) = ppt_from_mag(PPT_BAD, T(0));
}

// ---- back substitution ----------------------------------------------------
template <typename T, bool INTERIOR>
__device__ __forceinline__ void ppt_back(const Ppt<T>& g, int j, int p) {
  int lo, mi, dir;
  ppt_geom(g.n, g.L, g.P, p, lo, mi, dir);
  auto row = [&](int k) { return dir > 0 ? lo + k : lo + mi - 1 - k; };
  // separators on the near (left spike) and far side of the sweep
  const T s_near = INTERIOR ? g.sep[(size_t)(p - 1) * g.batch + j] : T(0);
  const T s_far = g.sep[(size_t)(dir > 0 ? p : p - 1) * g.batch + j];
  const T cw = relv(g, R_CW, p, j), w_prev = relv(g, R_WP, p, j);
  unsigned xmax = ppt_mag(s_far);
  bool bad = false;
  // U row k as (1/u0, u1, z, y', swap bit), loaded PPT_UB rows ahead (the
  // grid, not the registers, limits the warps per SM: more rows in flight
  // per thread is what hides the loads)
  T qi[PPT_UB], qu[PPT_UB], qz[PPT_UB], qy[PPT_UB];
  unsigned qs[PPT_UB];
  auto load = [&](int k, int u) {
    if (k >= 0) {
      const int i = row(k);
      const size_t o = fat(g, i, j);
      qi[u] = ld_stream(g.fi + o);
      qu[u] = ld_stream(g.fu + o);
      qz[u] = ld_stream(g.fz + o);
      qy[u] = ld_stream(g.fy + o);
      qs[u] = (g.sw[fat(g, i >> 5, j)] >> (i & 31)) & 1u;
    }
  };
#pragma unroll
  for (int u = 0; u < PPT_UB; ++u) load(mi - 1 - u, u);
  T x1 = fma(-cw, s_far, fma(-qz[0], s_near, qy[0])) * qi[0], x2 = T(0);
  if (mi >= 2) qy[1] = fma(-w_prev, s_far, qy[1]);  // row mi-2's far-spike term
  g.x[ix(g, row(mi - 1), j)] = x1;
  xmax = max(xmax, ppt_mag(x1));
  bad |= !ppt_finite(x1);
  for (int k0 = mi - 1; k0 > 0; k0 -= PPT_UB) {
    T ri[PPT_UB], ru[PPT_UB], rz[PPT_UB], ry[PPT_UB];
    unsigned rs[PPT_UB];
#pragma unroll
    for (int u = 0; u < PPT_UB; ++u) {
      ri[u] = qi[u];
      ru[u] = qu[u];
      rz[u] = qz[u];
      ry[u] = qy[u];
      rs[u] = qs[u];
    }
#pragma unroll
    for (int u = 0; u < PPT_UB; ++u) load(k0 - PPT_UB - u, u);
    // U row k0 - u (u >= 1) from this group, the next group's first for u = PPT_UB
#pragma unroll
    for (int u = 1; u <= PPT_UB; ++u) {
      const int k = k0 - u;
      if (k < 0) break;
      const T zi = u < PPT_UB ? rz[u] : qz[0], yi = u < PPT_UB ? ry[u] : qy[0];
      const T ui = u < PPT_UB ? ru[u] : qu[0], ii = u < PPT_UB ? ri[u] : qi[0];
      const unsigned si = u < PPT_UB ? rs[u] : qs[0];
      // z multiplies x two rows on (swap) or the near separator (no swap)
      const T zx = si ? x2 : s_near;
      const T xi = fma(-ui, x1, fma(-zi, zx, yi)) * ii;
      g.x[ix(g, row(k), j)] = xi;
      xmax = max(xmax, ppt_mag(xi));
      bad |= !ppt_finite(xi);
      x2 = x1;
      x1 = xi;
    }
  }
  relv(g, R_XMAX, p, j) = ppt_from_mag(bad ? PPT_BAD : xmax, T(0));
}

template <typename T>
__global__ void __launch_bounds__(128, 4) ppt_back_kernel(const Ppt<T> g) {  // (four CTAs per SM: the grid's)
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (j >= g.batch) return;
  if (p == 0 || p == g.P - 1)
    ppt_back<T, false>(g, j, p);
  else
    ppt_back<T, true>(g, j, p);
}

// ---- acceptance -------------------------------------------------------------
// The separator rows' residuals with the back-substituted neighbours
// against SEP_TOL (max|A| max|x| + max|d|) of their system; accepted systems
// get their separators written and info 0, the others are listed for the
// one-CTA solve.  32 systems (lane = system) and 16 warps per block: the
// warps reduce the partitions' maxima, then form the residuals, in
// parallel.  Counted (per warp) in g_ppt_counts.
__device__ unsigned long long g_ppt_counts[2];
constexpr int PPT_CHECK_WARPS = 16;

template <typename T>
__global__ void __launch_bounds__(32 * PPT_CHECK_WARPS) ppt_check_kernel(const Ppt<T> g) {
  constexpr unsigned NONFINITE = sizeof(T) == 8 ? 0x7ff00000u : 0x7f800000u;  // keys of Inf / NaN (and PPT_BAD)
  __shared__ unsigned s_m[3][PPT_CHECK_WARPS][32];
  __shared__ int s_bad[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  const bool live = j < g.batch;
  unsigned am = 0, dm = 0, xm = 0;
  for (int p = w; p < g.P && live; p += PPT_CHECK_WARPS) {
    am = max(am, ppt_mag(relv(g, R_AMAX, p, j)));
    dm = max(dm, ppt_mag(relv(g, R_DMAX, p, j)));
    xm = max(xm, ppt_mag(relv(g, R_XMAX, p, j)));
  }
  s_m[0][w][lane] = am;
  s_m[1][w][lane] = dm;
  s_m[2][w][lane] = xm;
  if (w == 0) s_bad[lane] = 0;
  __syncthreads();
#pragma unroll
  for (int v = 0; v < PPT_CHECK_WARPS; ++v) {
    am = max(am, s_m[0][v][lane]);
    dm = max(dm, s_m[1][v][lane]);
    xm = max(xm, s_m[2][v][lane]);
  }
  bool bad = am >= NONFINITE || xm >= NONFINITE;
  const double bound =
      PptTol<T>::SEP * fma((double)ppt_from_mag(am, T(0)), (double)ppt_from_mag(xm, T(0)), (double)ppt_from_mag(dm, T(0)));
  bool rb = false;
  for (int q = w; q + 1 < g.P && live && !bad; q += PPT_CHECK_WARPS) {
    const int R = (q + 1) * g.L - 1;
    const size_t o = ix(g, R, j);
    const T s = g.sep[(size_t)q * g.batch + j];
    const double r = fma(-(double)g.c[o], (double)g.x[ix(g, R + 1, j)],
                         fma(-(double)g.b[o], (double)s,
                             fma(-(double)g.a[o], (double)g.x[ix(g, R - 1, j)], (double)g.din[o])));
    rb |= !(fabs(r) <= bound) || !ppt_finite(s);
  }
  if (rb) s_bad[lane] = 1;
  __syncthreads();  // (every read of d's separator rows is done: x may alias d)
  bad = bad || s_bad[lane] != 0;
  if (w == 0) {
    const unsigned acc = __ballot_sync(0xffffffffu, live && !bad), rej = __ballot_sync(0xffffffffu, live && bad);
    if (lane == 0) {
      if (acc) atomicAdd(&g_ppt_counts[0], (unsigned long long)__popc(acc));
      if (rej) atomicAdd(&g_ppt_counts[1], (unsigned long long)__popc(rej));
    }
    if (live && bad) {
      if (g.inter)
        g.flag[j] = 1;
      else
        g.list[atomicAdd(g.cnt, 1)] = j;
    }
    if (live && !bad && g.info) g.info[j] = 0;
  }
  for (int q = w; q + 1 < g.P && live && !bad; q += PPT_CHECK_WARPS)
    g.x[ix(g, (q + 1) * g.L - 1, j)] = g.sep[(size_t)q * g.batch + j];
  // (interleaved) a listed system's x restarts from its right-hand side: the
  // masked sequential solve works in place on x
  if (g.inter && live && bad) {
    const T* src = g.dcopy ? g.dcopy : g.din;
    for (int i = w; i < g.n; i += PPT_CHECK_WARPS) g.x[ix(g, i, j)] = src[ix(g, i, j)];
  }
}

inline size_t ppt_align(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

// Partitions per system: about four warps per SM sub-partition over the
// batch, L = ceil(n / P) rounded up to a multiple of 32, at most PPT_MAX_P.
constexpr int PPT_MAX_P = 64;

// SM count of the current device, looked up once per device (and once when
// there is none: workspace-size queries run on machines without a GPU too).
static int ppt_sms() {
  static std::atomic<int> cache[65];
  int dev = 0;
  const bool have = cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64;
  std::atomic<int>& slot = cache[have ? dev : 64];
  int v = slot.load(std::memory_order_relaxed);
  if (v > 0) return v;
  v = 152;
  if (have && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) v = 152;
  if (v <= 0) v = 152;
  slot.store(v, std::memory_order_relaxed);
  return v;
}

int ppt_rows(int n, int batch) {
  const int sms = ppt_sms();
  const long long groups = (batch + 31) / 32;
  long long P = (4LL * 4 * sms + groups / 2) / std::max(1LL, groups);
  P = std::min<long long>(std::max<long long>(P, 3), PPT_MAX_P);
  const long long L = ((n + P - 1) / P + 31) / 32 * 32;
  if (L < 64 || (n + L - 1) / L < 3) return 0;
  return (int)L;
}

// Covered: FP64 systems longer than one CTA's shared memory holds (where the
// partitioned solve would take clusters of CTAs: measured on GB300 at 6144 /
// 8192 / 11000 rows x 1536-4096 systems, 1.7-2.4x faster than the clusters;
// at 4096 rows the persistent one-CTA solve is as fast in one launch instead
// of five) up to the clusters' reach, in batches whose partitions fill the
// GPU with at most PPT_MAX_P of them.
// Interleaved batches (where the one-CTA solve does not apply and the
// alternative is a thread per system): from 1024 rows, the same bounds
// otherwise; their listed systems take the masked sequential solve.
bool ppt_eligible(int layout, int n, int batch) {
  if (batch < 1024 || ppt_rows(n, batch) == 0) return false;
  const int one_cta = std::max(pge_variant_max_n<double>(2), pge_variant_max_n<double>(3));
  // (the longest system the listed systems' solve reaches: clusters of 8 CTAs, 27648 FP64 rows)
  if (layout == 2) return n >= 1024 && n <= pge_variant_max_n<double>(6);
  return layout == 0 && n > one_cta && n <= pge_variant_max_n<double>(6);
}

template <typename T>
size_t ppt_workspace_bytes(int n, int batch) {
  const size_t e = ppt_align((size_t)n * (size_t)batch * sizeof(T));
  return 5 * e + ppt_align(pivot_words(n, batch) * sizeof(unsigned)) +
         ppt_align((size_t)PPT_REL * PPT_MAX_P * batch * sizeof(T)) +
         ppt_align((size_t)PPT_MAX_P * batch * sizeof(T)) + 2 * ppt_align((size_t)batch * sizeof(int)) + 256;
}

template <typename T>
cudaError_t launch_ppt(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                       void* work, size_t work_bytes, cudaStream_t s, bool* used) {
  *used = false;
  if (!ppt_eligible(layout, n, batch) || !work || work_bytes < ppt_workspace_bytes<T>(n, batch)) return cudaSuccess;
  const int L = ppt_rows(n, batch);
  Ppt<T> g;
  g.a = a;
  g.b = b;
  g.c = c;
  g.din = d;
  g.x = x;
  char* w = static_cast<char*>(work);
  const size_t e = ppt_align((size_t)n * (size_t)batch * sizeof(T));
  g.fi = reinterpret_cast<T*>(w);
  g.fu = reinterpret_cast<T*>(w + e);
  g.fz = reinterpret_cast<T*>(w + 2 * e);
  g.fy = reinterpret_cast<T*>(w + 3 * e);
  g.dcopy = d == x ? reinterpret_cast<T*>(w + 4 * e) : nullptr;
  w += 5 * e;
  g.sw = reinterpret_cast<unsigned*>(w);
  w += ppt_align(pivot_words(n, batch) * sizeof(unsigned));
  g.rel = reinterpret_cast<T*>(w);
  w += ppt_align((size_t)PPT_REL * PPT_MAX_P * batch * sizeof(T));
  g.sep = reinterpret_cast<T*>(w);
  w += ppt_align((size_t)PPT_MAX_P * batch * sizeof(T));
  g.list = reinterpret_cast<int*>(w);
  w += ppt_align((size_t)batch * sizeof(int));
  g.flag = reinterpret_cast<int*>(w);
  w += ppt_align((size_t)batch * sizeof(int));
  g.cnt = reinterpret_cast<int*>(w);  // (right after flag: one memset clears both)
  g.info = info;
  g.n = n;
  g.batch = batch;
  g.L = L;
  g.P = (n + L - 1) / L;
  g.inter = layout == 2;
  cudaError_t err = cudaMemsetAsync(g.flag, 0, ppt_align((size_t)batch * sizeof(int)) + 2 * sizeof(int), s);
  if (err != cudaSuccess) return err;
  const dim3 grid((batch + 127) / 128, g.P);
  ppt_forward_kernel<T><<<grid, 128, 0, s>>>(g);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const size_t sep_smem = (size_t)4 * (g.P - 1) * 32 * sizeof(T);
  err = cudaFuncSetAttribute(ppt_separator_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sep_smem);
  if (err != cudaSuccess) return err;
  ppt_separator_kernel<T><<<(batch + 31) / 32, 32 * PPT_SEP_WARPS, sep_smem, s>>>(g);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  ppt_back_kernel<T><<<grid, 128, 0, s>>>(g);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  ppt_check_kernel<T><<<(batch + 31) / 32, 32 * PPT_CHECK_WARPS, 0, s>>>(g);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  // the listed systems: the partitioned solve from the (copy of the)
  // right-hand side; interleaved: the masked sequential solve in place on x
  // (restored by the check), the factor arrays as its workspace
  if (g.inter)
    err = launch_gtsv_seq_masked<T>(2, a, b, c, x, g.fi, g.fu, g.sw, info, n, batch, g.flag, s);
  else
    err = launch_pge_list<T>(a, b, c, g.dcopy ? g.dcopy : d, x, info, n, batch, g.list, g.cnt, g.cnt + 1, s);
  if (err == cudaSuccess) *used = true;
  return err;
}

cudaError_t ppt_counts(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_ppt_counts, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess && reset) {
    const unsigned long long z[2] = {0ull, 0ull};
    e = cudaMemcpyToSymbol(g_ppt_counts, z, sizeof(z));
  }
  return e;
}

#define INST(T)                                                                                                \
  template size_t ppt_workspace_bytes<T>(int, int);                                                             \
  template cudaError_t launch_ppt<T>(int, const T*, const T*, const T*, const T*, T*, int*, int, int, void*,      \
                                     size_t, cudaStream_t, bool*);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
