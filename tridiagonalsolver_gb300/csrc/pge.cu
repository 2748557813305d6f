// Partitioned Gaussian elimination with partial pivoting (WM-pGE), one CTA
// per system, the whole system staged in shared memory.
//
// The NT threads of a CTA split the system into NT partitions of m rows;
// in each partition the first m-1 rows are "interior" and the last row is a
// separator.  Thread t eliminates its interior block with partial pivoting
// (the row interchanges of LAPACK ?gtsv) for three right-hand sides at once:
// d, the left spike a_first e_1 (coupling to the previous separator) and the
// right spike c_last e_{m-1} (coupling to its own separator); the first and
// last rows of the block's solution operator applied to them turn each
// separator row into a row of a tridiagonal system in the NT separators,
// solved by parallel cyclic reduction in shared memory (log2 NT steps), or,
// when PCR's result fails a backward-error check, with partial pivoting by
// one warp.  With the separators known, one back substitution per block
// gives the interior unknowns, and x is written back with coalesced stores.
// Systems whose separator rows miss the residual bound and then an exact
// backward-error check (possible when an interior block is nearly singular
// although the whole matrix is not) take a sequential partial-pivoting
// solve by one thread of the CTA, which also produces LAPACK's info value
// for singular matrices.
//
// Parallelism per system is NT chains instead of the one or two chains of a
// Thomas-type sweep, which on GB300 matters most for FP64: the FP64 pipe
// issues one warp instruction per ~70 cycles per SM sub-partition, so the
// sweep needs every sub-partition busy.  Per row the interior work is 13
// FP64 operations forward (elimination and the first row of U^{-1}) and 4
// in the back substitution.
//
// Reference: the partition idea is the reference's WM-pGE
// (Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:17-884, without pivoting there);
// the pivoting is that of its MKL row (Tridiagonal_AVX512/
// tridiagonal_basic.cpp:131-143).
#include <algorithm>
#include <cooperative_groups.h>
#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

__device__ __forceinline__ bool finite_val(double v) { return ((bits_of(v) >> 52) & 0x7ffull) != 0x7ffull; }
__device__ __forceinline__ bool finite_val(float v) { return ((bits_of(v) >> 23) & 0xffu) != 0xffu; }

// Magnitude bits (|v| as an unsigned pattern, ordered like |v|) and the
// biased exponent, on the integer pipe.
__device__ __forceinline__ unsigned long long mag(double v) { return bits_of(v) & 0x7fffffffffffffffull; }
__device__ __forceinline__ unsigned mag(float v) { return bits_of(v) & 0x7fffffffu; }
// Magnitude key in 32 bits (FP64: the high word, which orders |v| up to a
// relative 2^-20 -- enough for the acceptance test's maxima -- and keeps
// the running maxima single 32-bit integer instructions).
__device__ __forceinline__ unsigned magh(double v) { return (unsigned)(bits_of(v) >> 32) & 0x7fffffffu; }
__device__ __forceinline__ unsigned magh(float v) { return mag(v); }
__device__ __forceinline__ int expo(double v) { return (int)((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ff; }
__device__ __forceinline__ int expo(float v) { return (int)((unsigned)__float_as_int(v) >> 23) & 0xff; }
template <typename T>
struct Fmt;
template <>
struct Fmt<double> {
  static constexpr int BIAS = 1023;
  static constexpr double SEP_TOL = 2.5e-13;  // backward error accepted (separator rows, then all rows)
  __device__ static double from_mag(unsigned m) { return __longlong_as_double((long long)m << 32); }
};
template <>
struct Fmt<float> {
  static constexpr int BIAS = 127;
  static constexpr double SEP_TOL = 5e-7;
  __device__ static float from_mag(unsigned m) { return __int_as_float((int)m); }
};

// Sequential partial-pivoting solve (the algorithm of LAPACK ?gtsv) of the
// n-row system in a, b, c, d by one thread, in place: U row i overwrites row
// i (1/u0 -> a, u1 -> b, u2 -> c, y' -> d), x overwrites d.  Returns LAPACK's
// info (0, or k+1 for the first zero pivot; then d is left as y').  a_0 and
// c_{n-1} are not read.
template <typename T>
__device__ int seq_pivoted_inplace(T* a, T* b, T* c, T* d, int n) {
  int info = 0;
  T cb = b[0], cc = n > 1 ? c[0] : T(0), cy = d[0];
  for (int i = 0; i + 1 < n; ++i) {
    const T na = a[i + 1], nb = b[i + 1];
    const T nc = i + 2 < n ? c[i + 1] : T(0);
    const T ny = d[i + 1];
    const bool sw = !abs_ge(cb, na);
    const T piv = sw ? na : cb;
    if (is_zero(piv) && !info) info = i + 1;
    const T inv = Div<T>(piv).inv();
    const T l = (sw ? cb : na) * inv;
    const T u1 = sw ? nb : cc;
    const T uy = sw ? ny : cy;
    a[i] = inv;
    b[i] = u1;
    c[i] = sw ? nc : T(0);
    d[i] = uy;
    cb = fma(-l, u1, sw ? cc : nb);
    cc = fma(-l, sw ? nc : T(0), sw ? T(0) : nc);
    cy = fma(-l, uy, sw ? cy : ny);
  }
  if (is_zero(cb) && !info) info = n;
  if (info) return info;
  T x1 = cy * Div<T>(cb).inv(), x2 = T(0);
  d[n - 1] = x1;
  for (int i = n - 2; i >= 0; --i) {
    const T xi = fma(-c[i], x2, fma(-b[i], x1, d[i])) * a[i];
    d[i] = xi;
    x2 = x1;
    x1 = xi;
  }
  return 0;
}

constexpr int PGE_TMP = 4 * 32;

// In-kernel refinement steps before the sequential fallback.
constexpr int PGE_REFINE = 2;

// Systems that took the sequential fallback since the last reset (per device).
__device__ unsigned long long g_pge_fallbacks = 0ull;
// Per-path counts since the last reset (per device): [0] systems whose PCR
// separator solution was rejected and re-solved with pivoting (first pass),
// [1] systems whose separator rows missed the bound, so that the exact
// backward error was measured, [2] refinement passes run.
__device__ unsigned long long g_pge_paths[3] = {0ull, 0ull, 0ull};

// A chunk of K consecutive rows of a tridiagonal system held in registers:
// rows 0..K-2 are interior, row K-1 is the chunk's top-level row.  The
// interior is eliminated with partial pivoting for three right-hand sides
// (d, the left coupling a_0 e_0, the right coupling c_{K-2} e_{K-2}) and
// fully back-substituted, so that interior row i is
//     x_i = Y_i - V_i s_prev - W_i s_own,
// s_prev being the previous chunk's top row and s_own this chunk's.
template <typename T, int K>
struct ChunkSpikes {
  static constexpr int MI = K - 1;
  T Y[MI], V[MI], W[MI];
  T as, bs, cs, ds;  // the top row

  __device__ bool eliminate(const T (&a_)[K], const T (&b_)[K], const T (&c_)[K], const T (&d_)[K]) {
    bool bad = false;
    T inv[MI], u1[MI], u2[MI], ry[MI], rv[MI];
    T cb = b_[0], cc = MI > 1 ? c_[0] : T(0), cy = d_[0], cv = a_[0], cw = MI == 1 ? c_[0] : T(0);
    T w_prev = T(0);
#pragma unroll
    for (int i = 0; i + 1 < MI; ++i) {
      const T na = a_[i + 1], nb = b_[i + 1], cn = c_[i + 1], ny = d_[i + 1];
      const bool last = i + 2 == MI;
      const T nc = last ? T(0) : cn;
      const bool sw = !abs_ge(cb, na);
      const T piv = sw ? na : cb;
      bad |= is_zero(piv);
      inv[i] = Div<T>(piv).inv();
      const T l = (sw ? cb : na) * inv[i];
      u1[i] = sw ? nb : cc;
      u2[i] = sw ? nc : T(0);
      ry[i] = sw ? ny : cy;
      rv[i] = sw ? T(0) : cv;
      cb = fma(-l, u1[i], sw ? cc : nb);
      cc = fma(-l, sw ? nc : T(0), sw ? T(0) : nc);
      cy = fma(-l, ry[i], sw ? cy : ny);
      cv = sw ? cv : -l * cv;
      if (last) {
        w_prev = sw ? cn : cw;
        cw = fma(-l, w_prev, sw ? cw : cn);
      }
    }
    bad |= is_zero(cb);
    inv[MI - 1] = Div<T>(cb).inv();
    u1[MI - 1] = T(0);
    u2[MI - 1] = T(0);
    ry[MI - 1] = cy;
    rv[MI - 1] = cv;
#pragma unroll
    for (int i = MI - 1; i >= 0; --i) {
      const T y1 = i + 1 < MI ? Y[i + 1] : T(0), v1 = i + 1 < MI ? V[i + 1] : T(0), w1 = i + 1 < MI ? W[i + 1] : T(0);
      const T y2 = i + 2 < MI ? Y[i + 2] : T(0), v2 = i + 2 < MI ? V[i + 2] : T(0), w2 = i + 2 < MI ? W[i + 2] : T(0);
      const T wi = i == MI - 1 ? cw : (i == MI - 2 ? w_prev : T(0));
      Y[i] = fma(-u2[i], y2, fma(-u1[i], y1, ry[i])) * inv[i];
      V[i] = fma(-u2[i], v2, fma(-u1[i], v1, rv[i])) * inv[i];
      W[i] = fma(-u2[i], w2, fma(-u1[i], w1, wi)) * inv[i];
    }
    as = a_[K - 1];
    bs = b_[K - 1];
    cs = c_[K - 1];
    ds = d_[K - 1];
    return bad;
  }
  // The top row in terms of the neighbouring top rows, given the next
  // chunk's first-row values (zero and has_next = false for the last chunk).
  __device__ void top_row(T Yf, T Vf, T Wf, bool has_next, T& ta, T& tb, T& tc, T& td) const {
    const T c = has_next ? cs : T(0);
    ta = -as * V[MI - 1];
    tb = fma(-c, has_next ? Vf : T(0), fma(-as, W[MI - 1], bs));
    tc = -c * (has_next ? Wf : T(0));
    td = fma(-c, has_next ? Yf : T(0), fma(-as, Y[MI - 1], ds));
  }
  __device__ T value(int i, T sp, T st) const { return fma(-W[i], st, fma(-V[i], sp, Y[i])); }
};

// Pivoted solve of the NT-row separator system (rows sa/sb/sc/sd at SEP[0],
// SEP[NT], SEP[2NT], SEP[3NT]) by one warp, solution to sx[0..NT).  Lane l
// takes the K = NT/32 consecutive rows lK .. lK+K-1 as a chunk; the 32
// chunk top rows form a tridiagonal system that lane 0 solves sequentially
// with partial pivoting.  Returns true on breakdown.
template <typename T, int NT>
__device__ bool sep_solve_pivoted(const T* SEP, T* sx, T* tmp, int lane) {
  constexpr int K = NT / 32;
  static_assert(K >= 2, "at least two separators per lane");
  const int r0 = lane * K;
  T a_[K], b_[K], c_[K], d_[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    a_[k] = SEP[r0 + k];
    b_[k] = SEP[NT + r0 + k];
    c_[k] = SEP[2 * NT + r0 + k];
    d_[k] = SEP[3 * NT + r0 + k];
  }
  ChunkSpikes<T, K> ch;
  bool bad = ch.eliminate(a_, b_, c_, d_);
  const T Yf = shfl_down(ch.Y[0], 1), Vf = shfl_down(ch.V[0], 1), Wf = shfl_down(ch.W[0], 1);
  ch.top_row(Yf, Vf, Wf, lane < 31, tmp[lane], tmp[32 + lane], tmp[64 + lane], tmp[96 + lane]);
  __syncwarp();
  int top_bad = 0;
  if (lane == 0) top_bad = seq_pivoted_inplace<T>(tmp, tmp + 32, tmp + 64, tmp + 96, 32);
  bad |= __shfl_sync(FULL, top_bad, 0) != 0;
  __syncwarp();
  const T sp = lane > 0 ? tmp[96 + lane - 1] : T(0);
  const T st = tmp[96 + lane];
#pragma unroll
  for (int i = 0; i < K - 1; ++i) sx[r0 + i] = ch.value(i, sp, st);
  sx[r0 + K - 1] = st;
  return bad;
}

// Arguments of the partitioned kernels.  Systems are uniform (system j at
// j*stride, n rows) or ragged (system s = rows [offsets[s], offsets[s+1]) of
// the packed arrays); `list` maps a CTA (cluster) to its system when a launch
// serves one size bucket of a ragged batch.  MODE 0 writes x; MODE 1 is the
// adjoint: the coefficient pointers describe A^T (a -> c - 1, c -> a + 1),
// d is xbar, and the epilogue writes lambda to x and the gradients
// ga = -lambda x_{i-1}, gb = -lambda x_i, gc = -lambda x_{i+1} using the
// forward solution xf.
template <typename T>
struct PgeIO {
  const T *a, *b, *c, *d;
  T* x;
  const T* xf;
  T *ga, *gb, *gc;
  int* info;
  const long long* offsets;
  const int* list;
  size_t stride;
  int n;
  int pf_ahead;  // uniform batches: CTA b prefetches system b + pf_ahead into L2 (0: off)
  int* err;      // the library's device error word (bounded waits)
  // chunked long systems (MODE 2 / 3, uniform contiguous batches): CTA b is
  // chunk b % nchunks of system b / nchunks, chunk_rows rows of it
  int nchunks, chunk_rows;
  T* sep;        // [4][batch][nchunks NT]: the separator systems (sub, diag, super, rhs)
  T* carry;      // [batch][nchunks][4]: Y, V, W of partition 0's first row, c of the last separator row
  const T* xsep;  // [batch][nchunks NT]: the separators (MODE 3)
  int* flag;     // [batch]: MODE 3 sets 1 where a separator row misses its bound
  // ragged chunked systems (cl_sys non-NULL): CTA b is chunk cl_ch[b] of
  // system cl_sys[b] (rows [offsets[s], offsets[s+1])), whose separator rows
  // start at row sep_off[s] of the separator arrays (sep_total rows each) and
  // its chunks' carries at sep_off[s] / NT; systems with kinds[s] != want
  // are skipped
  const int* cl_sys;
  const int* cl_ch;
  const long long* sep_off;
  size_t sep_total;
  // (non-NULL) only the systems s with only[s] != 0 are served: the chunked
  // passes, and the entries the resident CTAs take by ticket
  const int* only;
  // size buckets of a ragged batch served by resident CTAs (clusters): each
  // takes the next entry of list[0 .. count) -- count from *dcount where a
  // device pass wrote the list -- from the ticket counter (zero before the
  // launch) until none is left, and skips the systems s with kinds[s] !=
  // want (kinds NULL: serves every entry)
  int* ticket;
  int count;
  const int* dcount;
  const unsigned char* kinds;
  int want;
  // the persistent TMA-staged kernel: its (next, done) ticket pair
  // (ring_tickets())
  int* ring;
};

// Tensor maps of the TMA-staged FP64 kernel (pge_kernel with SWZ): a, b, c,
// d, x of a uniform batch viewed as [partitions][2][16] elements, i.e. each
// 32-row partition as two 128-byte rows.
struct PgeMaps {
  CUtensorMap m[5];
};

// Rows per partition of the TMA-staged kernel.
constexpr int PGE_SWZ_M = 32;

// The TMA-staged kernel is persistent: each CTA takes systems by ticket (one
// ahead of the one it solves, so that it can load it early; a CTA held up by
// a system that needs the slow paths takes fewer) and solves them out of
// three half buffers of shared memory (a half buffer = rows 0-15 or 16-31 of
// every partition, for the four arrays).  The j-th
// system of a CTA has its first half in buffer 0 (j even) or 2 (j odd) and
// its second half in buffer 1.  The next system's first half is loaded into
// the other of buffers 0 / 2 while this one is solved; its second half
// follows into buffer 1 once this system's x (stored from buffers F and 1)
// has left shared memory, as the next system begins (of the refill points
// measured -- sweep rows 0, 1, 2, 4, 8 -- the earliest was fastest).  Every thread keeps the
// same copy of this state (the control flow that changes it is uniform).
struct PgeRing {
  int j;              // systems this CTA has begun
  unsigned fills[3];  // loads issued into each buffer (one mbarrier phase each)
  unsigned pend;      // bit b: a load into buffer b not yet waited for
  int next;           // the CTA's next system (io.count or more: none)
};

// Write rows r = lo + t, lo + t + nt, ... < hi of the result, value(r) from
// shared memory.  MODE 1 also writes the gradients; the forward solution's
// loads of U rows are issued before their stores (the outputs could alias
// xf as far as the compiler knows, which would otherwise serialise one load
// latency per row).
template <typename T, int MODE, typename Val>
__device__ __forceinline__ void pge_store_rows(const PgeIO<T>& io, size_t base, int n, int lo, int hi, int t, int nt,
                                               Val value) {
  if constexpr (MODE != 1) {
    for (int r = lo + t; r < hi; r += nt) io.x[base + r] = value(r);
  } else {
    const T* __restrict__ xf = io.xf + base;
    constexpr int U = 8;
    for (int r0 = lo + t; r0 < hi; r0 += U * nt) {
      T xl[U], xc[U], xr[U], v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + u * nt;
        xl[u] = xc[u] = xr[u] = v[u] = T(0);
        if (r < hi) {
          if (r > 0) xl[u] = __ldg(xf + r - 1);
          xc[u] = __ldg(xf + r);
          if (r < n - 1) xr[u] = __ldg(xf + r + 1);
          v[u] = value(r);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + u * nt;
        if (r < hi) {
          io.x[base + r] = v[u];
          io.ga[base + r] = r > 0 ? -v[u] * xl[u] : T(0);
          io.gb[base + r] = -v[u] * xc[u];
          io.gc[base + r] = r < n - 1 ? -v[u] * xr[u] : T(0);
        }
      }
    }
  }
}

// System addressing of CTA (or cluster) `bid`; m = rows per partition for R
// partitions (at least 2, so the last partitions may be identity rows).
template <typename T>
__device__ __forceinline__ void pge_system(const PgeIO<T>& io, int bid, int R, int& sys, size_t& base, int& n, int& m,
                                           int& ms) {
  sys = io.list ? io.list[bid] : bid;
  if (io.offsets) {
    base = (size_t)io.offsets[sys];
    n = (int)(io.offsets[sys + 1] - io.offsets[sys]);
  } else {
    base = (size_t)sys * io.stride;
    n = io.n;
  }
  m = (n + R - 1) / R;
  if (m < 2) m = 2;
  ms = m | 1;
}

// Staging modes of pge_kernel (template parameter LAY) and the shared-memory
// position of row i of partition p in each:
//  * PGE_DENSE: the system's rows in order (row r of array k at delta_k + r,
//    delta_k = the row's global address modulo 16 bytes, so that global and
//    shared 16-byte boundaries coincide), moved by one bulk copy per array;
//    the partition size m is odd, so the sweeps' column accesses -- lane t,
//    row i of partition t -- are conflict-free;
//  * PGE_SWZ (FP64, m = 32): each half of each array as [NT][16] elements
//    (the halves in two of the ring's half buffers, hs elements apart), half
//    h of partition p one 128-byte row whose 16-byte pairs are XOR-swizzled
//    by p mod 8 (the 128-byte swizzle of the tensor maps); column accesses
//    meet at most four-way bank conflicts.
constexpr int PGE_DENSE = 1, PGE_SWZ = 2;

template <int NT, int LAY>
__device__ __forceinline__ int pge_off(int p, int i, int m, int hs) {
  if constexpr (LAY == PGE_SWZ) return (i >> 4) * hs + p * 16 + ((((i >> 1) & 7) ^ (p & 7)) << 1) + (i & 1);
  else return p * m + i;  // (each staged array's base shifted by its delta)
}

// Elements per staged array: NT partitions of stride ms, plus the dense
// layout's shift, rounded to 16 bytes.
template <typename T, int NT>
__host__ __device__ constexpr int pge_array_elems(int ms) {
  return (NT * ms + 2 * (16 / (int)sizeof(T)) - 1) / (16 / (int)sizeof(T)) * (16 / (int)sizeof(T));
}

template <typename T, int NT, int MODE, int LAY>
__device__ __forceinline__ void pge_body(const PgeIO<T>& io, const PgeMaps& maps, const int bid, uint64_t* s_bar,
                                         PgeRing* rg = nullptr) {
  constexpr int VE = 16 / (int)sizeof(T);  // elements per 16 bytes
  int sys, n, m, ms;
  size_t base;
  int ch = 0;                       // chunk of a long system (MODE 2 / 3)
  size_t sq = 0;                    // its first separator row in io.sep / io.xsep
  bool zero_a0 = true, zero_cl = true;  // this CTA holds the system's first / last row
  if constexpr (MODE >= 2) {
    int nch;
    if (io.cl_sys) {
      sys = io.cl_sys[bid];
      ch = io.cl_ch[bid];
      if ((io.kinds && io.kinds[sys] != io.want) || (io.only && !io.only[sys])) return;  // (the whole CTA)
      const long long s0 = io.offsets[sys];
      const int nsys = (int)(io.offsets[sys + 1] - s0);
      nch = (nsys + io.chunk_rows - 1) / io.chunk_rows;
      base = (size_t)s0 + (size_t)ch * io.chunk_rows;
      n = min(io.chunk_rows, nsys - ch * io.chunk_rows);
      sq = (size_t)io.sep_off[sys];
    } else {
      sys = bid / io.nchunks;
      ch = bid % io.nchunks;
      nch = io.nchunks;
      base = (size_t)sys * io.stride + (size_t)ch * io.chunk_rows;
      n = min(io.chunk_rows, io.n - ch * io.chunk_rows);
      sq = (size_t)sys * io.nchunks * NT;
    }
    m = ms = io.chunk_rows / NT;  // odd (the launch's choice)
    zero_a0 = ch == 0;
    zero_cl = ch == nch - 1;
  } else {
    pge_system(io, bid, NT, sys, base, n, m, ms);
  }
  if constexpr (LAY == PGE_SWZ) ms = PGE_SWZ_M;  // (the launch guarantees n = NT * 32)
  if constexpr (LAY == PGE_DENSE) m |= 1;        // odd partitions (ms = m)
  const T* __restrict__ ga = io.a;
  const T* __restrict__ gb = io.b;
  const T* __restrict__ gc = io.c;
  const T* gd = io.d;
  int* info = io.info;
  extern __shared__ __align__(16) unsigned char pge_smem[];
  unsigned char* sm = pge_smem;
  if constexpr (LAY == PGE_SWZ) sm += (1024u - (smem_u32(pge_smem) & 1023u)) & 1023u;  // 128-byte swizzle: 1 KB aligned
  const int astride = pge_array_elems<T, NT>(ms);
  T* S0 = reinterpret_cast<T*>(sm);
  // dense layout: each staged array shifted by its rows' 16-byte phase
  auto phase = [&](const T* g) {
    return LAY == PGE_DENSE ? (int)((reinterpret_cast<uintptr_t>(g + base) / sizeof(T)) % VE) : 0;
  };
  const int dl[4] = {phase(ga), phase(gb), phase(gc), phase(gd)};
  T* SA = S0 + dl[0];
  T* SB = S0 + astride + dl[1];
  T* SC = S0 + 2 * astride + dl[2];
  T* SD = S0 + 3 * astride + dl[3];
  T* SX = S0 + 4 * astride;  // x kept across refinement passes
  T* SEP = SX + astride;     // [3][4][NT] separator rows: original + ping-pong
  // TMA-staged ring: this system's halves in buffers F and 1 (hs elements
  // apart), the refinement copy of x (rare) in the third buffer
  constexpr int HB = 4 * NT * 16;  // elements per half buffer
  const int F = LAY == PGE_SWZ && (rg->j & 1) ? 2 : 0;
  const int hs = (1 - F) * HB;
  if constexpr (LAY == PGE_SWZ) {
    SA = S0 + F * HB;
    SB = SA + NT * 16;
    SC = SA + 2 * NT * 16;
    SD = SA + 3 * NT * 16;
    SX = S0 + (2 - F) * HB;
    SEP = S0 + 3 * HB;
  }
  auto off = [&](int p, int i) { return pge_off<NT, LAY>(p, i, m, hs); };
  T* FST = SEP + 12 * NT;  // [3][NT]: Y, V, W of each partition's first row
  T* TMP = FST + 3 * NT;  // [PGE_TMP]: the FP32 separator solve's top level
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  using MagT = unsigned;
  __shared__ MagT s_amax, s_dmax, s_xmax;
  __shared__ T s_xprev, s_xnext;  // x of the neighbouring chunks' adjacent rows (MODE 3)
  MagT amax = 0, dmax = 0;
  if (t == 0) {
    s_amax = 0;
    s_dmax = 0;
    s_xmax = 0;
    s_xprev = T(0);
    s_xnext = T(0);
  }
  // dense layout: rows [r0[k], r1[k]) of array k start and end on 16-byte
  // boundaries in global and shared memory and move in bulk; the rest
  // element-wise.  Row 0 of a and row n-1 of c are never read (zero; the
  // adjoint's shifted pointers would read outside the arrays there), so
  // they stay out of the bulk ranges.
  int r0[4] = {0, 0, 0, 0}, r1[4] = {0, 0, 0, 0};
  if constexpr (LAY == PGE_DENSE) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      r0[k] = min(n, (VE - dl[k]) % VE);
      r1[k] = r0[k] + (n - r0[k]) / VE * VE;
    }
    if (zero_a0 && r0[0] == 0) r0[0] = min(VE, r1[0]);
    if (zero_cl && r1[2] == n && r1[2] > r0[2]) r1[2] -= VE;
  }

  // ---- stage the system.  SWZ: one TMA box (16 rows x NT partitions) per
  // array and half, each half counted on its own mbarrier, so that the
  // forward sweep starts on rows 0-15 while rows 16-31 are in flight.
  // DENSE: one bulk copy per array (rows [r0, r1)), the few rows around it
  // and the identity rows past n by plain copies.  (An SM issues about one
  // bulk or element copy per 15 cycles: element copies of 4 or 8 bytes, or
  // one bulk copy per partition, ran at 7-17 bytes per clock.)
  // (TMA-staged ring) half h of system s into half buffer b: issued by
  // thread 0, counted by every thread; wait_fill(b) waits for the latest one
  auto fill = [&](int b, int h, int s) {
    if (t == 0) {
      mbar_arrive_expect_tx(&s_bar[b], (unsigned)(HB * sizeof(T)));
      for (int k = 0; k < 4; ++k) tma_load_3d(S0 + b * HB + k * NT * 16, &maps.m[k], 0, h, s * NT, &s_bar[b]);
    }
    ++rg->fills[b];
    rg->pend |= 1u << b;
  };
  auto wait_fill = [&](int b) {
    rg->pend &= ~(1u << b);
    return mbar_wait(&s_bar[b], (rg->fills[b] - 1u) & 1u, io.err);
  };
  const int nxt = LAY == PGE_SWZ ? rg->next : 0;  // (ring) this CTA's next system
  const bool has_next = LAY == PGE_SWZ && nxt < io.count;
  bool clobbered = false;  // (ring) the refinement copy of x overwrote the next system's first half
  if constexpr (LAY == PGE_SWZ) {
    if (rg->j == 0) {
      if (t == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        mbar_init(&s_bar[2], 1);
        fence_mbar_init();
      }
      fill(0, 0, sys);
      fill(1, 1, sys);
      if (has_next) fill(2, 0, nxt);
    }
  } else if constexpr (LAY == PGE_DENSE) {
    T* const Sk[4] = {SA, SB, SC, SD};
    const T* const Gk[4] = {ga, gb, gc, gd};
    if (t == 0) {
      mbar_init(&s_bar[0], 1);
      fence_mbar_init();
      unsigned total = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) total += (unsigned)((r1[k] - r0[k]) * sizeof(T));
      mbar_arrive_expect_tx(&s_bar[0], total);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (r1[k] > r0[k])
          bulk_load_1d(Sk[k] + r0[k], Gk[k] + base + r0[k], (unsigned)((r1[k] - r0[k]) * sizeof(T)), &s_bar[0]);
    }
    // rows outside the bulk ranges (fewer than 16 bytes at either end, plus
    // row 0 of a and row n-1 of c), identity past n
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      auto plain = [&](int r) {
        Sk[k][r] = (k == 0 && r == 0 && zero_a0) || (k == 2 && r == n - 1 && zero_cl) ? T(0) : Gk[k][base + r];
      };
      if (t < r0[k]) plain(t);
      if (t < n - r1[k]) plain(r1[k] + t);
      for (int r = n + t; r < NT * m; r += NT) Sk[k][r] = k == 1 ? T(1) : T(0);
    }
    __syncthreads();  // (the mbarrier's initialisation, before anyone waits)
    if (!mbar_wait(&s_bar[0], 0, io.err) && t == 0) {
      // a copy that never landed (the device error word has the timeout):
      // solve identity rows there rather than stale shared memory
#pragma unroll
      for (int k = 0; k < 4; ++k)
        for (int r = r0[k]; r < r1[k]; ++r) Sk[k][r] = k == 1 ? T(1) : T(0);
    }
  }
  // One CTA per SM fits: the CTA that runs here next (about one wave later)
  // finds its system in L2 instead of HBM.
  if (io.pf_ahead > 0 && t == 0 && bid + io.pf_ahead < (int)gridDim.x) {
    const size_t nb = (size_t)(bid + io.pf_ahead) * io.stride;
    const unsigned bytes = (unsigned)((size_t)n * sizeof(T)) & ~15u;
    const T* arr[4] = {ga, gb, gc, gd};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(arr[k] + nb), "r"(bytes) : "memory");
  }
  __syncthreads();

  bool accepted = false;
#pragma unroll 1
  for (int pass = 0; pass <= PGE_REFINE; ++pass) {
  // ---- forward elimination of partition t's interior block (rows 0 ..
  // mi-1) with partial pivoting, for three right-hand sides: d, the left
  // spike a_0 e_0 and the right spike c_{mi-1} e_{mi-1}.  U row i is stored
  // as (1/u0_i -> A, u1_i -> B, z_i -> C, y'_i -> D) and swap bit i of swm:
  // when rows i and i+1 were interchanged, u2_i = z_i (= c_{i+1}) and
  // v'_i = 0, else u2_i = 0 and v'_i = z_i -- one of the two is always zero,
  // so one array holds both and the back substitution's term is
  // z_i * (swap ? x_{i+2} : s_{t-1}).  The separator
  // system needs the first and last rows of U^{-1} applied to the three
  // eliminated right-hand sides: the last row is y'/u0 of the last U row;
  // the first row omega = e_0^T U^{-1} follows the recurrence
  //   omega_i u0_i + omega_{i-1} u1_{i-1} + omega_{i-2} u2_{i-2} = [i = 0],
  // accumulated into omega . y', omega . v', omega . w' during the sweep.
  const int mi = m - 1;
  auto A = [&](int i) -> T& { return SA[off(t, i)]; };
  auto B = [&](int i) -> T& { return SB[off(t, i)]; };
  auto C = [&](int i) -> T& { return SC[off(t, i)]; };
  auto D = [&](int i) -> T& { return SD[off(t, i)]; };
  unsigned long long swm = 0ull;  // swap bits of U rows 0 .. mi-2 (m <= 64)
  bool bad = false;  // this pass: breakdown, non-finite or (pass 0) separator residual
  T cb, cc, cy, cv, cw;                        // the candidate row (b, c, y', v', w')
  T w_prev = T(0);                             // w' of U row mi-2 (the only other nonzero w')
  T om1 = T(0), om2 = T(0);                    // omega_{i-1}, omega_{i-2}
  T kro = T(1);                                // [i = 0] of the omega recurrence
  T pu1 = T(0), pu2a = T(0), pu2b = T(0);      // u1_{i-1}, u2_{i-1}, u2_{i-2}
  T Y0 = T(0), V0 = T(0);                      // omega . y', omega . v'
  T as, bs, cs, ds;                            // the separator row m-1
  auto first_row = [&](T a0, T b0, T c0, T d0) {
    cb = b0;
    cc = mi > 1 ? c0 : T(0);
    cy = d0;
    cv = a0;
    cw = mi == 1 ? c0 : T(0);
    amax = max(amax, max(magh(a0), max(magh(b0), magh(c0))));  // magnitudes for the acceptance test
    dmax = max(dmax, magh(d0));
  };
  // row i+1 (a, b, c, y) against the candidate row: U row i.  LAST (row
  // i+1 is the last interior row, i = mi-2) is a compile-time tag: as a
  // run-time test the right spike's product below was formed on every row
  // and discarded on all but one.
  auto eliminate = [&](int i, T na, T nb, T cn, T ny, auto last_tag) {
    constexpr bool last = decltype(last_tag)::value;
    amax = max(amax, max(magh(na), max(magh(nb), magh(cn))));
    dmax = max(dmax, magh(ny));
    const T nc = last ? T(0) : cn;
    const bool sw = !abs_ge(cb, na);
    const T piv = sw ? na : cb;
    bad |= is_zero(piv);
    const T inv = Div<T>(piv).inv();
    const T l = (sw ? cb : na) * inv;
    const T u1 = sw ? nb : cc;
    const T u2 = keep_if(sw, nc);
    const T uy = sw ? ny : cy;
    const T uv = keep_if(!sw, cv);
    const T zs = sw ? nc : cv;  // the nonzero one of u2 and v'
    const T om = fma(-om2, pu2b, fma(-om1, pu1, kro)) * inv;
    kro = T(0);
    Y0 = fma(om, uy, Y0);
    V0 = fma(om, uv, V0);
    om2 = om1;
    om1 = om;
    pu2b = pu2a;
    pu2a = u2;
    pu1 = u1;
    A(i) = inv;
    B(i) = u1;
    C(i) = zs;  // c_i was read two rows ago
    D(i) = uy;
    swm |= (unsigned long long)sw << i;
    cb = fma(-l, u1, sw ? cc : nb);
    // the row left behind keeps one of c_{i+2} (no swap) and the left spike
    // (swap); the other is scaled by -l: one product for both
    const T tq = -l * zs;
    cc = sw ? tq : nc;
    cy = fma(-l, uy, sw ? cy : ny);
    cv = sw ? cv : tq;
    if constexpr (last) {  // the right spike enters with row mi-1
      w_prev = sw ? cn : cw;
      cw = fma(-l, w_prev, sw ? cw : cn);
    }
  };
  {
    // first pass of a TMA-staged system: wait for each half as the sweep
    // reaches it (a timeout marks the pass bad: the system is then restaged
    // and solved by the refinement passes)
    if constexpr (LAY == PGE_SWZ)
      if (pass == 0) {
        if (rg->j > 0) {
          // the previous system's x stores leave buffers 1 and 2-F: this
          // system's second half and the next system's first half go there
          if (t == 0) bulk_wait_read<0>();
          fill(1, 1, sys);
          if (has_next) fill(2 - F, 0, nxt);
        }
        bad |= !wait_fill(F);
      }
    // a_0 and c_{n-1} are zero by definition (TMA staging copies whatever
    // the arrays hold there)
    first_row(t == 0 && zero_a0 ? T(0) : A(0), B(0), C(0), D(0));
    // software-pipelined: row i+2 (at most the separator row, which always
    // exists) is loaded while row i+1 is eliminated
    T pa = A(1), pb = B(1), pc = C(1), py = D(1);
    auto step = [&](int i) {
      const T na = pa, nb = pb, cn = pc, ny = py;
      pa = A(i + 2);
      pb = B(i + 2);
      pc = C(i + 2);
      py = D(i + 2);
      eliminate(i, na, nb, cn, ny, std::false_type{});
    };
    if constexpr (LAY == PGE_SWZ) {
      // (m = 32: rows 0-15 in buffer F, rows 16-31 in buffer 1; the wait
      // for the second half sits between two loops, out of their bodies)
      int i = 0;
      for (; i < 14; ++i) step(i);
      if (pass == 0) bad |= !wait_fill(1);  // (step 14 loads row 16)
      for (; i + 2 < mi; ++i) step(i);
    } else {
      for (int i = 0; i + 2 < mi; ++i) step(i);
    }
    as = A(mi);
    bs = B(mi);
    cs = t * m + mi == n - 1 && zero_cl ? T(0) : C(mi);
    ds = D(mi);
    if (mi >= 2) eliminate(mi - 2, pa, pb, pc, py, std::true_type{});
  }
  // U row mi-1 is the remaining candidate row (u1 = u2 = 0)
  bad |= is_zero(cb);
  const T inv_last = Div<T>(cb).inv();
  {
    const T om = fma(-om2, pu2b, fma(-om1, pu1, kro)) * inv_last;
    Y0 = fma(om, cy, Y0);
    V0 = fma(om, cv, V0);
    const T W0 = fma(om1, w_prev, om * cw);
    FST[t] = Y0;
    FST[NT + t] = V0;
    FST[2 * NT + t] = W0;
  }
  const T Ylast = cy * inv_last, Vlast = cv * inv_last, Wlast = cw * inv_last;
  A(mi - 1) = inv_last;
  B(mi - 1) = T(0);
  C(mi - 1) = cv;  // z of the last U row: v' (no u2; its swap bit is 0)
  D(mi - 1) = cy;
  __syncthreads();

  // ---- separator system: row m-1 of partition t couples to the last
  // interior row of t and the first row of t+1
  amax = max(amax, max(magh(as), max(magh(bs), magh(cs))));
  dmax = max(dmax, magh(ds));
  if (pass == 0) {
    atomicMax(&s_amax, amax);
    atomicMax(&s_dmax, dmax);
  }
  {
    const bool has_next = t + 1 < NT;
    const T Yf = has_next ? FST[t + 1] : T(0);
    const T Vf = has_next ? FST[NT + t + 1] : T(0);
    const T Wf = has_next ? FST[2 * NT + t + 1] : T(0);
    SEP[t] = -as * Vlast;
    SEP[NT + t] = fma(-cs, Vf, fma(-as, Wlast, bs));
    SEP[2 * NT + t] = -cs * Wf;
    SEP[3 * NT + t] = fma(-cs, Yf, fma(-as, Ylast, ds));
    if constexpr (MODE == 2) {
      // a long system's chunk: its separator rows go to the system-wide
      // separator system; the last one still lacks the next chunk's first
      // row (added by pge_long_link from `carry`)
      const size_t bsz = io.sep_total;
      const size_t q = sq + (size_t)ch * NT + t;
      io.sep[q] = SEP[t];
      io.sep[bsz + q] = SEP[NT + t];
      io.sep[2 * bsz + q] = SEP[2 * NT + t];
      io.sep[3 * bsz + q] = SEP[3 * NT + t];
      T* cy_ = io.carry + (sq / NT + ch) * 4;
      if (t == 0) {
        cy_[0] = FST[0];
        cy_[1] = FST[NT];
        cy_[2] = FST[2 * NT];
      }
      if (t == NT - 1) cy_[3] = cs;
      return;
    }
  }
  __syncthreads();
  if constexpr (MODE == 3) {
    // the separators from the system-wide solve
    FST[t] = io.xsep[sq + (size_t)ch * NT + t];
  } else {
  // Parallel cyclic reduction of the separator system (SEP[0..4NT) keeps the
  // original rows, SEP[4NT..12NT) is the ping-pong pair) ...  Thread t owns
  // row t through all steps and keeps it in registers; what its neighbours
  // read is published as (a, 1/b, c, d), so each row's reciprocal is formed
  // once per step by its owner instead of once by each of its two readers.
  {
    T ra = SEP[t], rb = SEP[NT + t], rc = SEP[2 * NT + t], rd = SEP[3 * NT + t];
    T ri = Div<T>(rb).inv();
    T* cur = SEP + 4 * NT;
    cur[t] = ra;
    cur[NT + t] = ri;
    cur[2 * NT + t] = rc;
    cur[3 * NT + t] = rd;
    __syncthreads();
    int ph = 2;
#pragma unroll 1
    for (int s = 1; s < NT; s <<= 1) {
      T nb = rb, nd = rd, na = T(0), nc = T(0);
      if (t >= s) {
        const T al = ra * cur[NT + t - s];
        nb = fma(-al, cur[2 * NT + t - s], nb);
        nd = fma(-al, cur[3 * NT + t - s], nd);
        na = -al * cur[t - s];
      }
      if (t + s < NT) {
        const T gm = rc * cur[NT + t + s];
        nb = fma(-gm, cur[t + s], nb);
        nd = fma(-gm, cur[3 * NT + t + s], nd);
        nc = -gm * cur[2 * NT + t + s];
      }
      ra = na;
      rb = nb;
      rc = nc;
      rd = nd;
      ri = Div<T>(rb).inv();
      if (2 * s < NT) {  // (after the last step every row stands alone)
        T* nxt = SEP + ph * 4 * NT;
        nxt[t] = ra;
        nxt[NT + t] = ri;
        nxt[2 * NT + t] = rc;
        nxt[3 * NT + t] = rd;
        cur = nxt;
        ph = 3 - ph;
        __syncthreads();
      }
    }
    FST[t] = rd * ri;  // FST is free again: separator values
  }
  __syncthreads();
  // ... accepted when its normwise backward error on the separator system is
  // within a few units of roundoff; otherwise (PCR does not pivot, and on
  // non-dominant separator systems its growth can be large) warp 0 solves
  // the separator system again with partial pivoting.
  {
    const T st = FST[t];
    const T sp = t > 0 ? FST[t - 1] : T(0), sn = t + 1 < NT ? FST[t + 1] : T(0);
    const T sa = SEP[t], sb = SEP[NT + t], sc = SEP[2 * NT + t], sd = SEP[3 * NT + t];
    const T r = fma(-sc, sn, fma(-sb, st, fma(-sa, sp, sd)));
    const T scale = fabs(sa * sp) + fabs(sb * st) + fabs(sc * sn) + fabs(sd);
    const T tol = sizeof(T) == 8 ? T(16 * 1.1102230246251565e-16) : T(4 * 5.9604645e-8);
    const bool reject = !(fabs(r) <= tol * scale);  // also catches NaN/Inf
    if (__syncthreads_or(reject)) {
      if (pass == 0 && t == 0) atomicAdd(&g_pge_paths[0], 1ull);
      if (warp == 0) bad |= sep_solve_pivoted<T, NT>(SEP, FST, TMP, lane);
    }
  }
  }  // MODE != 3
  __syncthreads();
  // ---- back substitution of the interior block with the separators in
  // place: x_i = (y'_i - v'_i s_{t-1} - w'_i s_t - u1_i x_{i+1} - u2_i x_{i+2})
  // / u0_i, i.e. the interior rows are solved directly for their true
  // right-hand side (backward stable with partial pivoting).  What remains
  // to check is the separator rows: their residuals are formed exactly and
  // must meet SEP_TOL relative to max|A| max|x| + max|d|; a failing system
  // gets an exact backward-error check of all rows, then (if that fails
  // too) the sequential partial-pivoting solve.
  T sp = t > 0 ? FST[t - 1] : T(0);
  if constexpr (MODE == 3)
    if (t == 0 && ch > 0) {
      sp = io.xsep[sq + (size_t)ch * NT - 1];
      s_xprev = sp;  // (the previous chunk's last row is its last separator)
    }
  const T st = FST[t];
  MagT xmax = magh(st);
  T x_last;
  {
    T x1 = (fma(-cw, st, fma(-C(mi - 1), sp, D(mi - 1)))) * inv_last;
    T x2 = T(0);
    D(mi - 1) = x1;
    xmax = max(xmax, magh(x1));
    bad |= !finite_val(x1);
    x_last = x1;
    // software-pipelined: row i-1's factors are loaded while row i is solved
    int j = mi - 2 >= 0 ? mi - 2 : 0;
    T qz = C(j), qd = D(j), qb = B(j), qa = A(j);
    // (row mi-2, the one row with a right-spike term, is peeled off the loop
    // by the compile-time tag: as a run-time test its product was formed on
    // every row)
    auto back_row = [&](int i, auto spike_tag) {
      const T zi = qz, di = qd, bi = qb, ai = qa;
      j = i > 0 ? i - 1 : 0;
      qz = C(j);
      qd = D(j);
      qb = B(j);
      qa = A(j);
      // z_i multiplies x_{i+2} (swap) or the previous separator (no swap)
      const T zx = (swm >> i) & 1ull ? x2 : sp;
      T r = fma(-zi, zx, di);
      if constexpr (decltype(spike_tag)::value) r = fma(-w_prev, st, r);
      const T xi = fma(-bi, x1, r) * ai;  // one op on x_{i+1}, then the reciprocal
      D(i) = xi;
      xmax = max(xmax, magh(xi));
      bad |= !finite_val(xi);
      x2 = x1;
      x1 = xi;
    };
    if (mi >= 2) back_row(mi - 2, std::true_type{});
    for (int i = mi - 3; i >= 0; --i) back_row(i, std::false_type{});
    bad |= !finite_val(st);
    D(mi) = st;
    FST[NT + t] = D(0);  // first x of the partition, for the separator residual of t-1
    if (pass == 0) atomicMax(&s_xmax, xmax);
    __syncthreads();
    T x_next = t + 1 < NT ? FST[NT + t + 1] : T(0);
    if constexpr (MODE == 3) {
      if (t + 1 == NT && !zero_cl) {
        // the next chunk's first row: x = Y - V s_t - W s_{t+1}
        const T* cy_ = io.carry + (sq / NT + ch + 1) * 4;
        const T s_next = io.xsep[sq + (size_t)(ch + 1) * NT];
        x_next = fma(-cy_[2], s_next, fma(-cy_[1], st, cy_[0]));
        s_xnext = x_next;
      }
    }
    // (one row per partition: formed in FP64 for both precisions)
    const double r = fma(-(double)cs, (double)x_next,
                         fma(-(double)bs, (double)st, fma(-(double)as, (double)x_last, (double)ds)));
    const T amx = Fmt<T>::from_mag(s_amax), xmx = Fmt<T>::from_mag(s_xmax), dmx = Fmt<T>::from_mag(s_dmax);
    if (pass == 0) bad |= !(fabs(r) <= Fmt<T>::SEP_TOL * fma((double)amx, (double)xmx, (double)dmx));
  }
  // ---- acceptance.  A pass-0 result whose separator rows meet the bound
  // is kept as is.  Otherwise the normwise backward error
  //   max|d - A x| / (|A|_inf |x|_inf + |d|_inf)
  // of the current x (pass 0: the result, later passes: the sum of the
  // result and its corrections) is measured exactly (FP64, inputs re-read
  // from global memory); when it misses SEP_TOL, x is refined: the FP64
  // residual becomes the right-hand side of another pass (a, b, c
  // restaged), whose solution is added to x.  After PGE_REFINE corrections
  // the sequential partial-pivoting solve takes over.
  const bool pass_bad = __syncthreads_or(bad);
  if (pass == 0 && !pass_bad) {
    accepted = true;
    break;
  }
  if (t == 0) atomicAdd(&g_pge_paths[pass == 0 ? 1 : 2], 1ull);
  auto sidx = [&](int r) { return off(r / m, r % m); };
  if (pass > 0 && !pass_bad) {
    // x = x_prev (held in SX) + correction
    for (int r = t; r < n; r += NT) SD[sidx(r)] += SX[r];
    __syncthreads();
  }
  if (!pass_bad || pass == 0) {
    __shared__ unsigned long long s_rmax, s_anorm, s_xn, s_dn;
    if (t == 0) {
      s_rmax = 0ull;
      s_anorm = 0ull;
      s_xn = 0ull;
      s_dn = 0ull;
    }
    __syncthreads();
    unsigned long long rmax = 0ull, anorm = 0ull, xn = 0ull, dn = 0ull;
    bool nonfinite = false;
    // (a long system's chunk: its first and last rows couple to x of the
    // neighbouring chunks, s_xprev / s_xnext)
    for (int r = t; r < n; r += NT) {
      const double ar = r > 0 || !zero_a0 ? (double)ga[base + r] : 0.0, br = (double)gb[base + r];
      const double cr = r < n - 1 || !zero_cl ? (double)gc[base + r] : 0.0, dr = (double)gd[base + r];
      const double xr = (double)SD[sidx(r)];
      double res = fma(-br, xr, dr);
      res = fma(-ar, r > 0 ? (double)SD[sidx(r - 1)] : (double)s_xprev, res);
      res = fma(-cr, r < n - 1 ? (double)SD[sidx(r + 1)] : (double)s_xnext, res);
      nonfinite |= !finite_val(res);
      rmax = max(rmax, mag(res));
      anorm = max(anorm, mag(fabs(ar) + fabs(br) + fabs(cr)));
      xn = max(xn, mag(xr));
      dn = max(dn, mag(dr));
    }
    atomicMax(&s_rmax, rmax);
    atomicMax(&s_anorm, anorm);
    atomicMax(&s_xn, xn);
    atomicMax(&s_dn, dn);
    __syncthreads();
    const double eta = __longlong_as_double((long long)s_rmax) /
                       fma(__longlong_as_double((long long)s_anorm), __longlong_as_double((long long)s_xn),
                           __longlong_as_double((long long)s_dn));
    if (!__syncthreads_or(nonfinite || !(eta <= Fmt<T>::SEP_TOL))) {
      accepted = true;
      break;
    }
    if constexpr (MODE == 3) {
      // a chunk cannot refine alone: mark the system for the sequential
      // solve (counted once per system)
      if (t == 0 && atomicExch(&io.flag[sys], 1) == 0) atomicAdd(&g_pge_fallbacks, 1ull);
      accepted = true;
      break;
    }
    if (pass == PGE_REFINE) break;
    if constexpr (LAY == PGE_SWZ) {
      // SX is the next system's first-half buffer: let that load land, take
      // the buffer, and load it again when this system is done
      if (rg->pend & (1u << (2 - F))) wait_fill(2 - F);
      clobbered = has_next;
    }
    // keep x in SX (row r at r) and stage the FP64 residual as the next
    // right-hand side
    for (int r = t; r < n; r += NT) SX[r] = SD[sidx(r)];
    __syncthreads();
  } else {
    break;  // a correction pass broke down
  }
  for (int r = t; r < NT * m; r += NT) {
    const int q = sidx(r);
    if (r < n) {
      const T ar = r > 0 ? ga[base + r] : T(0), br = gb[base + r], cr = r < n - 1 ? gc[base + r] : T(0);
      double res = fma(-(double)br, (double)SX[r], (double)gd[base + r]);
      if (r > 0) res = fma(-(double)ar, (double)SX[r - 1], res);
      if (r < n - 1) res = fma(-(double)cr, (double)SX[r + 1], res);
      SA[q] = ar;
      SB[q] = br;
      SC[q] = cr;
      SD[q] = (T)res;
    } else {
      SA[q] = T(0);
      SB[q] = T(1);
      SC[q] = T(0);
      SD[q] = T(0);
    }
  }
  __syncthreads();
  }  // passes

  if (!accepted) {
    // restage the system densely (4 arrays of n rows fit in the 5 NT ms
    // staging elements; the ring: in buffers F and 1, contiguous) and solve
    // it in place by one thread
    T* FA = LAY == PGE_SWZ ? S0 + (F == 0 ? 0 : HB) : SA;
    T* FB = FA + n;
    T* FC = FB + n;
    T* FD = FC + n;
    __syncthreads();
    for (int r = t; r < n; r += NT) {
      FA[r] = r > 0 ? ga[base + r] : T(0);
      FB[r] = gb[base + r];
      FC[r] = r < n - 1 ? gc[base + r] : T(0);
      FD[r] = gd[base + r];
    }
    __shared__ int s_info;
    __syncthreads();
    if (t == 0) {
      atomicAdd(&g_pge_fallbacks, 1ull);
      s_info = seq_pivoted_inplace<T>(FA, FB, FC, FD, n);
      if (info) info[sys] = s_info;
    }
    __syncthreads();
    if (s_info == 0)
      pge_store_rows<T, MODE>(io, base, n, 0, n, t, NT, [&](int r) { return FD[r]; });
    if constexpr (LAY == PGE_SWZ) {
      fence_async_smem();  // (the buffers are reloaded by the TMA)
      __syncthreads();
      if (clobbered) fill(2 - F, 0, nxt);
    }
    return;
  }
  if (MODE < 2 && info && t == 0) info[sys] = 0;
  if constexpr (LAY == PGE_SWZ) {
    // x by two TMA stores (the rows were written by several threads in a
    // refinement pass: fence, then barrier)
    fence_async_smem();
    __syncthreads();
    if (t == 0) {
      tma_store_3d(&maps.m[4], 0, 0, sys * NT, SD);
      tma_store_3d(&maps.m[4], 0, 1, sys * NT, SD + hs);
      bulk_commit();
      // (not waited for here: the next system's sweep, or the kernel's end,
      // waits until the stores have read buffers F and 1)
    }
    if (clobbered) fill(2 - F, 0, nxt);
  } else if (LAY == PGE_DENSE && (MODE == 0 || MODE == 3) && phase(io.x) == dl[3]) {
    // rows [q0, q1) of x by one bulk store (x in the same 16-byte phase as
    // d), the rest element-wise
    const int q0 = min(n, (VE - dl[3]) % VE), q1 = q0 + (n - q0) / VE * VE;
    fence_async_smem();
    __syncthreads();
    if (t == 0 && q1 > q0) {
      bulk_store_1d(io.x + base + q0, SD + q0, (unsigned)((q1 - q0) * sizeof(T)));
      bulk_commit();
    }
    if (t < q0) io.x[base + t] = SD[t];
    if (t < n - q1) io.x[base + q1 + t] = SD[q1 + t];
    if (t == 0 && q1 > q0) bulk_wait_read<0>();
  } else {
    pge_store_rows<T, MODE>(io, base, n, 0, n, t, NT, [&](int r) { return SD[r]; });  // (dense: row r at r)
  }
}

// The next entry of a ticket-driven bucket (the same for every thread of the
// CTA), or -1 when the bucket is exhausted or a device error was recorded.
template <typename T>
__device__ __forceinline__ int pge_next_item(const PgeIO<T>& io, int* s_item) {
  if (threadIdx.x == 0) {
    const int k = atomicAdd(io.ticket, 1);
    const int cnt = io.dcount ? *(volatile const int*)io.dcount : io.count;
    *s_item = k < cnt && (!io.err || *(volatile int*)io.err == 0) ? k : -1;
  }
  __syncthreads();
  const int k = *s_item;
  __syncthreads();  // (read by all before thread 0 writes the next one)
  return k;
}

template <typename T, int NT, int MODE, int LAY>
__global__ void __launch_bounds__(NT, 1) pge_kernel(const PgeIO<T> io, const __grid_constant__ PgeMaps maps) {
  __shared__ __align__(8) uint64_t s_bar[3];
  if constexpr (LAY == PGE_SWZ) {
    // persistent: systems blockIdx.x, + gridDim.x, ... < io.count through
    // the ring of half buffers; a device error (a load that never landed)
    // ends the loop
    __shared__ int s_stop, s_tk[2];
    PgeRing rg{0, {0u, 0u, 0u}, 0u, 0};
    if (threadIdx.x == 0) {
      s_tk[0] = atomicAdd(io.ring, 1);
      s_tk[1] = atomicAdd(io.ring, 1);
    }
    __syncthreads();
    int k = s_tk[0];
    rg.next = s_tk[1];
    while (k < io.count) {
      // the ticket after the next one (whose first half the next sweep
      // loads) and the device error word, asked for now and read after this
      // system: their latency hides behind its solve
      int tk = 0, err = 0;
      if (threadIdx.x == 0) {
        tk = rg.next < io.count ? atomicAdd(io.ring, 1) : io.count;
        err = *(volatile int*)io.err;
      }
      pge_body<T, NT, MODE, LAY>(io, maps, k, s_bar, &rg);
      ++rg.j;
      if (threadIdx.x == 0) {
        s_tk[0] = tk;
        s_stop = err != 0;
      }
      __syncthreads();
      if (s_stop) break;
      k = rg.next;
      rg.next = s_tk[0];
    }
    // loads and stores still in flight end before the shared memory is released
    for (int b = 0; b < 3; ++b)
      if (rg.pend & (1u << b)) mbar_wait(&s_bar[b], (rg.fills[b] - 1u) & 1u, io.err);
    if (threadIdx.x == 0) {
      bulk_wait_read<0>();
      // every CTA counts itself out once it takes no more tickets; the last
      // one zeroes the pair for the launch that uses it next
      __threadfence();
      if (atomicAdd(io.ring + 1, 1) == (int)gridDim.x - 1) {
        atomicExch(io.ring, 0);
        atomicExch(io.ring + 1, 0);
      }
    }
    return;
  }
  if constexpr (LAY == PGE_DENSE && MODE <= 1) {
    if (io.ticket) {
      // resident CTAs drain one size bucket of a ragged batch
      __shared__ int s_item;
      for (int k = pge_next_item(io, &s_item); k >= 0; k = pge_next_item(io, &s_item)) {
        if (io.kinds && io.kinds[io.list[k]] != io.want) continue;
        if (io.only && !io.only[io.list[k]]) continue;
        pge_body<T, NT, MODE, LAY>(io, maps, k, s_bar);
        __syncthreads();
        if (threadIdx.x == 0) mbar_inval(&s_bar[0]);  // re-armed by the next system
      }
      return;
    }
  }
  pge_body<T, NT, MODE, LAY>(io, maps, blockIdx.x, s_bar);
}

// ---------------------------------------------------------------------------
// Cluster version for systems longer than one CTA's shared memory: a cluster
// of CL CTAs holds one system, CTA r the rows [r NT m, (r+1) NT m), so the
// system is read from HBM once and kept in the cluster's distributed shared
// memory.  Partitions, forward elimination, back substitution and the
// acceptance test are those of pge_kernel with the partition index
// P = r NT + t; the separator system of the R = CL NT partitions is gathered
// into CTA 0 and solved there with partial pivoting in two levels (each
// thread eliminates a chunk of CL separators, warp 0 solves the NT chunk
// tops).  Neighbouring values across CTA boundaries travel through DSMEM.
// A result that fails the exact backward-error check after PGE_REFINE_CL
// correction passes is still written, with info = n + 1.

constexpr int PGE_REFINE_CL = 3;

template <typename T, int NT, int CL>
struct PgcLayout {
  static constexpr int R = CL * NT;
  // element offsets after the 6 NT ms staging arrays
  static constexpr int FST = 0, XF = 3 * NT, RED = 4 * NT, SOL = RED + 4 * R, XCH = SOL + R, TOP = XCH + 3 * NT,
                       TSOL = TOP + 4 * NT, TMP = TSOL + NT, END = TMP + PGE_TMP;
};

template <typename T, int NT, int CL, int MODE>
__device__ __forceinline__ void pgc_body(const PgeIO<T>& io, const int bid, uint64_t* s_barp) {
  namespace cg = cooperative_groups;
  using Lay = PgcLayout<T, NT, CL>;
  constexpr int R = Lay::R;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  constexpr int VE = 16 / (int)sizeof(T);  // elements per 16 bytes
  int sys, n, m, ms;
  size_t base;
  pge_system(io, bid, R, sys, base, n, m, ms);
  // dense layout (as pge_kernel's PGE_DENSE): odd partitions, this CTA's
  // rows in order, each staged array shifted by its rows' 16-byte phase
  // (the same in every CTA: a CTA's rows span a multiple of 16 bytes)
  m |= 1;
  ms = m;
  const int rows = NT * m;  // rows per CTA
  const int row0 = rank * rows;
  const int astride = pge_array_elems<T, NT>(ms);
  extern __shared__ __align__(16) unsigned char pge_smem[];
  T* S0 = reinterpret_cast<T*>(pge_smem);
  auto phase = [&](const T* g) { return (int)((reinterpret_cast<uintptr_t>(g + base + row0) / sizeof(T)) % VE); };
  T* SA = S0 + phase(io.a);
  T* SB = S0 + astride + phase(io.b);
  T* SC = S0 + 2 * astride + phase(io.c);
  T* SD = S0 + 3 * astride + phase(io.d);
  T* SV = S0 + 4 * astride;
  T* SX = SV + astride;
  T* EXT = SX + astride;
  T* FST = EXT + Lay::FST;
  T* XF = EXT + Lay::XF;
  T* RED = EXT + Lay::RED;
  T* SOL = EXT + Lay::SOL;
  T* XCH = EXT + Lay::XCH;
  T* TOP = EXT + Lay::TOP;
  T* TSOL = EXT + Lay::TSOL;
  T* TMP = EXT + Lay::TMP;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int P = rank * NT + t;
  const T* __restrict__ ga = io.a;
  const T* __restrict__ gb = io.b;
  const T* __restrict__ gc = io.c;
  const T* gd = io.d;
  int* info = io.info;
  using MagT = unsigned;
  // Cluster-wide maxima and flags: every CTA accumulates into its own
  // shared variables (CTA-local atomics), and after a cluster barrier the
  // threads combine the CL values with plain distributed-shared-memory loads.
  // (Atomics on another CTA's shared memory through map_shared_rank lost
  // updates here: the maxima they produced depended on timing.)
  __shared__ MagT s_amax, s_dmax, s_xmax;
  __shared__ unsigned long long s_rmax, s_anorm, s_xn, s_dn;
  __shared__ int s_bad, s_nf;
  auto cl_max = [&](auto& v) {
    auto m = v;
#pragma unroll
    for (int r = 0; r < CL; ++r) {
      const auto w = *cluster.map_shared_rank(&v, r);
      m = w > m ? w : m;
    }
    return m;
  };
  T* RED0 = cluster.map_shared_rank(RED, 0);
  T* SOL0 = cluster.map_shared_rank(SOL, 0);
  if (t == 0) {
    s_amax = 0;
    s_dmax = 0;
    s_xmax = 0;
    s_rmax = s_anorm = s_xn = s_dn = 0ull;
    s_bad = 0;
    s_nf = 0;
  }
  auto sidx = [&](int lr) { return (lr / m) * ms + (lr % m); };  // local row -> staging index

  // ---- stage this CTA's rows (local rows [0, hi) inside the system): one
  // bulk copy per array of its 16-byte aligned rows [r0, r1), the rest and
  // the identity rows past n by plain copies; the system's row 0 of a and
  // row n-1 of c stay out of the bulk ranges (zero, and outside the arrays
  // for the adjoint's shifted pointers)
  const int hi = max(0, min(rows, n - row0));
  uint64_t& s_bar = *s_barp;
  {
    T* const Sk[4] = {SA, SB, SC, SD};
    const T* const Gk[4] = {ga, gb, gc, gd};
    int r0[4], r1[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      r0[k] = min(hi, (VE - phase(Gk[k])) % VE);
      r1[k] = r0[k] + (hi - r0[k]) / VE * VE;
    }
    if (row0 == 0 && r0[0] == 0) r0[0] = min(VE, r1[0]);
    if (row0 + r1[2] == n && r1[2] > r0[2]) r1[2] -= VE;
    if (t == 0) {
      mbar_init(&s_bar, 1);
      fence_mbar_init();
      unsigned total = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) total += (unsigned)((r1[k] - r0[k]) * sizeof(T));
      mbar_arrive_expect_tx(&s_bar, total);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (r1[k] > r0[k])
          bulk_load_1d(Sk[k] + r0[k], Gk[k] + base + row0 + r0[k], (unsigned)((r1[k] - r0[k]) * sizeof(T)), &s_bar);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      auto plain = [&](int lr) {
        const int r = row0 + lr;
        Sk[k][lr] = (k == 0 && r == 0) || (k == 2 && r == n - 1) ? T(0) : Gk[k][base + r];
      };
      if (t < r0[k]) plain(t);
      if (t < hi - r1[k]) plain(r1[k] + t);
      for (int lr = hi + t; lr < rows; lr += NT) Sk[k][lr] = k == 1 ? T(1) : T(0);
    }
    __syncthreads();  // (the mbarrier's initialisation, before anyone waits)
    if (!mbar_wait(&s_bar, 0, io.err) && t == 0) {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        for (int lr = r0[k]; lr < r1[k]; ++lr) Sk[k][lr] = k == 1 ? T(1) : T(0);
    }
  }
  cluster.sync();  // staging done everywhere, every CTA's accumulators initialised
  MagT amax = 0, dmax = 0;

  const int mi = m - 1;
  T* A = SA + t * ms;
  T* B = SB + t * ms;
  T* C = SC + t * ms;
  T* D = SD + t * ms;
  T* V = SV + t * ms;
  bool accepted = false;
#pragma unroll 1
  for (int pass = 0; pass <= PGE_REFINE_CL; ++pass) {
    // ---- forward elimination of the partition (as pge_kernel)
    bool bad = false;
    unsigned long long swaps = 0ull;
    T cb = B[0], cc = mi > 1 ? C[0] : T(0), cy = D[0], cv = A[0], cw = mi == 1 ? C[0] : T(0);
    amax = max(amax, max(magh(cv), max(magh(cb), magh(C[0]))));  // magnitudes for the acceptance test
    dmax = max(dmax, magh(cy));
    T w_prev = T(0);
    T om1 = T(0), om2 = T(0);
    T kro = T(1);
    T pu1 = T(0), pu2a = T(0), pu2b = T(0);
    T Y0 = T(0), V0 = T(0);
    // software-pipelined: row i+2 (at most the separator row, which always
    // exists) is loaded while row i+1 is eliminated
    // (the last interior row, i = mi-2, is peeled off the loop by the
    // compile-time tag: as a run-time test the right spike's product was
    // formed on every row)
    T pa = A[1], pb = B[1], pc = C[1], py = D[1];
    auto elim_row = [&](int i, auto last_tag) {
      constexpr bool last = decltype(last_tag)::value;
      const T na = pa, nb = pb, cn = pc, ny = py;
      amax = max(amax, max(magh(na), max(magh(nb), magh(cn))));
      dmax = max(dmax, magh(ny));
      pa = A[i + 2];
      pb = B[i + 2];
      pc = C[i + 2];
      py = D[i + 2];
      const T nc = last ? T(0) : cn;
      const bool sw = !abs_ge(cb, na);
      const T piv = sw ? na : cb;
      bad |= is_zero(piv);
      const T inv = Div<T>(piv).inv();
      const T l = (sw ? cb : na) * inv;
      const T u1 = sw ? nb : cc;
      const T u2 = keep_if(sw, nc);
      const T uy = sw ? ny : cy;
      const T uv = keep_if(!sw, cv);
      const T om = fma(-om2, pu2b, fma(-om1, pu1, kro)) * inv;
      kro = T(0);
      Y0 = fma(om, uy, Y0);
      V0 = fma(om, uv, V0);
      om2 = om1;
      om1 = om;
      pu2b = pu2a;
      pu2a = u2;
      pu1 = u1;
      A[i] = inv;
      B[i] = u1;
      D[i] = uy;
      V[i] = uv;
      swaps |= (unsigned long long)sw << i;
      cb = fma(-l, u1, sw ? cc : nb);
      // the row left behind keeps one of c_{i+2} (no swap) and the left spike
      // (swap); the other is scaled by -l: one product for both
      const T tq = -l * (sw ? nc : cv);
      cc = sw ? tq : nc;
      cy = fma(-l, uy, sw ? cy : ny);
      cv = sw ? cv : tq;
      if constexpr (last) {
        w_prev = sw ? cn : cw;
        cw = fma(-l, w_prev, sw ? cw : cn);
      }
    };
    for (int i = 0; i + 2 < mi; ++i) elim_row(i, std::false_type{});
    if (mi >= 2) elim_row(mi - 2, std::true_type{});
    bad |= is_zero(cb);
    const T inv_last = Div<T>(cb).inv();
    {
      const T om = fma(-om2, pu2b, fma(-om1, pu1, kro)) * inv_last;
      Y0 = fma(om, cy, Y0);
      V0 = fma(om, cv, V0);
      FST[t] = Y0;
      FST[NT + t] = V0;
      FST[2 * NT + t] = fma(om1, w_prev, om * cw);
    }
    const T Ylast = cy * inv_last, Vlast = cv * inv_last, Wlast = cw * inv_last;
    A[mi - 1] = inv_last;
    B[mi - 1] = T(0);
    D[mi - 1] = cy;
    V[mi - 1] = cv;
    cluster.sync();

    // ---- separator row of partition P, into CTA 0's gather buffer
    const T as = A[mi], bs = B[mi], cs = C[mi], ds = D[mi];
    amax = max(amax, max(magh(as), max(magh(bs), magh(cs))));
    dmax = max(dmax, magh(ds));
    if (pass == 0) {
      atomicMax(&s_amax, amax);
      atomicMax(&s_dmax, dmax);
    }
    {
      T Yf = T(0), Vf = T(0), Wf = T(0);
      if (t + 1 < NT) {
        Yf = FST[t + 1];
        Vf = FST[NT + t + 1];
        Wf = FST[2 * NT + t + 1];
      } else if (rank + 1 < CL) {
        const T* nf = cluster.map_shared_rank(FST, rank + 1);
        Yf = nf[0];
        Vf = nf[NT];
        Wf = nf[2 * NT];
      }
      RED0[P] = -as * Vlast;
      RED0[R + P] = fma(-cs, Vf, fma(-as, Wlast, bs));
      RED0[2 * R + P] = -cs * Wf;
      RED0[3 * R + P] = fma(-cs, Yf, fma(-as, Ylast, ds));
    }
    cluster.sync();

    // ---- CTA 0: the R-row separator system with partial pivoting, in two
    // levels (chunks of CL rows per thread, then warp 0 on the NT tops)
    if (rank == 0) {
      T a_[CL], b_[CL], c_[CL], d_[CL];
#pragma unroll
      for (int k = 0; k < CL; ++k) {
        a_[k] = RED[t * CL + k];
        b_[k] = RED[R + t * CL + k];
        c_[k] = RED[2 * R + t * CL + k];
        d_[k] = RED[3 * R + t * CL + k];
      }
      ChunkSpikes<T, CL> ch;
      bool rbad = ch.eliminate(a_, b_, c_, d_);
      XCH[t] = ch.Y[0];
      XCH[NT + t] = ch.V[0];
      XCH[2 * NT + t] = ch.W[0];
      __syncthreads();
      const bool has_next = t + 1 < NT;
      ch.top_row(has_next ? XCH[t + 1] : T(0), has_next ? XCH[NT + t + 1] : T(0),
                 has_next ? XCH[2 * NT + t + 1] : T(0), has_next, TOP[t], TOP[NT + t], TOP[2 * NT + t],
                 TOP[3 * NT + t]);
      __syncthreads();
      if (warp == 0) rbad |= sep_solve_pivoted<T, NT>(TOP, TSOL, TMP, lane);
      __syncthreads();
      const T sp = t > 0 ? TSOL[t - 1] : T(0), st = TSOL[t];
#pragma unroll
      for (int k = 0; k < CL - 1; ++k) SOL[t * CL + k] = ch.value(k, sp, st);
      SOL[t * CL + CL - 1] = st;
      if (rbad) atomicOr(&s_bad, 1);
    }
    cluster.sync();

    // ---- back substitution with the separators in place (as pge_kernel)
    const T sp = P > 0 ? SOL0[P - 1] : T(0);
    const T st = SOL0[P];
    MagT xmax = magh(st);
    T x_last;
    {
      T x1 = (fma(-cw, st, fma(-V[mi - 1], sp, D[mi - 1]))) * inv_last;
      T x2 = T(0);
      D[mi - 1] = x1;
      xmax = max(xmax, magh(x1));
      bad |= !finite_val(x1);
      x_last = x1;
      // software-pipelined: row i-1's factors are loaded while row i is solved
      int j = mi - 2 >= 0 ? mi - 2 : 0;
      T qv = V[j], qd = D[j], qb = B[j], qa = A[j], qc = C[j + 1];
      // (row mi-2, the one row with a right-spike term, peeled off the loop)
      auto back_row = [&](int i, auto spike_tag) {
        const T vi = qv, di = qd, bi = qb, ai = qa, ci1 = qc;
        j = i > 0 ? i - 1 : 0;
        qv = V[j];
        qd = D[j];
        qb = B[j];
        qa = A[j];
        qc = C[j + 1];
        const T u2 = keep_if(((swaps >> i) & 1ull) && i + 2 < mi, ci1);
        T r = fma(-vi, sp, di);
        if constexpr (decltype(spike_tag)::value) r = fma(-w_prev, st, r);
        const T xi = fma(-bi, x1, fma(-u2, x2, r)) * ai;  // x_{i+2} term first: two ops depend on x_{i+1}
        D[i] = xi;
        xmax = max(xmax, magh(xi));
        bad |= !finite_val(xi);
        x2 = x1;
        x1 = xi;
      };
      if (mi >= 2) back_row(mi - 2, std::true_type{});
      for (int i = mi - 3; i >= 0; --i) back_row(i, std::false_type{});
      bad |= !finite_val(st);
      D[mi] = st;
      XF[t] = D[0];
      if (pass == 0) atomicMax(&s_xmax, xmax);
    }
    cluster.sync();
    {
      T x_next = T(0);
      if (t + 1 < NT) x_next = XF[t + 1];
      else if (rank + 1 < CL) x_next = cluster.map_shared_rank(XF, rank + 1)[0];
      const double r = fma(-(double)cs, (double)x_next,
                           fma(-(double)bs, (double)st, fma(-(double)as, (double)x_last, (double)ds)));
      const T amx = Fmt<T>::from_mag(cl_max(s_amax)), xmx = Fmt<T>::from_mag(cl_max(s_xmax)),
              dmx = Fmt<T>::from_mag(cl_max(s_dmax));
      if (pass == 0) bad |= !(fabs(r) <= Fmt<T>::SEP_TOL * fma((double)amx, (double)xmx, (double)dmx));
    }
    if (__syncthreads_or(bad) && t == 0) s_bad = 1;
    cluster.sync();
    const bool pass_bad = cl_max(s_bad) != 0;
    cluster.sync();  // everyone has read the flags
    if (t == 0) s_bad = 0;
    if (pass == 0 && !pass_bad) {
      accepted = true;
      break;
    }
    if (rank == 0 && t == 0) atomicAdd(&g_pge_paths[pass == 0 ? 1 : 2], 1ull);
    // x of a neighbouring row that may live in another CTA (staging array `arr`)
    auto xat = [&](const T* arr, int r) -> T {
      const int lr = r - row0;
      if (lr >= 0 && lr < rows) return arr[sidx(lr)];
      const int rk = r / rows;
      return cluster.map_shared_rank(arr, rk)[sidx(r - rk * rows)];
    };
    if (pass > 0 && !pass_bad) {
      for (int r = t; r < rows; r += NT)
        if (row0 + r < n) SD[sidx(r)] += SX[sidx(r)];
      cluster.sync();
    }
    if (pass_bad && pass > 0) break;  // a correction pass broke down
    // exact normwise backward error of the current x (cluster-wide maxima)
    {
      unsigned long long rmax = 0ull, anorm = 0ull, xn = 0ull, dn = 0ull;
      bool nonfinite = false;
      for (int lr = t; lr < rows; lr += NT) {
        const int r = row0 + lr;
        if (r >= n) break;
        const double ar = r > 0 ? (double)ga[base + r] : 0.0, br = (double)gb[base + r];
        const double cr = r < n - 1 ? (double)gc[base + r] : 0.0, dr = (double)gd[base + r];
        const double xr = (double)SD[sidx(lr)];
        double res = fma(-br, xr, dr);
        if (r > 0) res = fma(-ar, (double)xat(SD, r - 1), res);
        if (r < n - 1) res = fma(-cr, (double)xat(SD, r + 1), res);
        nonfinite |= !finite_val(res);
        rmax = max(rmax, mag(res));
        anorm = max(anorm, mag(fabs(ar) + fabs(br) + fabs(cr)));
        xn = max(xn, mag(xr));
        dn = max(dn, mag(dr));
      }
      atomicMax(&s_rmax, rmax);
      atomicMax(&s_anorm, anorm);
      atomicMax(&s_xn, xn);
      atomicMax(&s_dn, dn);
      if (nonfinite) s_nf = 1;
      cluster.sync();
      const double eta = __longlong_as_double((long long)cl_max(s_rmax)) /
                         fma(__longlong_as_double((long long)cl_max(s_anorm)),
                             __longlong_as_double((long long)cl_max(s_xn)), __longlong_as_double((long long)cl_max(s_dn)));
      const bool ok = cl_max(s_nf) == 0 && eta <= Fmt<T>::SEP_TOL;
      cluster.sync();  // everyone has read the accumulators
      if (t == 0) {
        s_rmax = s_anorm = s_xn = s_dn = 0ull;
        s_nf = 0;
      }
      if (ok) {
        accepted = true;
        break;
      }
    }
    if (pass == PGE_REFINE_CL) break;
    // keep x in SX; the FP64 residual becomes the next right-hand side
    for (int lr = t; lr < rows; lr += NT)
      if (row0 + lr < n) SX[sidx(lr)] = SD[sidx(lr)];
    cluster.sync();
    for (int lr = t; lr < rows; lr += NT) {
      const int r = row0 + lr;
      const int q = sidx(lr);
      if (r < n) {
        const T ar = r > 0 ? ga[base + r] : T(0), br = gb[base + r], cr = r < n - 1 ? gc[base + r] : T(0);
        double res = fma(-(double)br, (double)SX[q], (double)gd[base + r]);
        if (r > 0) res = fma(-(double)ar, (double)xat(SX, r - 1), res);
        if (r < n - 1) res = fma(-(double)cr, (double)xat(SX, r + 1), res);
        SA[q] = ar;
        SB[q] = br;
        SC[q] = cr;
        SD[q] = (T)res;
      } else {
        SA[q] = T(0);
        SB[q] = T(1);
        SC[q] = T(0);
        SD[q] = T(0);
      }
    }
    cluster.sync();
  }  // passes
  if (info && rank == 0 && t == 0) info[sys] = accepted ? 0 : n + 1;
  if (!accepted && rank == 0 && t == 0) atomicAdd(&g_pge_fallbacks, 1ull);
  if (MODE == 0 && phase(io.x) == phase(io.d)) {
    // this CTA's rows of x: the 16-byte aligned ones by one bulk store (x in
    // the same phase as d), the rest element-wise
    const int q0 = min(hi, (VE - phase(io.d)) % VE), q1 = q0 + (hi - q0) / VE * VE;
    fence_async_smem();
    __syncthreads();
    if (t == 0 && q1 > q0) {
      bulk_store_1d(io.x + base + row0 + q0, SD + q0, (unsigned)((q1 - q0) * sizeof(T)));
      bulk_commit();
    }
    if (t < q0) io.x[base + row0 + t] = SD[t];
    if (t < hi - q1) io.x[base + row0 + q1 + t] = SD[q1 + t];
    if (t == 0 && q1 > q0) bulk_wait_read<0>();
  } else {
    pge_store_rows<T, MODE>(io, base, n, row0, row0 + hi, t, NT, [&](int r) { return SD[r - row0]; });
  }
  cluster.sync();  // no CTA leaves while others may still read its shared memory
}

// L2 prefetch of CTA `rank`'s rows of bucket entry k (the system a resident
// cluster solves next): the four arrays' rows [row0 + 1, row0 + rows - 1)
// within the system -- a row dropped at each end and the range aligned
// inward to 16 bytes, so that it stays inside the arrays for the adjoint's
// shifted a and c as well.
template <typename T, int NT, int CL>
__device__ __forceinline__ void pgc_prefetch(const PgeIO<T>& io, int k, int rank) {
  int sys, n, m, ms;
  size_t base;
  pge_system(io, k, CL * NT, sys, base, n, m, ms);
  m |= 1;
  const int row0 = rank * NT * m;
  const int lo = row0 + 1, hi = min(n, row0 + NT * m) - 1;
  if (hi <= lo) return;
  const T* arr[4] = {io.a, io.b, io.c, io.d};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uintptr_t s = (reinterpret_cast<uintptr_t>(arr[q] + base + lo) + 15) & ~uintptr_t(15);
    const uintptr_t e = reinterpret_cast<uintptr_t>(arr[q] + base + hi) & ~uintptr_t(15);
    if (e > s)
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(s), "r"((unsigned)(e - s)) : "memory");
  }
}

// TICKET: resident clusters drain one size bucket of a ragged batch (CTA 0
// of the cluster takes the ticket, the others read it through distributed
// shared memory); a separate instance, so the one-cluster-per-system kernel
// keeps its register allocation.  Each cluster holds its next ticket while
// it solves the current system, and every CTA prefetches its rows of that
// next system into L2, so that the next staging reads L2 instead of HBM.
template <typename T, int NT, int CL, int MODE, bool TICKET = false>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NT, 1) pgc_kernel(const PgeIO<T> io) {
  __shared__ __align__(8) uint64_t s_bar;
  if constexpr (!TICKET) {
    pgc_body<T, NT, CL, MODE>(io, blockIdx.x / CL, &s_bar);
  } else {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ int s_item;
    const int rank = (int)cluster.block_rank();
    auto take = [&]() {  // the next ticket, -1 past the bucket's end
      if (rank == 0 && threadIdx.x == 0) {
        const int k = atomicAdd(io.ticket, 1);
        const int cnt = io.dcount ? *(volatile const int*)io.dcount : io.count;
        s_item = k < cnt && (!io.err || *(volatile int*)io.err == 0) ? k : -1;
      }
      cluster.sync();
      const int k = *cluster.map_shared_rank(&s_item, 0);
      cluster.sync();  // (read by all before CTA 0 writes the next one)
      return k;
    };
    auto wanted = [&](int k) {
      return !(io.kinds && io.kinds[io.list[k]] != io.want) && !(io.only && !io.only[io.list[k]]);
    };
    int k = take();
    while (k >= 0) {
      const int kn = take();
      if (kn >= 0 && threadIdx.x == 0 && wanted(kn)) pgc_prefetch<T, NT, CL>(io, kn, rank);
      if (wanted(k)) {
        pgc_body<T, NT, CL, MODE>(io, k, &s_bar);  // (ends with a cluster barrier)
        if (threadIdx.x == 0) mbar_inval(&s_bar);   // re-armed by the next system
      }
      k = kn;
    }
  }
}

template <typename T, int NT>
static size_t pge_smem_bytes(int ms) {
  return ((size_t)5 * pge_array_elems<T, NT>(ms) + 15 * (size_t)NT + PGE_TMP) * sizeof(T);
}

constexpr size_t PGE_SMEM_MAX = 227 * 1024 - 128;  // dynamic + the kernels' few static bytes

// Largest rows-per-partition m for which a variant's shared memory fits.
template <typename T, int NT>
static int pge_mmax() {
  int m = 2;
  while (m + 1 <= 64 && pge_smem_bytes<T, NT>((m + 1) | 1) <= PGE_SMEM_MAX) ++m;
  return pge_smem_bytes<T, NT>(m | 1) <= PGE_SMEM_MAX ? m : 0;
}

template <typename T, int NT, int CL>
static size_t pgc_smem_bytes(int ms) {
  return ((size_t)6 * pge_array_elems<T, NT>(ms) + PgcLayout<T, NT, CL>::END) * sizeof(T);
}

template <typename T, int NT, int CL>
static int pgc_mmax() {
  int m = 2;
  while (m + 1 <= 64 && pgc_smem_bytes<T, NT, CL>((m + 1) | 1) <= PGE_SMEM_MAX) ++m;
  return pgc_smem_bytes<T, NT, CL>(m | 1) <= PGE_SMEM_MAX ? m : 0;
}

// Variants: 0 = none, 1/2/3 = one CTA with 64/128/256 partitions,
// 4/5/6 = a cluster of 2/4/8 CTAs with 128 partitions each
// (pge_variant_partitions in kernels.h).

template <typename T>
int pge_variant_mmax(int v) {
  switch (v) {
    case 1: return pge_mmax<T, 64>();
    case 2: return pge_mmax<T, 128>();
    case 3: return pge_mmax<T, 256>();
    case 4: return pgc_mmax<T, 128, 2>();
    case 5: return pgc_mmax<T, 128, 4>();
    case 6: return pgc_mmax<T, 128, 8>();
    default: return 0;
  }
}

template <typename T>
int pge_variant_max_n(int v) {
  if (v < 1 || v > 6) return 0;
  return pge_variant_partitions(v) * pge_variant_mmax<T>(v);
}

template <typename T, int NT, int MODE, int LAY>
static cudaError_t pge_launch_k(const PgeIO<T>& io_in, const PgeMaps& maps, int grid, size_t smem, cudaStream_t s) {
  PgeIO<T> io = io_in;
  cudaError_t e =
      cudaFuncSetAttribute(pge_kernel<T, NT, MODE, LAY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if constexpr (LAY == PGE_SWZ) {
    // persistent: io.count systems over as many CTAs as stay resident
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pge_kernel<T, NT, MODE, LAY>, NT, smem);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    io.count = grid;
    io.ring = ring_tickets();
    if (!io.ring || !io.err) return cudaErrorMemoryAllocation;
    grid = std::min(grid, sms * per);
    pge_kernel<T, NT, MODE, LAY><<<grid, NT, smem, s>>>(io, maps);
    return cudaGetLastError();
  }
  // L2 prefetch one wave ahead for uniform batches with 16-byte aligned systems
  const uintptr_t al = reinterpret_cast<uintptr_t>(io.a) | reinterpret_cast<uintptr_t>(io.b) |
                       reinterpret_cast<uintptr_t>(io.c) | reinterpret_cast<uintptr_t>(io.d);
  if (!io.offsets && !io.list && (al & 15u) == 0 && (io.stride * sizeof(T)) % 16 == 0) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pge_kernel<T, NT, MODE, LAY>, NT, smem) == cudaSuccess &&
        per > 0 && grid > sms * per)
      io.pf_ahead = sms * per;
  }
  if (io.ticket) {
    // a ticket-driven bucket: as many CTAs as stay resident at once
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pge_kernel<T, NT, MODE, LAY>, NT, smem) == cudaSuccess &&
        per > 0)
      grid = std::min(grid, sms * per);
  }
  pge_kernel<T, NT, MODE, LAY><<<grid, NT, smem, s>>>(io, maps);
  return cudaGetLastError();
}

template <typename T, int NT, int MODE>
static cudaError_t pge_launch(const PgeIO<T>& io_in, int grid, int m_max, cudaStream_t s) {
  PgeIO<T> io = io_in;
  io.pf_ahead = 0;
  io.err = error_word();
  PgeMaps maps{};
  // TMA staging: FP64 solve of a uniform contiguous batch with 32 rows per
  // partition (n = 32 NT), arrays 16-byte aligned
  if constexpr (MODE == 0 && sizeof(T) == 8) {
    // three half buffers (the ring), the separator rows, first-row values and scratch
    const size_t smem_swz = 1024 + ((size_t)3 * 4 * NT * 16 + 15 * (size_t)NT + PGE_TMP) * sizeof(T);
    if (!io.offsets && !io.list && io.n == PGE_SWZ_M * NT && io.stride == (size_t)io.n && smem_swz <= PGE_SMEM_MAX &&
        (uint64_t)NT * grid < (1ull << 31)) {
      const T* arr[5] = {io.a, io.b, io.c, io.d, io.x};
      bool ok = true;
      for (int k = 0; k < 5 && ok; ++k)
        ok = encode_tmap_3d(&maps.m[k], arr[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, 16, 2, (uint64_t)NT * grid, 128,
                            PGE_SWZ_M * 8, 16, 1, NT, CU_TENSOR_MAP_SWIZZLE_128B);
      if (ok) return pge_launch_k<T, NT, MODE, PGE_SWZ>(io, maps, grid, smem_swz, s);
    }
  }
  // every other shape: each system's rows in order, staged in bulk
  return pge_launch_k<T, NT, MODE, PGE_DENSE>(io, maps, grid, pge_smem_bytes<T, NT>(m_max | 1), s);
}

template <typename T, int NT, int CL, int MODE>
static cudaError_t pgc_launch(const PgeIO<T>& io, int grid, int ms, cudaStream_t s) {
  const size_t smem = pgc_smem_bytes<T, NT, CL>(ms);
  if (io.ticket) {
    // a ticket-driven bucket: as many clusters as stay resident at once
    cudaError_t e = cudaFuncSetAttribute(pgc_kernel<T, NT, CL, MODE, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid * CL);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, pgc_kernel<T, NT, CL, MODE, true>, &cfg) == cudaSuccess && ncl > 0)
      grid = std::min(grid, ncl);
    pgc_kernel<T, NT, CL, MODE, true><<<(unsigned)grid * CL, NT, smem, s>>>(io);
    return cudaGetLastError();
  }
  cudaError_t e =
      cudaFuncSetAttribute(pgc_kernel<T, NT, CL, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  pgc_kernel<T, NT, CL, MODE><<<(unsigned)grid * CL, NT, smem, s>>>(io);
  return cudaGetLastError();
}

// Launch `grid` systems with variant v, shared memory sized for m_max rows
// per partition.
template <typename T, int MODE>
static cudaError_t pge_launch_variant(int v, const PgeIO<T>& io, int grid, int m_max, cudaStream_t s) {
  if (m_max < 2) m_max = 2;
  const int ms = m_max | 1;
  switch (v) {
    case 1: return pge_launch<T, 64, MODE>(io, grid, m_max, s);
    case 2: return pge_launch<T, 128, MODE>(io, grid, m_max, s);
    case 3: return pge_launch<T, 256, MODE>(io, grid, m_max, s);
    case 4: return pgc_launch<T, 128, 2, MODE>(io, grid, ms, s);
    case 5: return pgc_launch<T, 128, 4, MODE>(io, grid, ms, s);
    case 6: return pgc_launch<T, 128, 8, MODE>(io, grid, ms, s);
    default: return cudaErrorInvalidValue;
  }
}

// Default variant for n rows: about 32 rows per partition where one CTA
// holds the system -- 64 partitions up to n = 2048, 128 up to 4096, 256
// beyond (shorter partitions make the log2(NT)-step separator solve the
// larger part of the work; measured on GB300 by the ragged autotuner) --
// else the smallest cluster.  0 when no variant covers n.
template <typename T>
int pge_default_variant(int n) {
  if (n < 65) return 0;
  if (n <= 2048 && n <= pge_variant_max_n<T>(1)) return 1;
  if (n <= 4096 && n <= pge_variant_max_n<T>(2)) return 2;
  if (n <= pge_variant_max_n<T>(3)) return 3;
  if (n <= pge_variant_max_n<T>(2)) return 2;
  for (int v = 4; v <= 6; ++v)
    if (n <= pge_variant_max_n<T>(v)) return v;
  return 0;
}

template <typename T>
bool pge_eligible(int layout, int n) {
  if (layout != CONTIG && layout != PACKED) return false;
  return pge_default_variant<T>(n) != 0;
}

template <typename T>
static PgeIO<T> uniform_io(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n) {
  PgeIO<T> io{};
  io.a = a;
  io.b = b;
  io.c = c;
  io.d = d;
  io.x = x;
  io.info = info;
  io.stride = layout == PACKED ? 4 * (size_t)n : (size_t)n;
  io.n = n;
  return io;
}

template <typename T>
cudaError_t launch_pge(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                       cudaStream_t s, bool* used) {
  *used = false;
  if (!pge_eligible<T>(layout, n)) return cudaSuccess;
  const int v = pge_default_variant<T>(n);
  *used = true;
  const int m = (n + pge_variant_partitions(v) - 1) / pge_variant_partitions(v);
  return pge_launch_variant<T, 0>(v, uniform_io<T>(layout, a, b, c, d, x, info, n), batch, m, s);
}

// ---------------------------------------------------------------------------
// Long systems (uniform contiguous batches beyond the one-CTA and cluster
// sizes): the partitioned solve in chunks of PGE_LONG_NT partitions of
// PGE_LONG_M rows, one CTA per chunk, in four launches --
//   1. pge_kernel MODE 2: each chunk eliminates its partitions (as the
//      one-CTA solve) and writes their separator rows into the system-wide
//      separator system, plus the first-row relation of its first partition
//      and the last separator's c for the link;
//   2. pge_long_link: completes the separator row at each chunk boundary;
//   3. the separator systems (PGE_LONG_NT rows per chunk), solved by the
//      partitioned solve itself (one CTA or a cluster per system);
//   4. pge_kernel MODE 3: each chunk eliminates again, back-substitutes with
//      its separators and checks its separator rows' residuals (as pass 0 of
//      the one-CTA solve, with the chunk's maxima: never a looser bound);
// then x goes to d where every chunk passed, and the systems with a failing
// chunk (a chunk cannot refine on its own) take the sequential
// partial-pivoting solve.
constexpr int PGE_LONG_NT = 128, PGE_LONG_M = 33;

template <typename T>
__global__ void __launch_bounds__(256) pge_long_link(T* sep, const T* carry, int nchunks, int batch) {
  const size_t ptot = (size_t)nchunks * PGE_LONG_NT, bsz = ptot * batch;
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;  // (system, chunk boundary)
  const int nb = nchunks - 1;
  if (nb <= 0 || k >= (long long)batch * nb) return;
  const int j = (int)(k / nb), c = (int)(k % nb);
  const T cs = carry[((size_t)j * nchunks + c) * 4 + 3];  // c of chunk c's last separator row
  const T* f = carry + ((size_t)j * nchunks + c + 1) * 4;  // Y, V, W of chunk c+1's first row
  const size_t q = (size_t)j * ptot + (size_t)(c + 1) * PGE_LONG_NT - 1;
  sep[bsz + q] = fma(-cs, f[1], sep[bsz + q]);
  sep[2 * bsz + q] = -cs * f[2];
  sep[3 * bsz + q] = fma(-cs, f[0], sep[3 * bsz + q]);
}

// x -> d for the systems without a mark; bps blocks per system.
template <typename T>
__global__ void __launch_bounds__(256) pge_long_commit(T* __restrict__ d, const T* __restrict__ x,
                                                       const int* __restrict__ flag, int n, int bps) {
  const int j = (int)(blockIdx.x / bps), k = (int)(blockIdx.x % bps);
  if (flag[j]) return;
  const size_t o = (size_t)j * n;
  for (int i = k * blockDim.x + threadIdx.x; i < n; i += bps * blockDim.x) d[o + i] = x[o + i];
}

template <typename T>
bool pge_long_eligible(int n) {
  if (n <= PGE_LONG_NT * PGE_LONG_M) return false;
  const int nchunks = (n + PGE_LONG_NT * PGE_LONG_M - 1) / (PGE_LONG_NT * PGE_LONG_M);
  return pge_eligible<T>(CONTIG, nchunks * PGE_LONG_NT) &&
         pge_smem_bytes<T, PGE_LONG_NT>(PGE_LONG_M) <= PGE_SMEM_MAX;
}

template <typename T>
cudaError_t launch_pge_long(const T* a, const T* b, const T* c, T* d, int* info, int n, int batch, T* w1, T* w2,
                            unsigned* piv, int* flag, cudaStream_t s, bool* used) {
  *used = false;
  if (!pge_long_eligible<T>(n)) return cudaSuccess;
  const int rows = PGE_LONG_NT * PGE_LONG_M;
  const int nchunks = (n + rows - 1) / rows;
  const size_t ptot = (size_t)nchunks * PGE_LONG_NT, bsz = ptot * batch;
  // w1: the separator systems, their solution and the chunk links (about
  // 0.15 n per system); w2: x until it is committed.  (One CTA per chunk:
  // the grid must stay an int.)
  if (5 * ptot + 4 * (size_t)nchunks > (size_t)n) return cudaSuccess;
  if ((long long)batch * nchunks > 0x7fffffffLL || (long long)batch * 64 > 0x7fffffffLL) return cudaSuccess;
  T* sep = w1;
  T* xsep = w1 + 4 * bsz;
  T* carry = xsep + bsz;
  *used = true;
  PgeIO<T> io{};
  io.a = a;
  io.b = b;
  io.c = c;
  io.d = d;
  io.stride = (size_t)n;
  io.n = n;
  io.err = error_word();
  io.nchunks = nchunks;
  io.chunk_rows = rows;
  io.sep = sep;
  io.carry = carry;
  io.xsep = xsep;
  io.flag = flag;
  io.sep_total = bsz;
  const size_t smem = pge_smem_bytes<T, PGE_LONG_NT>(PGE_LONG_M);
  const PgeMaps maps{};
  const int grid = batch * nchunks;
  cudaError_t e = cudaFuncSetAttribute(pge_kernel<T, PGE_LONG_NT, 2, PGE_DENSE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(pge_kernel<T, PGE_LONG_NT, 3, PGE_DENSE>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  pge_kernel<T, PGE_LONG_NT, 2, PGE_DENSE><<<grid, PGE_LONG_NT, smem, s>>>(io, maps);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (nchunks > 1) {
    const long long links = (long long)batch * (nchunks - 1);
    pge_long_link<T><<<(unsigned)((links + 255) / 256), 256, 0, s>>>(sep, carry, nchunks, batch);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  bool sep_used = false;
  e = launch_pge<T>(CONTIG, sep, sep + bsz, sep + 2 * bsz, sep + 3 * bsz, xsep, nullptr, (int)ptot, batch, s,
                    &sep_used);
  if (e != cudaSuccess) return e;
  if (!sep_used) return cudaErrorInvalidValue;  // (pge_long_eligible checked the size)
  if ((e = cudaMemsetAsync(flag, 0, (size_t)batch * sizeof(int), s)) != cudaSuccess) return e;
  io.x = w2;
  pge_kernel<T, PGE_LONG_NT, 3, PGE_DENSE><<<grid, PGE_LONG_NT, smem, s>>>(io, maps);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int bps = (n + 255) / 256 < 64 ? (n + 255) / 256 : 64;
  pge_long_commit<T><<<(unsigned)((size_t)bps * batch), 256, 0, s>>>(d, w2, flag, n, bps);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // the flagged systems: sequential partial pivoting in place on d (their
  // right-hand side is still there), w1/w2 now free for its factors
  return launch_gtsv_seq_masked<T>(CONTIG, a, b, c, d, w1, w2, piv, info, n, batch, flag, s);
}

// Ragged long systems in chunks (the passes above, per system of a size
// bucket of a ragged batch): C chunk entries (cl_sys, cl_ch) cover every
// system of the bucket's size class, the passes skip the systems with
// kinds[s] != want; separator rows of system s at sep_off[s] (sep_total rows
// per array), the separators' systems solved by the partitioned solve of
// variant sep_variant on their ragged offsets (sep_off, the bucket's list,
// count / *dcount entries, ticket); x is written to x, and flag[s] set where
// a chunk misses its bound (the caller re-solves those).
constexpr int PGE_LONG_ROWS = PGE_LONG_NT * PGE_LONG_M;

template <typename T>
__global__ void __launch_bounds__(256) pge_long_link_ragged(T* sep, const T* carry, const int* cl_sys,
                                                            const int* cl_ch, int C, const long long* offsets,
                                                            const long long* sep_off, size_t sep_total,
                                                            const unsigned char* kinds, int want, const int* only,
                                                            int chunk_rows) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C) return;
  const int sys = cl_sys[k], ch = cl_ch[k];
  if ((kinds && kinds[sys] != want) || (only && !only[sys])) return;
  const int nch = (int)((offsets[sys + 1] - offsets[sys] + chunk_rows - 1) / chunk_rows);
  if (ch + 1 >= nch) return;
  const size_t sq = (size_t)sep_off[sys];
  const T cs = carry[(sq / PGE_LONG_NT + ch) * 4 + 3];  // c of chunk ch's last separator row
  const T* f = carry + (sq / PGE_LONG_NT + ch + 1) * 4;  // Y, V, W of chunk ch+1's first row
  const size_t q = sq + (size_t)(ch + 1) * PGE_LONG_NT - 1;
  sep[sep_total + q] = fma(-cs, f[1], sep[sep_total + q]);
  sep[2 * sep_total + q] = -cs * f[2];
  sep[3 * sep_total + q] = fma(-cs, f[0], sep[3 * sep_total + q]);
}

int pge_long_chunk_rows() { return PGE_LONG_ROWS; }
// the chunks of a re-solve: partitions of 31 rows, so that their boundaries
// fall elsewhere than the first pass's
int pge_long_retry_rows() { return PGE_LONG_NT * 31; }

template <typename T>
int pge_long_ragged_max_n() {
  // the separators' system (PGE_LONG_NT rows per chunk) within one partitioned variant
  int best = 0;
  for (int v = 1; v <= 6; ++v) best = std::max(best, pge_variant_max_n<T>(v));
  const long long n = (long long)(best / PGE_LONG_NT) * (PGE_LONG_NT * 31);  // (the re-solve's chunks are the shorter)
  return pge_smem_bytes<T, PGE_LONG_NT>(PGE_LONG_M) <= PGE_SMEM_MAX ? (int)std::min<long long>(n, 1 << 30) : 0;
}

template <typename T>
cudaError_t launch_pge_long_ragged(const T* a, const T* b, const T* c, const T* d, T* x, const long long* offsets,
                                   const int* cl_sys, const int* cl_ch, int C, const long long* sep_off,
                                   size_t sep_total, T* sep, T* xsep, T* carry, int* flag, int sep_variant,
                                   int sep_m_max, const int* list, int count, const BucketTicket* tk,
                                   cudaStream_t s, int chunk_rows) {
  if (C <= 0 || count <= 0) return cudaSuccess;
  if (chunk_rows <= 0 || chunk_rows % PGE_LONG_NT || (chunk_rows / PGE_LONG_NT) % 2 == 0 ||
      chunk_rows > PGE_LONG_ROWS)
    return cudaErrorInvalidValue;
  PgeIO<T> io{};
  io.a = a;
  io.b = b;
  io.c = c;
  io.d = d;
  io.offsets = offsets;
  io.err = error_word();
  io.chunk_rows = chunk_rows;
  io.sep = sep;
  io.carry = carry;
  io.xsep = xsep;
  io.flag = flag;
  io.only = tk ? tk->only : nullptr;
  io.cl_sys = cl_sys;
  io.cl_ch = cl_ch;
  io.sep_off = sep_off;
  io.sep_total = sep_total;
  io.kinds = tk ? tk->kinds : nullptr;
  io.want = tk ? tk->want : 0;
  const size_t smem = pge_smem_bytes<T, PGE_LONG_NT>(PGE_LONG_M);
  const PgeMaps maps{};
  cudaError_t e = cudaFuncSetAttribute(pge_kernel<T, PGE_LONG_NT, 2, PGE_DENSE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(pge_kernel<T, PGE_LONG_NT, 3, PGE_DENSE>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  pge_kernel<T, PGE_LONG_NT, 2, PGE_DENSE><<<C, PGE_LONG_NT, smem, s>>>(io, maps);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  pge_long_link_ragged<T><<<(C + 255) / 256, 256, 0, s>>>(sep, carry, cl_sys, cl_ch, C, offsets, sep_off, sep_total,
                                                         io.kinds, io.want, io.only, chunk_rows);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  e = launch_pge_ragged<T>(sep_variant, 0, sep, sep + sep_total, sep + 2 * sep_total, sep + 3 * sep_total, xsep,
                           nullptr, nullptr, nullptr, nullptr, nullptr, sep_off, list, count, sep_m_max, s, tk);
  if (e != cudaSuccess) return e;
  io.x = x;
  pge_kernel<T, PGE_LONG_NT, 3, PGE_DENSE><<<C, PGE_LONG_NT, smem, s>>>(io, maps);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pge_strided(const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                               size_t stride, cudaStream_t s, bool* used) {
  *used = false;
  if (!pge_eligible<T>(CONTIG, n) || stride < (size_t)n) return cudaSuccess;
  const int v = pge_default_variant<T>(n);
  *used = true;
  PgeIO<T> io = uniform_io<T>(CONTIG, a, b, c, d, x, info, n);
  io.stride = stride;
  const int m = (n + pge_variant_partitions(v) - 1) / pge_variant_partitions(v);
  return pge_launch_variant<T, 0>(v, io, batch, m, s);
}

template <typename T>
cudaError_t launch_pge_adjoint(int layout, const T* a, const T* b, const T* c, const T* xf, const T* xbar, T* ga,
                               T* gb, T* gc, T* gd, int* info, int n, int batch, cudaStream_t s, bool* used) {
  *used = false;
  if (!pge_eligible<T>(layout, n)) return cudaSuccess;
  const int v = pge_default_variant<T>(n);
  *used = true;
  // A^T: sub-diagonal c_{i-1}, super-diagonal a_{i+1} (the shifted pointers
  // are only dereferenced at rows 1..n-1 and 0..n-2 respectively)
  PgeIO<T> io = uniform_io<T>(layout, c - 1, b, a + 1, xbar, gd, info, n);
  io.xf = xf;
  io.ga = ga;
  io.gb = gb;
  io.gc = gc;
  const int m = (n + pge_variant_partitions(v) - 1) / pge_variant_partitions(v);
  return pge_launch_variant<T, 1>(v, io, batch, m, s);
}

template <typename T>
cudaError_t launch_pge_ragged(int variant, int mode, const T* a, const T* b, const T* c, const T* d, T* x,
                              const T* xf, T* ga, T* gb, T* gc, int* info, const long long* offsets, const int* list,
                              int count, int m_max, cudaStream_t s, const BucketTicket* tk) {
  if (count <= 0) return cudaSuccess;
  PgeIO<T> io{};
  io.err = error_word();
  if (tk && tk->ticket) {
    io.ticket = tk->ticket;
    io.count = count;
    io.dcount = tk->dcount;
    io.kinds = tk->kinds;
    io.want = tk->want;
    io.only = tk->only;
  }
  io.b = b;
  io.d = d;
  io.x = x;
  io.info = info;
  io.offsets = offsets;
  io.list = list;
  if (mode == 0) {
    io.a = a;
    io.c = c;
    return pge_launch_variant<T, 0>(variant, io, count, m_max, s);
  }
  io.a = c - 1;
  io.c = a + 1;
  io.xf = xf;
  io.ga = ga;
  io.gb = gb;
  io.gc = gc;
  return pge_launch_variant<T, 1>(variant, io, count, m_max, s);
}

// The systems list[0 .. *dcount) of a uniform contiguous batch (at most
// `batch` of them), drained by resident CTAs through `ticket` (zero before
// the launch): the fallback of the thread-per-partition solve (ppt.cu).
template <typename T>
cudaError_t launch_pge_list(const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                            const int* list, const int* dcount, int* ticket, cudaStream_t s) {
  const int v = pge_default_variant<T>(n);
  if (v == 0) return cudaErrorInvalidValue;
  PgeIO<T> io{};
  io.err = error_word();
  io.a = a;
  io.b = b;
  io.c = c;
  io.d = d;
  io.x = x;
  io.info = info;
  io.n = n;
  io.stride = (size_t)n;
  io.list = list;
  io.ticket = ticket;
  io.count = batch;
  io.dcount = dcount;
  const int parts = pge_variant_partitions(v);
  return pge_launch_variant<T, 0>(v, io, batch, (n + parts - 1) / parts, s);
}

cudaError_t pge_fallback_count(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_pge_fallbacks, sizeof(*out));
  if (e == cudaSuccess && reset) {
    const unsigned long long zero = 0ull;
    e = cudaMemcpyToSymbol(g_pge_fallbacks, &zero, sizeof(zero));
  }
  return e;
}

cudaError_t pge_path_counts(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_pge_paths, 3 * sizeof(*out));
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(out + 3, g_pge_fallbacks, sizeof(*out));
  if (e == cudaSuccess && reset) {
    const unsigned long long zero[3] = {0ull, 0ull, 0ull};
    e = cudaMemcpyToSymbol(g_pge_paths, zero, sizeof(zero));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_pge_fallbacks, zero, sizeof(zero[0]));
  }
  return e;
}

#define INST(T)                                                                                                   \
  template bool pge_eligible<T>(int, int);                                                                        \
  template int pge_default_variant<T>(int);                                                                       \
  template int pge_variant_max_n<T>(int);                                                                         \
  template int pge_variant_mmax<T>(int);                                                                          \
  template cudaError_t launch_pge<T>(int, const T*, const T*, const T*, const T*, T*, int*, int, int, cudaStream_t, \
                                     bool*);                                                                      \
  template bool pge_long_eligible<T>(int);                                                                        \
  template int pge_long_ragged_max_n<T>();                                                                        \
  template cudaError_t launch_pge_long_ragged<T>(const T*, const T*, const T*, const T*, T*, const long long*,      \
                                                 const int*, const int*, int, const long long*, size_t, T*, T*, T*, \
                                                 int*, int, int, const int*, int, const BucketTicket*, cudaStream_t, \
                                                 int);                                                            \
  template cudaError_t launch_pge_long<T>(const T*, const T*, const T*, T*, int*, int, int, T*, T*, unsigned*, int*, \
                                          cudaStream_t, bool*);                                                   \
  template cudaError_t launch_pge_strided<T>(const T*, const T*, const T*, const T*, T*, int*, int, int, size_t,  \
                                             cudaStream_t, bool*);                                                \
  template cudaError_t launch_pge_adjoint<T>(int, const T*, const T*, const T*, const T*, const T*, T*, T*, T*, T*, \
                                             int*, int, int, cudaStream_t, bool*);                                \
  template cudaError_t launch_pge_ragged<T>(int, int, const T*, const T*, const T*, const T*, T*, const T*, T*, T*, \
                                            T*, int*, const long long*, const int*, int, int, cudaStream_t,       \
                                            const BucketTicket*);                                                 \
  template cudaError_t launch_pge_list<T>(const T*, const T*, const T*, const T*, T*, int*, int, int, const int*,  \
                                          const int*, int*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
