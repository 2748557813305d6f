// WM-pGE: partitioned Gaussian elimination with the reduced interface
// system solved by PCR, one warp per system, everything on chip.
//
// Lane t owns a contiguous chunk of m rows [s, e] in registers (HBM traffic
// is the algorithmic 5n: read a, b, c, d once, write x once).  The last row
// e of every chunk is a separator; the rows [s, e-1] are the chunk's
// interior.  With x_L = x_{s-1} (previous separator) and x_R = x_e:
//   * a bottom-up elimination of the interior gives the first interior row
//     as x_s = y''_s - a''_s x_L + v''_s x_R (needed by lane t-1);
//   * a top-down elimination gives x_i = y'_i + w'_i x_L - c'_i x_{i+1}
//     (kept in registers for the back substitution);
//   * substituting both into separator row e gives one tridiagonal equation
//     per lane in the separators, solved by 5 PCR steps over warp shuffles;
//   * each lane back-substitutes its interior from (x_L, x_R).
// The reduced system inherits diagonal dominance from A, so PCR needs no
// pivoting for the dominant systems this kernel serves.
//
// Reference: the WM-pGE ("Wang-Mou partition + parallel GE") kernels,
// Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:17-884, and their CPU versions
// Tridiagonal_AVX512/tridiagonal_d_avx512.cpp:74-416 (block elimination over
// a partition, cross-block elimination, per-block back sweep).  The reference
// streams 64-row tiles through a warp and spills c', d' to global memory;
// this version keeps the whole system in registers.
#include "common.cuh"
#include "kernels.h"
#include "pcr.cuh"
#include "tw.cuh"

namespace tdg {

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using V = float4;
  static constexpr int N = 4;
  __device__ static __forceinline__ float get(const V& v, int q) {
    return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w;
  }
  template <int M>
  __device__ static __forceinline__ V make(const float (&r)[M], int k) {
    return make_float4(r[k], r[k + 1], r[k + 2], r[k + 3]);
  }
};
template <>
struct Vec16<double> {
  using V = double2;
  static constexpr int N = 2;
  __device__ static __forceinline__ double get(const V& v, int q) { return q == 0 ? v.x : v.y; }
  template <int M>
  __device__ static __forceinline__ V make(const double (&r)[M], int k) {
    return make_double2(r[k], r[k + 1]);
  }
};

// Load rows [s, s+M) of one array into registers (rows outside [s, s+m) get
// `fill`).  With vec, n and m are multiples of the vector width, so a
// chunk's valid length is too and no vector load crosses the end of a
// system.
template <typename T, int M, bool RO>
__device__ __forceinline__ void load_chunk(T (&r)[M], const T* p, int s, int m, bool vec, T fill) {
  using W = Vec16<T>;
  constexpr int NV = W::N;
  if (vec) {
#pragma unroll
    for (int k = 0; k < M; k += NV) {
      if (k < m) {
        const typename W::V* pp = reinterpret_cast<const typename W::V*>(p + s + k);
        const typename W::V v = RO ? __ldg(pp) : *pp;
#pragma unroll
        for (int q = 0; q < NV; ++q) r[k + q] = W::get(v, q);
      } else {
#pragma unroll
        for (int q = 0; q < NV; ++q) r[k + q] = fill;
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < M; ++k) r[k] = k < m ? (RO ? __ldg(p + s + k) : p[s + k]) : fill;
  }
}

template <typename T, int M>
__device__ __forceinline__ void store_chunk(const T (&r)[M], T* p, int s, int m, bool vec) {
  using W = Vec16<T>;
  constexpr int NV = W::N;
  if (vec) {
#pragma unroll
    for (int k = 0; k < M; k += NV)
      if (k < m) *reinterpret_cast<typename W::V*>(p + s + k) = W::make(r, k);
  } else {
#pragma unroll
    for (int k = 0; k < M; ++k)
      if (k < m) p[s + k] = r[k];
  }
}

// PCR over segments of G lanes of a warp (G = 4..32, one system per
// segment): equation alpha x_{t-1} + beta x_t + gamma x_{t+1} = delta per
// lane, t = lane % G; returns x_t.  Each lane shuffles its own 1/beta (formed
// once, by its owner, instead of by each of its two readers: the same value).
template <typename T, int G>
__device__ __forceinline__ T warp_pcr(T al, T be, T ga, T de, int tl) {
#pragma unroll
  for (int s = 1; s < G; s <<= 1) {
    const T ib = Div<T>(be).inv();
    T aL = __shfl_up_sync(FULL, al, s, G), iL = __shfl_up_sync(FULL, ib, s, G);
    T gL = __shfl_up_sync(FULL, ga, s, G), dL = __shfl_up_sync(FULL, de, s, G);
    T aR = __shfl_down_sync(FULL, al, s, G), iR = __shfl_down_sync(FULL, ib, s, G);
    T gR = __shfl_down_sync(FULL, ga, s, G), dR = __shfl_down_sync(FULL, de, s, G);
    if (tl < s) { aL = T(0); iL = T(1); gL = T(0); dL = T(0); }
    if (tl + s >= G) { aR = T(0); iR = T(1); gR = T(0); dR = T(0); }
    const T k1 = al * iL;
    const T k2 = ga * iR;
    const T nb = fma(-k2, aR, fma(-k1, gL, be));
    const T nd = fma(-k2, dR, fma(-k1, dL, de));
    al = -k1 * aL;
    ga = -k2 * gR;
    be = nb;
    de = nd;
  }
  return Div<T>(be).div(de);
}

// The per-lane WM-pGE solve of one system whose chunk (m rows starting at
// row s) is already in registers A, B, C, D; returns x of the chunk in X.
template <typename T, int M, int G>
__device__ __forceinline__ void wm_lane_solve(T (&A)[M], T (&B)[M], T (&C)[M], T (&D)[M], T (&X)[M], int n, int s,
                                              int m, int mt, int lane) {
  if (s == 0) A[0] = T(0);             // a_0 is not part of the system
  const int last = n - 1 - s;          // local index of row n-1 (if in this chunk)
#pragma unroll
  for (int k = 0; k < M; ++k)
    if (k == last) C[k] = T(0);        // c_{n-1} is not part of the system
  const int ni = mt - 1;               // interior rows [0, ni)

  // bottom-up over the interior: first-row coefficients
  T ap = T(0), yp = T(0), vp = T(0);
#pragma unroll
  for (int kk = 0; kk < M - 1; ++kk) {
    const int k = M - 2 - kk;
    if (k < ni) {
      const bool lastrow = (k == ni - 1);
      const T ck = lastrow ? T(0) : C[k];  // coupling to x_R handled by v''
      const Div<T> q(fma(-ck, ap, B[k]));
      const T nap = q.div(A[k]);
      const T nyp = q.div(fma(-ck, yp, D[k]));
      const T nvp = lastrow ? -q.div(C[k]) : -q.div(ck * vp);
      ap = nap;
      yp = nyp;
      vp = nvp;
    }
  }
  // first interior row of this chunk: x_s = yp - ap x_L + vp x_R;
  // an empty interior means the "first interior row" is the separator itself
  const T f_y = ni > 0 ? yp : T(0);
  const T f_a = ni > 0 ? ap : T(0);
  const T f_v = ni > 0 ? vp : T(1);

  // top-down over the interior: c' -> C, y' -> D, w' -> A
  T cp = T(0), yq = T(0), wq = T(0);
#pragma unroll
  for (int k = 0; k < M - 1; ++k) {
    if (k < ni) {
      const T ak = A[k];
      const Div<T> q(fma(-ak, cp, B[k]));
      cp = q.div(C[k]);
      yq = q.div(fma(-ak, yq, D[k]));
      wq = k == 0 ? -q.div(ak) : -q.div(ak * wq);
      C[k] = cp;
      D[k] = yq;
      A[k] = wq;
    }
  }
  // last interior row: x_{e-1} = yq + wq x_L - cp x_R (empty interior: x_{e-1} = x_L)
  const T l_y = ni > 0 ? yq : T(0);
  const T l_w = ni > 0 ? wq : T(1);
  const T l_c = ni > 0 ? cp : T(0);

  // separator row e = s + ni
  T ae = T(0), be = T(1), ce = T(0), de = T(0);
#pragma unroll
  for (int k = 0; k < M; ++k)
    if (k == ni) { ae = A[k]; be = B[k]; ce = C[k]; de = D[k]; }
  const T n_y = __shfl_down_sync(FULL, f_y, 1, G), n_a = __shfl_down_sync(FULL, f_a, 1, G);
  const T n_v = __shfl_down_sync(FULL, f_v, 1, G);
  const bool has_next = (lane < G - 1) && (s + m < n);
  T al, bt, gm, dl;
  if (mt > 0) {
    al = ae * l_w;
    bt = fma(-ae, l_c, be);
    dl = fma(-ae, l_y, de);
    gm = T(0);
    if (has_next) {
      bt = fma(-ce, n_a, bt);
      dl = fma(-ce, n_y, dl);
      gm = ce * n_v;
    }
  } else {
    al = T(0); bt = T(1); gm = T(0); dl = T(0);
  }
  const T xe = warp_pcr<T, G>(al, bt, gm, dl, lane);
  T xL = __shfl_up_sync(FULL, xe, 1, G);
  if (lane == 0) xL = T(0);

  // back substitution: x_e, then interior from the top-down coefficients
  T xn = xe;
#pragma unroll
  for (int kk = 0; kk < M; ++kk) {
    const int k = M - 1 - kk;
    if (k == ni) X[k] = xe;
    if (k < ni) {
      xn = fma(A[k], xL, fma(-C[k], xn, D[k]));
      X[k] = xn;
    }
  }
}

// CR-PCR hybrid on the same chunk layout: the lane's M = 2^k rows are
// reduced by k levels of odd/even cyclic reduction in registers (only the
// first row of a lane needs the previous lane's row, one shuffle per level),
// leaving one row per lane; the G reduced rows are solved by segmented warp
// PCR; the eliminated rows are recovered level by level, each from the
// coefficients it had when it was eliminated (kept in place in A..D).
// Rows past n are identity rows (they decouple: c_{n-1} = 0).
//
// Reference: the cyclic-reduction solvers, CR_kernel
// (Tridiagonal_CUDA/tridiagonal_basic.cu:32-164) and the register-packed
// CR_reg{4,8,16} kernels (Tridiagonal_CUDA/tridiagonal_onchip.cu:218-820):
// registers hold R rows per thread, then a shared CR / PCR tail.
template <typename T, int M, int G>
__device__ __forceinline__ void crpcr_lane_solve(T (&A)[M], T (&B)[M], T (&C)[M], T (&D)[M], T (&X)[M], int n,
                                                 int s, int m, int mt, int tl) {
  static_assert((M & (M - 1)) == 0, "rows per lane must be a power of two");
  // rows of this chunk beyond n (or an empty chunk) become identity rows
#pragma unroll
  for (int k = 0; k < M; ++k) {
    if (k >= mt) { A[k] = T(0); B[k] = T(1); C[k] = T(0); D[k] = T(0); }
  }
  if (s == 0) A[0] = T(0);
  const int last = n - 1 - s;
#pragma unroll
  for (int k = 0; k < M; ++k)
    if (k == last) C[k] = T(0);
  (void)m;
  // forward reduction
#pragma unroll
  for (int st = 1; st < M; st <<= 1) {
    // previous lane's row M - st (its last row surviving to this level)
    T pa = __shfl_up_sync(FULL, A[M - st], 1, G), pb = __shfl_up_sync(FULL, B[M - st], 1, G);
    T pc = __shfl_up_sync(FULL, C[M - st], 1, G), pd = __shfl_up_sync(FULL, D[M - st], 1, G);
    if (tl == 0) { pa = T(0); pb = T(1); pc = T(0); pd = T(0); }
#pragma unroll
    for (int i = 0; i < M; i += 2 * st) {
      const T la = i == 0 ? pa : A[i - st], lb = i == 0 ? pb : B[i - st];
      const T lc = i == 0 ? pc : C[i - st], ld = i == 0 ? pd : D[i - st];
      const T ra = A[i + st], rb = B[i + st], rc = C[i + st], rd = D[i + st];
      const T k1 = A[i] * Div<T>(lb).inv();
      const T k2 = C[i] * Div<T>(rb).inv();
      const T nb = fma(-k2, ra, fma(-k1, lc, B[i]));
      const T nd = fma(-k2, rd, fma(-k1, ld, D[i]));
      A[i] = -k1 * la;
      C[i] = -k2 * rc;
      B[i] = nb;
      D[i] = nd;
    }
  }
  // reduced system: row 0 of every lane, coupled to row 0 of the neighbours
  const T x0 = warp_pcr<T, G>(A[0], B[0], C[0], D[0], tl);
  T xr = __shfl_down_sync(FULL, x0, 1, G);  // x of the next lane's row 0
  if (tl == G - 1) xr = T(0);
  X[0] = x0;
  // back substitution
#pragma unroll
  for (int st = M >> 1; st >= 1; st >>= 1) {
#pragma unroll
    for (int i = st; i < M; i += 2 * st) {
      const T xl = X[i - st];
      const T xrr = (i + st < M) ? X[i + st] : xr;
      X[i] = Div<T>(B[i]).div(fma(-C[i], xrr, fma(-A[i], xl, D[i])));
    }
  }
}

// Per-lane solve selector for the chunk-layout kernels.
enum ChunkAlgo { CHUNK_WM = 0, CHUNK_CRPCR = 1, CHUNK_PCR = 2 };

template <int ALG, typename T, int M, int G>
__device__ __forceinline__ void chunk_solve(T (&A)[M], T (&B)[M], T (&C)[M], T (&D)[M], T (&X)[M], int n, int s,
                                            int m, int mt, int tl) {
  if constexpr (ALG == CHUNK_CRPCR)
    crpcr_lane_solve<T, M, G>(A, B, C, D, X, n, s, m, mt, tl);
  else
    wm_lane_solve<T, M, G>(A, B, C, D, X, n, s, m, mt, tl);
}

// One warp per system, direct (L1-cached) loads; any n with m <= M.
// Layout CONTIG (stride n between systems) or PACKED (stride 4n; the
// caller passes the four array pointers of system 0).
template <int ALG, typename T, int M>
__global__ void __launch_bounds__(128) wm_warp_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                      const T* __restrict__ c, const T* d, T* x, int n, int batch,
                                                      size_t sys_stride, int m, bool vec) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= batch) return;
  const size_t base = (size_t)j * sys_stride;
  const int s = lane * m;
  const int mt = max(0, min(m, n - s));  // rows of this lane's chunk
  T A[M], B[M], C[M], D[M], X[M];
  load_chunk<T, M, true>(A, a + base, s, mt, vec, T(0));
  load_chunk<T, M, true>(B, b + base, s, mt, vec, T(1));
  load_chunk<T, M, true>(C, c + base, s, mt, vec, T(0));
  load_chunk<T, M, false>(D, d + base, s, mt, vec, T(0));
  chunk_solve<ALG, T, M, 32>(A, B, C, D, X, n, s, m, mt, lane);
  store_chunk<T, M>(X, x + base, s, mt, vec);
}

// ---------------------------------------------------------------------------
// Persistent TMA-fed variant for n = G*m (G = 4..32 lanes per system, m rows
// per lane, m*sizeof(T) in {16, 32, 64, 128} bytes).  Each array is viewed
// as a 2-D tensor of G*batch chunk rows of m elements; one box {m, 32} holds
// the 32/G systems of one warp.  The chunk width picks the shared-memory
// swizzle (none / 32B / 64B / 128B) that makes each lane's 16-byte reads of
// its own chunk conflict free.  Every warp runs a ring of WM_SLOTS input
// buffers; a buffer is refilled as soon as its lanes have read it (PCR: once
// its chain transpose, which passes through the buffer, is done), so
// WM_SLOTS-1 loads stay in flight while the warp solves, and x leaves
// through a separate buffer by TMA store (PCR: straight to global memory).
constexpr int WM_SLOTS = 3;

template <typename T, int M>
struct WmSlot {
  alignas(1024) T buf[4][32 * M];
};
template <typename T, int M>
struct WmOut {
  alignas(1024) T buf[32 * M];
};

// FP32 PCR and CR-PCR with 64-byte lane rows instead run 12 warps per SM
// with a two-slot ring: their warps are latency bound (one system after
// another), so more of them beat a deeper ring; the launch bound caps their
// registers at 168, which they fit without spilling (FP64 PCR would spill).
constexpr int WM_WIDE_WARPS = 12;
template <int ALG, typename T, int M>
constexpr bool wm_wide() {
  return (ALG == CHUNK_PCR || ALG == CHUNK_CRPCR) && sizeof(T) == 4 &&
         (sizeof(WmSlot<T, M>) * 2 + sizeof(WmOut<T, M>)) * WM_WIDE_WARPS <= 221184;
}
template <int ALG, typename T, int M>
constexpr int wm_slots() {
  return wm_wide<ALG, T, M>() ? 2 : WM_SLOTS;
}

// warps per CTA: as many as fit their buffers in 210 KB, at most 8 (the
// wide kernels: 12 in 216 KB)
template <int ALG, typename T, int M>
constexpr int wm_warps() {
  return wm_wide<ALG, T, M>() ? WM_WIDE_WARPS
         : (sizeof(WmSlot<T, M>) * WM_SLOTS + sizeof(WmOut<T, M>)) * 8 <= 215040 ? 8
         : (sizeof(WmSlot<T, M>) * WM_SLOTS + sizeof(WmOut<T, M>)) * 4 <= 215040 ? 4 : 2;
}

// byte offset of (chunk row t, 16-byte unit q) under the TMA swizzle whose
// span equals the row width
template <int ROWB>
__device__ __forceinline__ int wm_swz(int t, int q) {
  const int logical = t * ROWB + q * 16;
  constexpr int mask = ROWB >= 128 ? 7 : ROWB == 64 ? 3 : ROWB == 32 ? 1 : 0;
  return logical ^ (((logical >> 7) & mask) << 4);
}

// PCR whole-lane exchange through the warp's output buffer (free while the
// PCR steps run): each lane writes its chunk of one array as 16-byte units at
// the buffer's swizzled offsets, then reads the chunks of lanes lane -/+ ls
// (mod 32).  Any 8 consecutive chunk rows hit 8 distinct bank groups under
// the 64-byte swizzle, so writes and reads are conflict free; 3 Q/NV shared
// accesses per array replace 2 Q shuffles.
template <typename T, int ROWB>
struct WmXch {
  unsigned char* buf;
  template <int Q>
  __device__ __forceinline__ void lanes(const T (&v)[Q], T (&lo)[Q], T (&hi)[Q], int lane, int ls) const {
    using W = Vec16<T>;
    constexpr int NV = W::N;
    static_assert(Q * (int)sizeof(T) == ROWB, "one chunk per buffer row");
#pragma unroll
    for (int u = 0; u < Q / NV; ++u)
      *reinterpret_cast<typename W::V*>(buf + wm_swz<ROWB>(lane, u)) = W::make(v, u * NV);
    __syncwarp();
    const int tl = (lane - ls) & 31, th = (lane + ls) & 31;
#pragma unroll
    for (int u = 0; u < Q / NV; ++u) {
      const typename W::V x = *reinterpret_cast<const typename W::V*>(buf + wm_swz<ROWB>(tl, u));
      const typename W::V y = *reinterpret_cast<const typename W::V*>(buf + wm_swz<ROWB>(th, u));
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        lo[u * NV + k] = W::get(x, k);
        hi[u * NV + k] = W::get(y, k);
      }
    }
    __syncwarp();
  }
};

// PCR-half-pThomas chain phase for 64-byte lane rows (Q = 16 FP32, Q = 8
// FP64), after four PCR steps: row r couples only to r -/+ 16, so chain
// c = r mod 16 (positions p = r div 16, 2Q rows) is a tridiagonal system of
// its own.  Lanes 2c and 2c+1 solve it from both ends: lane 2c eliminates
// positions 0 .. Q-1 top-down, lane 2c+1 positions 2Q-1 .. Q bottom-up (its
// sub- and super-diagonal exchange roles), each leaving one row
//     x_own + e x_partner = f
// of the two middle unknowns; one shuffle and a 2 x 2 solve give both, and
// each lane back-substitutes its half.  Both lanes run the same instructions
// on slots k = 0 .. Q-1 (position k, resp. 2Q-1-k).
//
// The rows reach their lanes through `xch`, four arrays of 32 x 64 bytes
// (the ring slot the system came in, free once its rows are in registers;
// the TMA swizzle): row L of each array holds lane L's Q slots, which it
// reads as 16-byte units (conflict free); lane l's row Q l + q goes to lane
// L = 2 (r & 15) + h, slot k, where h = [p >= Q], k = h ? 2Q-1-p : p.  p is
// the same for all q of a lane and L = L0 + 2q with (L >> 1) & 3 = q & 3, so
// the byte offset is q * 128 + base[q & 3].  a, b, c, d go to arrays 0-3 in
// one round, and each lane reads its sub-/super-diagonal from array 0 or 2
// by its parity.  Then `refill` runs (the slot is free again: the caller
// loads the next box into it).  The a of row 0 and the c of row 32 Q - 1,
// and after four steps A of rows < 16 and C of rows >= 32 Q - 16, are zero,
// so the chains start and end clean.
//
// x goes straight to the system's rows in global memory (xs): for each slot
// the warp writes two runs of 16 consecutive rows.
template <typename T, int Q, typename Refill>
__device__ __forceinline__ void wm_pcr_half(T (&A)[Q], T (&B)[Q], T (&C)[Q], T (&D)[Q], int lane,
                                            unsigned char* xch, T* xs, const Refill& refill) {
  using W = Vec16<T>;
  constexpr int NV = W::N;
  constexpr int ES = (int)sizeof(T);
  static_assert(Q * ES == 64 && Q / NV == 4, "64-byte lane rows");
  const int r0 = Q * lane;
  const int p = r0 >> 4;
  const int h = p >= Q ? 1 : 0;
  const int k = h ? 2 * Q - 1 - p : p;
  const int L0 = 2 * (r0 & 15) + h;
  int base[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) base[j] = L0 * 64 + (((k / NV) ^ j) << 4) + (k % NV) * ES;
  constexpr int AB = 32 * Q * ES;  // bytes per exchanged array
  const int rb = lane * 64, rx = (lane >> 1) & 3;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int o = q * 128 + base[q & 3];
    *reinterpret_cast<T*>(xch + o) = A[q];
    *reinterpret_cast<T*>(xch + AB + o) = B[q];
    *reinterpret_cast<T*>(xch + 2 * AB + o) = C[q];
    *reinterpret_cast<T*>(xch + 3 * AB + o) = D[q];
  }
  __syncwarp();
  T LO[Q], MI[Q], HI[Q], RH[Q];
  const int odd = lane & 1;  // bottom-up lane: c below, a above
  auto read = [&](const unsigned char* src, T (&dst)[Q]) {
#pragma unroll
    for (int u = 0; u < Q / NV; ++u) {
      const typename W::V w = *reinterpret_cast<const typename W::V*>(src + rb + ((u ^ rx) << 4));
#pragma unroll
      for (int i = 0; i < NV; ++i) dst[u * NV + i] = W::get(w, i);
    }
  };
  read(xch + (odd ? 2 : 0) * AB, LO);
  read(xch + (odd ? 0 : 2) * AB, HI);
  read(xch + AB, MI);
  read(xch + 3 * AB, RH);
  // the exchange arrays are free: order these accesses before the async
  // proxy's refill of them
  fence_async_smem();
  __syncwarp();
  refill();
  // elimination towards the middle
  T e = T(0), f = T(0);
#pragma unroll
  for (int s = 0; s < Q; ++s) {
    const Div<T> piv(fma(-LO[s], e, MI[s]));
    e = piv.div(HI[s]);
    f = piv.div(fma(-LO[s], f, RH[s]));
    HI[s] = e;
    RH[s] = f;
  }
  const T pe = __shfl_xor_sync(FULL, e, 1), pf = __shfl_xor_sync(FULL, f, 1);
  T xv = Div<T>(fma(-e, pe, T(1))).div(fma(-e, pf, f));
  RH[Q - 1] = xv;
#pragma unroll
  for (int ss = 1; ss < Q; ++ss) {
    const int s = Q - 1 - ss;
    xv = fma(-HI[s], xv, RH[s]);
    RH[s] = xv;
  }
  // x of slot s: row c + 16 p(s), p(s) = h ? 2Q-1-s : s
  const int c = lane >> 1, hh = lane & 1;
  T* xr = xs + c + hh * 16 * (2 * Q - 1);  // the row of slot 0
  const int step = hh ? -16 : 16;          // rows per slot
#pragma unroll
  for (int s = 0; s < Q; ++s) xr[s * step] = RH[s];
}

template <int ALG, typename T, int M, int G>
__global__ void __launch_bounds__(32 * wm_warps<ALG, T, M>(), 1)
    wm_tma_kernel(const __grid_constant__ TwMaps maps, int n, int nboxes, int* err, T* xout) {
  constexpr int WARPS = wm_warps<ALG, T, M>();
  constexpr int SLOTS = wm_slots<ALG, T, M>();
  using W = Vec16<T>;
  constexpr int NV = W::N;
  constexpr int ROWB = M * (int)sizeof(T);
  constexpr int BYTES = 32 * M * (int)sizeof(T);
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WmSlot<T, M>* slots = reinterpret_cast<WmSlot<T, M>*>(base) + warp * SLOTS;
  WmOut<T, M>* out = reinterpret_cast<WmOut<T, M>*>(base + sizeof(WmSlot<T, M>) * SLOTS * WARPS) + warp;
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + (sizeof(WmSlot<T, M>) * SLOTS + sizeof(WmOut<T, M>)) * WARPS) +
                   warp * SLOTS;
  const int gw = blockIdx.x * WARPS + warp, nw = gridDim.x * WARPS;
  if (lane == 0) {
    for (int q = 0; q < SLOTS; ++q) mbar_init(&bars[q], 1);
    fence_mbar_init();
  }
  __syncwarp();
  auto load = [&](int i, int q) {  // box i of this warp -> slot q
    const int bx = gw + i * nw;
    mbar_arrive_expect_tx(&bars[q], 4 * BYTES);
#pragma unroll
    for (int k = 0; k < 4; ++k) tma_load_2d(slots[q].buf[k], &maps.m[k], 0, bx * 32, &bars[q]);
  };
  const int count = gw < nboxes ? (nboxes - gw + nw - 1) / nw : 0;
  if (lane == 0)
    for (int i = 0; i < count && i < SLOTS; ++i) load(i, i);
  const int tl = lane % G;
  unsigned parity = 0;
  for (int i = 0; i < count; ++i) {
    const int q = i % SLOTS;
    const bool ok = __all_sync(FULL, mbar_wait(&bars[q], (parity >> q) & 1u, err));
    parity ^= 1u << q;
    if (!ok) break;
    T A[M], B[M], C[M], D[M], X[M];
#pragma unroll
    for (int u = 0; u < M / NV; ++u) {
      const int off = wm_swz<ROWB>(lane, u);
      const typename W::V va = *reinterpret_cast<const typename W::V*>(reinterpret_cast<unsigned char*>(slots[q].buf[0]) + off);
      const typename W::V vb = *reinterpret_cast<const typename W::V*>(reinterpret_cast<unsigned char*>(slots[q].buf[1]) + off);
      const typename W::V vc = *reinterpret_cast<const typename W::V*>(reinterpret_cast<unsigned char*>(slots[q].buf[2]) + off);
      const typename W::V vd = *reinterpret_cast<const typename W::V*>(reinterpret_cast<unsigned char*>(slots[q].buf[3]) + off);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        A[u * NV + v] = W::get(va, v);
        B[u * NV + v] = W::get(vb, v);
        C[u * NV + v] = W::get(vc, v);
        D[u * NV + v] = W::get(vd, v);
      }
    }
    __syncwarp();
    // the slot is free again: refill it with the box SLOTS ahead (PCR first
    // uses it for its chain transpose)
    auto refill = [&]() {
      if (lane == 0 && i + SLOTS < count) load(i + SLOTS, q);
    };
    if constexpr (ALG != CHUNK_PCR) refill();
    if constexpr (ALG == CHUNK_PCR) {
      // PCR-half-pThomas (32 lanes per system): four PCR steps on the chunks
      // (a of row 0 and c of the last row are not part of the system), their
      // whole-lane exchanges (FP64) through the warp's second buffer; then
      // the stride-16 chains by lane pairs, transposed through the slot,
      // which is refilled after; x straight to global memory (each warp
      // store two runs of 16 consecutive rows)
      if (lane == 0) A[0] = T(0);
      if (lane == 31) C[M - 1] = T(0);
      unsigned char* ob = reinterpret_cast<unsigned char*>(out->buf);
      pcr_chunk_steps<T, M, 4>(A, B, C, D, lane, WmXch<T, ROWB>{ob});
      wm_pcr_half<T, M>(A, B, C, D, lane, reinterpret_cast<unsigned char*>(slots[q].buf),
                        xout + (size_t)(gw + i * nw) * 32 * M, refill);
    } else {
      chunk_solve<ALG, T, M, G>(A, B, C, D, X, n, tl * M, M, M, tl);
      if (lane == 0) bulk_wait_read<0>();  // previous x store has left the buffer
      __syncwarp();
#pragma unroll
      for (int u = 0; u < M / NV; ++u) {
        const int off = wm_swz<ROWB>(lane, u);
        *reinterpret_cast<typename W::V*>(reinterpret_cast<unsigned char*>(out->buf) + off) = W::make(X, u * NV);
      }
      fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        tma_store_2d(&maps.m[4], 0, (gw + i * nw) * 32, out->buf);
        bulk_commit();
      }
    }
  }
  if (lane == 0) bulk_wait_all();
}

template <int ALG, typename T, int M, int G>
static bool launch_wm_tma_m(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch, cudaStream_t st,
                            cudaError_t* e) {
  constexpr int ROWB = M * (int)sizeof(T);
  constexpr int WARPS = wm_warps<ALG, T, M>();
  constexpr int SLOTS = wm_slots<ALG, T, M>();
  const CUtensorMapSwizzle sw = ROWB == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                : ROWB == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                : ROWB == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                                             : CU_TENSOR_MAP_SWIZZLE_NONE;
  const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const uint64_t rows = (uint64_t)G * batch;  // chunk rows
  TwMaps maps;
  const T* ptrs[5] = {a, b, c, d, x};
  for (int k = 0; k < 5; ++k)
    if (!encode_tmap_2d(&maps.m[k], ptrs[k], dt, sizeof(T), (uint64_t)M, rows, (uint64_t)M * sizeof(T), M, 32, sw))
      return false;
  const int nboxes = (int)((rows + 31) / 32);
  const size_t smem =
      (sizeof(WmSlot<T, M>) * SLOTS + sizeof(WmOut<T, M>)) * WARPS + 8 * SLOTS * WARPS + 1024;
  *e = cudaFuncSetAttribute(wm_tma_kernel<ALG, T, M, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (*e != cudaSuccess) return true;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int need = (nboxes + WARPS - 1) / WARPS;
  const int grid = need < sms ? need : sms;
  wm_tma_kernel<ALG, T, M, G><<<grid, 32 * WARPS, smem, st>>>(maps, n, nboxes, error_word(), x);
  *e = cudaGetLastError();
  return true;
}

template <int ALG, typename T, int M>
static cudaError_t launch_wm_m(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                               size_t stride, int m, cudaStream_t st) {
  constexpr int NV = Vec16<T>::N;
  const bool vec = (m % NV == 0) && (n % NV == 0) && (stride % NV == 0) &&
                   ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c) |
                     reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(x)) %
                        16 ==
                    0);
  const int warps_per_block = 4;
  dim3 grid((batch + warps_per_block - 1) / warps_per_block);
  wm_warp_kernel<ALG, T, M><<<grid, 32 * warps_per_block, 0, st>>>(a, b, c, d, x, n, batch, stride, m, vec);
  return cudaGetLastError();
}

// Chunk length m = ceil(n/32) (at least 2 rows), rounded up to the vector
// width when that keeps all 32 chunks within n; the template M is the
// smallest supported bound >= m.
template <int ALG, typename T>
static cudaError_t launch_chunk(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                                cudaStream_t st, bool* used) {
  *used = false;
  if (layout != CONTIG && layout != PACKED) return cudaSuccess;
  constexpr int NV = Vec16<T>::N;
  // whole-system TMA boxes: CONTIG, n = G*m with 16 rows per lane preferred
  // (FP64: 8), G in {4, 8, 16, 32}; x may alias d (each warp reads a box
  // completely before its x leaves)
  if (layout == CONTIG) {
    cudaError_t e = cudaSuccess;
    bool done = false;
    constexpr int MP = sizeof(T) == 4 ? 16 : 8;  // preferred rows per lane
    if (n == 4 * MP) done = launch_wm_tma_m<ALG, T, MP, 4>(a, b, c, d, x, n, batch, st, &e);
    else if (n == 8 * MP) done = launch_wm_tma_m<ALG, T, MP, 8>(a, b, c, d, x, n, batch, st, &e);
    else if (n == 16 * MP) done = launch_wm_tma_m<ALG, T, MP, 16>(a, b, c, d, x, n, batch, st, &e);
    else if (n == 32 * MP) done = launch_wm_tma_m<ALG, T, MP, 32>(a, b, c, d, x, n, batch, st, &e);
    else if (n == 64 * MP) done = launch_wm_tma_m<ALG, T, 2 * MP, 32>(a, b, c, d, x, n, batch, st, &e);
    if (done) {
      *used = true;
      return e;
    }
  }
  int m = (n + 31) / 32;
  if (m < 2) m = 2;
  const size_t stride = layout == PACKED ? 4 * (size_t)n : (size_t)n;
  const int maxm = sizeof(T) == 4 ? 32 : 16;
  if (n % NV == 0 && ((m + NV - 1) / NV) * NV <= maxm) m = ((m + NV - 1) / NV) * NV;
  if (m > maxm) return cudaSuccess;
  *used = true;
  if (m <= 4) return launch_wm_m<ALG, T, 4>(a, b, c, d, x, n, batch, stride, 4 > m && ALG == CHUNK_CRPCR ? 4 : m, st);
  if (m <= 8) return launch_wm_m<ALG, T, 8>(a, b, c, d, x, n, batch, stride, ALG == CHUNK_CRPCR ? 8 : m, st);
  if (m <= 16) return launch_wm_m<ALG, T, 16>(a, b, c, d, x, n, batch, stride, ALG == CHUNK_CRPCR ? 16 : m, st);
  if constexpr (sizeof(T) == 4)
    return launch_wm_m<ALG, T, 32>(a, b, c, d, x, n, batch, stride, ALG == CHUNK_CRPCR ? 32 : m, st);
  *used = false;
  return cudaSuccess;
}

// PCR for n = 32 * 16 (FP32) / 32 * 8 (FP64), contiguous layout, on the
// persistent TMA-fed kernel (the half variant: four PCR steps, lane-pair
// chains); other shapes: pcr.cu.
template <typename T>
cudaError_t launch_pcr_tma(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                           cudaStream_t st, bool* used) {
  *used = false;
  constexpr int MP = sizeof(T) == 4 ? 16 : 8;
  if (layout != CONTIG || n != 32 * MP) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  if (launch_wm_tma_m<CHUNK_PCR, T, MP, 32>(a, b, c, d, x, n, batch, st, &e)) *used = true;
  return e;
}

template <typename T>
cudaError_t launch_wm_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                           cudaStream_t st, bool* used) {
  return launch_chunk<CHUNK_WM, T>(layout, a, b, c, d, x, n, batch, st, used);
}
template <typename T>
cudaError_t launch_crpcr_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                              cudaStream_t st, bool* used) {
  return launch_chunk<CHUNK_CRPCR, T>(layout, a, b, c, d, x, n, batch, st, used);
}

#define INST(T)                                                                                                   \
  template cudaError_t launch_pcr_tma<T>(int, const T*, const T*, const T*, const T*, T*, int, int, cudaStream_t, \
                                         bool*);                                                                  \
  template cudaError_t launch_wm_warp<T>(int, const T*, const T*, const T*, const T*, T*, int, int, cudaStream_t, \
                                         bool*);                                                                  \
  template cudaError_t launch_crpcr_warp<T>(int, const T*, const T*, const T*, const T*, T*, int, int,            \
                                            cudaStream_t, bool*);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
