// Partitioned solve without pivoting, one CTA per system (contiguous and
// packed layouts): the partition method of the reference's WM-pGE
// (Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:17-884 partitions each system and
// eliminates without pivoting) reorganised for a whole system per CTA.
//
// Shape: each thread owns one 128-byte row of the system, i.e. M = 32 (FP32)
// or 16 (FP64) consecutive equations; n = R * M with R threads (R <= 256).
// The four arrays arrive by TMA (one 2-D box of R x 128 bytes each, 128-byte
// swizzle), so thread t's 16-byte units sit at t*128 + ((q ^ (t & 7)) * 16):
// the eight threads of a quarter warp reading unit q hit eight different
// 16-byte bank groups, and every shared-memory access is a conflict-free
// vector access.
//
// Per partition (rows s .. s+M-1 of thread t), the last row is the
// partition's separator y_t; the interior rows are eliminated top-down
// without pivoting, each expressed as
//     x_k = d'_k - c'_k x_{k+1} - v_k y_{t-1}
// (v carries the coupling a_s y_{t-1} of the first row), while the same
// sweep carries the first row's relation x_s = G + P x_{k+1} - L y_{t-1}
// (P is the running product of -c').  At the last interior row x_{k+1} is
// y_t, so each separator row gives one row of a tridiagonal system in
// y_0 .. y_{R-1}:
//     -a_r v_L y_{t-1} + (b_r - a_r c'_L - c_r L') y_t + c_r P' y_{t+1}
//         = d_r - a_r d'_L - c_r G'
// (primes: the next partition's first-row relation).  That system is solved
// by parallel cyclic reduction across the CTA, then every thread substitutes
// back bottom-up.  Stability: that of elimination without pivoting, i.e.
// the contract of Thomas, CR and PCR -- diagonally dominant (or otherwise
// pivoting-free) systems; the pivoted solves are tridiag_gtsv_* and
// TRIDIAG_ALGO_GTSV / PGE.
//
// Shared-memory passes: read a, b, c, d and write v, c', d' over a, b, d
// (top-down), read v, c', d' and write x over d (bottom-up); x leaves by one
// TMA store.  HBM traffic is the algorithmic 5 n sizeof(T) per system.
#include "../../include/tridiagonal.h"
#include "common.cuh"
#include "kernels.h"
#include "tma.cuh"
#include "tw.cuh"

namespace tdg {

constexpr int WMC_MAX_R = 256;
static_assert(WMC_GEN_MAX_ROWS == WMC_MAX_R, "general staging uses the single-CTA kernel");

// solve: a, b, c, d, x (PACKED: m[0] covers every array, x included);
// adjoint: a, b, c, xbar, x, then the outputs ga, gb, gc, gd; chunked
// solve: a, b, c, d, x with boxes of the full chunk, then the same five with
// boxes of the last (shorter) chunk
struct WmcMaps {
  CUtensorMap m[10];
};

// Chunked solve of long systems (MODE 2 / 3): a system of Rt partitions is
// cut into chunks of Rfull partitions (the last one Rlast); MODE 2 writes
// each partition's relations (WMC_REL values) to rel, MODE 3 reads the
// separators' solution y (Ppad values per system) and substitutes back.
constexpr int WMC_REL = 10;
template <typename T>
struct WmcChunk {
  int nchunks, Rfull, Rlast, Rt, Ppad;
  T* rel;
  const T* ysol;
  // element-wise staging of ragged long systems: CTA b serves chunk
  // cl_ch[b] of long system cl_li[b] (= ragged system l_sys[cl_li[b]]), whose
  // partitions start at roff[cl_li[b]] in rel and ysol
  const int* cl_li;
  const int* cl_ch;
  const int* l_sys;
  const long long* roff;
};

// General staging (any n, any offset; ragged batches): the CTA copies its
// system element by element with cp.async into the same swizzled layout
// and pads the last partition with identity rows (a = 0, b = 1, c = 0,
// d = 0); results leave with coalesced stores.  System j of the launch is
// list[j] (or j), rows [offsets[s], offsets[s+1]) (or s*stride .. + n).
template <typename T>
struct WmcGen {
  const T* in[5];  // solve: a, b, c, d; adjoint: a, b, c, xbar, x
  T* out[4];       // solve: x; adjoint: ga, gb, gc, gd
  const long long* offsets;
  const int* list;
  int* info;  // may be NULL: 0 written per system
  long long stride;
  int n;
  // ragged size buckets: systems s with kinds[kind_map ? kind_map[s] : s] !=
  // want are skipped (kinds NULL: none); with a ticket, resident CTAs take
  // the entries list[0 .. count) in turn (one-CTA solves only; count from
  // *dcount where a device pass wrote the list)
  const unsigned char* kinds;
  const int* kind_map;
  int want;
  int* ticket;
  int count;
  const int* dcount;
  RaggedCheck chk;  // (chk.kinds NULL: off) forward solves that check the rows they stage
};

template <typename T>
__device__ __forceinline__ void wmc_cp_async(T* smem, const T* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}

// 16 bytes (both addresses 16-byte aligned).
__device__ __forceinline__ void wmc_cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

template <typename T>
struct WmcVec;
template <>
struct WmcVec<float> {
  using V = float4;
  static constexpr int N = 4;
  __device__ static __forceinline__ void split(const V& v, float (&r)[4]) {
    r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
  }
  __device__ static __forceinline__ V join(const float (&r)[4]) { return make_float4(r[0], r[1], r[2], r[3]); }
};
template <>
struct WmcVec<double> {
  using V = double2;
  static constexpr int N = 2;
  __device__ static __forceinline__ void split(const V& v, double (&r)[2]) {
    r[0] = v.x; r[1] = v.y;
  }
  __device__ static __forceinline__ V join(const double (&r)[2]) { return make_double2(r[0], r[1]); }
};

// byte offset of 16-byte unit q of 128-byte row t under the 128-byte swizzle
__device__ __forceinline__ int wmc_swz(int t, int q) { return t * 128 + ((q ^ (t & 7)) << 4); }

template <typename T>
__host__ __device__ constexpr size_t wmc_array_bytes(int R) {
  return ((size_t)R * 128 + 1023) / 1024 * 1024;
}

template <typename T>
__host__ __device__ constexpr size_t wmc_smem_bytes(int R, int threads, int arrays) {
  return 1024 /* alignment slack */ + arrays * wmc_array_bytes<T>(R) + 8 * (size_t)threads * sizeof(T) + 16;
}

// element k of 128-byte row t of a staged array
template <typename T>
__device__ __forceinline__ T& wmc_elem(unsigned char* S, int t, int k) {
  constexpr int NV = 16 / (int)sizeof(T);
  return *reinterpret_cast<T*>(S + wmc_swz(t, k / NV) + (k % NV) * (int)sizeof(T));
}

// MODE 0: solve A x = d.  MODE 1 (adjoint of x = A^{-1} d for a loss with
// dL/dx = xbar): solve A^T lambda = xbar -- A^T has sub-diagonal c_{i-1} and
// super-diagonal a_{i+1}, formed in shared memory by a shift of the staged
// c and a -- then write gd = lambda, ga_i = -lambda_i x_{i-1},
// gb_i = -lambda_i x_i, gc_i = -lambda_i x_{i+1} (contiguous layout).
// MODE 2 / 3: one chunk of a long system per CTA (see WmcChunk); the
// separators' system between them is solved by a MODE 0 launch.
// GEN: element-wise staging (WmcGen); with TRANS the staged system is A^T
// (sub-diagonal c_{i-1}, super-diagonal a_{i+1}, read shifted from global
// memory) and MODE 3 writes lambda and the gradients (x from gen.in[4]).
template <typename T, int MODE, bool GEN, bool TRANS>
__device__ __forceinline__ void wmc_body(const WmcMaps& maps, int n, int R, int packed, int* err, const WmcChunk<T>& ck,
                                         const WmcGen<T>& gen, const int bid) {
  using W = WmcVec<T>;
  constexpr int NV = W::N;     // values per 16-byte unit
  constexpr int M = 8 * NV;    // rows per thread (128 bytes)
  constexpr int NA = MODE == 1 ? 5 : 4;  // staged arrays
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const size_t ab = wmc_array_bytes<T>(R);
  unsigned char* S[5] = {base, base + ab, base + 2 * ab, base + 3 * ab, base + 4 * ab};
  const int nt = blockDim.x;
  T* red = reinterpret_cast<T*>(base + NA * ab);  // 8 arrays of nt values
  T *ra = red, *rb = red + nt, *rc = red + 2 * nt, *rd = red + 3 * nt;
  T *xg = red + 4 * nt, *xp = red + 5 * nt, *xl = red + 6 * nt, *ys = red + 7 * nt;
  uint64_t* bar = reinterpret_cast<uint64_t*>(red + 8 * nt);

  constexpr bool CHUNKED = MODE >= 2;
  static_assert(!TRANS || (GEN && CHUNKED), "transposed staging serves the chunked element-wise path");
  int j = CHUNKED ? bid / ck.nchunks : bid;
  int ch = CHUNKED ? bid % ck.nchunks : 0;
  bool last_chunk = !CHUNKED || ch == ck.nchunks - 1;
  int Rc = CHUNKED && last_chunk ? ck.Rlast : R;  // partitions of this CTA
  int nn = n;                                      // rows of this system
  long long goff = 0;                              // first row of this CTA (GEN)
  int row_start = 0;                               // ... within its system
  int rows_here = n;                               // rows this CTA holds
  int lead = 0;                                    // identity rows before them (GEN)
  size_t rel_base = CHUNKED ? (size_t)j * ck.Rt + (size_t)ch * R : 0;     // partition index of t = 0
  size_t y_base = CHUNKED ? (size_t)j * ck.Ppad + (size_t)ch * R : 0;
  if constexpr (GEN) {
    int li = 0;
    if constexpr (CHUNKED) {
      li = ck.cl_li[bid];
      ch = ck.cl_ch[bid];
      j = ck.l_sys[li];
    } else {
      j = gen.list ? gen.list[bid] : bid;
    }
    const long long gsys = gen.offsets ? gen.offsets[j] : (long long)j * gen.stride;
    nn = gen.offsets ? (int)(gen.offsets[j + 1] - gsys) : gen.n;
    // a long ragged system's chunks start on 16-byte boundaries (of arrays
    // that start on one): chunk 0 holds the system's first rows after
    // `phase` identity rows, the others start `phase` rows early (the plan
    // counts the system's partitions and chunks with the phase)
    int phase = CHUNKED && gen.offsets ? (int)(gsys % NV) : 0;
    if ((nn + phase + M - 1) / M > WMC_GEN_MAX_ROWS * M) phase = 0;  // (its separators must stay within one CTA)
    lead = CHUNKED && ch == 0 ? phase : 0;
    row_start = CHUNKED ? (ch == 0 ? 0 : ch * R * M - phase) : 0;
    rows_here = min(nn - row_start, R * M - lead);
    Rc = (lead + rows_here + M - 1) / M;
    last_chunk = row_start + rows_here >= nn;
    goff = gsys + row_start;
    if constexpr (CHUNKED) rel_base = y_base = (size_t)ck.roff[li] + (size_t)ch * R;
  }
  const int mset = CHUNKED && last_chunk && ck.Rlast != R ? 5 : 0;
  const int row0 = CHUNKED ? j * ck.Rt + ch * R : j * R;  // first 128-byte row (non-packed, TMA)
  const int t = threadIdx.x;
  const bool active = t < Rc;
  if constexpr (GEN) {
    const int units = Rc * M / NV;
#pragma unroll
    for (int k = 0; k < NA; ++k) {
      // A as it is (TRANS too: A^T is formed below); a_0 and c_{n-1} are
      // not read.  Shared row i holds the CTA's row i - lead; a 16-byte unit
      // whose rows are all real (none of them a_0 or c_{n-1}) and whose
      // global address is 16-byte aligned moves as one copy, the others
      // element by element (identity rows: b = 1, the rest 0).
      const T* src = gen.in[k] + goff;
      const T pad = k == 1 ? T(1) : T(0);
      const bool aligned = ((reinterpret_cast<uintptr_t>(src) / sizeof(T) + (uintptr_t)(NV - lead)) % NV) == 0;
      auto unit = [&](int v) {
        const int i = v * NV, j0 = i - lead;  // first shared row of the unit, its row in the CTA
        unsigned char* dst = S[k] + wmc_swz(i / M, (i % M) / NV);
        const int r = row_start + j0;  // row within the system
        const bool whole = aligned && j0 >= 0 && j0 + NV <= rows_here && !(k == 0 && r == 0) && !(k == 2 && r + NV >= nn);
        if (whole) {
          wmc_cp_async16(dst, src + j0);
        } else {
#pragma unroll
          for (int e = 0; e < NV; ++e) {
            T* de = reinterpret_cast<T*>(dst) + e;
            const int jj = j0 + e;
            const bool real = jj >= 0 && jj < rows_here;
            const bool skip = (k == 0 && r + e == 0) || (k == 2 && r + e == nn - 1);
            if (real && !skip)
              wmc_cp_async(de, src + jj);
            else
              *de = real ? T(0) : pad;
          }
        }
      };
      // The units [vlo, vhi) are whole by construction -- past the lead rows
      // and a_0, before the chunk's last real row and c_{n-1} -- and move
      // with no per-unit tests; only the few units at the chunk's ends take
      // the tests above.
      int vlo = 0, vhi = 0;
      if (aligned) {
        vlo = (lead > 0 ? 1 : 0) + (k == 0 && row_start == 0 && lead == 0 ? 1 : 0);
        vhi = (rows_here + lead) / NV;
        if (k == 2) {
          const int xc = nn - row_start + lead - NV;  // whole c units need r + NV < nn
          vhi = min(vhi, xc > 0 ? (xc + NV - 1) / NV : 0);
        }
      }
      int v = t;
      for (; v < units && v < vlo; v += nt) unit(v);
      for (; v < vhi; v += nt) wmc_cp_async16(S[k] + wmc_swz(v >> 3, v & 7), src + (v * NV - lead));
      for (; v < units; v += nt) unit(v);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    if constexpr ((MODE == 0 || MODE == 2) && !TRANS) {
      if (gen.chk.kinds) {
        // a system that needs pivoting is not solved here: it goes to the
        // pivoted bucket of its size class (the staged rows are checked
        // before any arithmetic; a chunk checks its own rows)
        bool bad = false;
        if (active) {
          // 16-byte units of the partition's row; rows past the system are
          // identity rows, which pass
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            T av[NV], bv[NV], cv[NV];
            const int off = wmc_swz(t, u);
            W::split(*reinterpret_cast<const typename W::V*>(S[0] + off), av);
            W::split(*reinterpret_cast<const typename W::V*>(S[1] + off), bv);
            W::split(*reinterpret_cast<const typename W::V*>(S[2] + off), cv);
#pragma unroll
            for (int e = 0; e < NV; ++e) bad |= !dominant_row(av[e], bv[e], cv[e]);
          }
        }
        if (__syncthreads_or(bad)) {
          if (t == 0) {
            gen.chk.kinds[j] = 0;
            if (!CHUNKED || atomicExch(&gen.chk.claim[j], 1) == 0) {
              int cls = 0;
              while ((1ll << cls) < (long long)nn) ++cls;
              const int r = gen.chk.reg[2 * cls];
              if (r >= 0) gen.chk.klists[r + atomicAdd(&gen.chk.kcount[2 * cls], 1)] = j;
            }
          }
          return;
        }
      }
    }
    if constexpr (TRANS) {
      // A^T of the staged A, as MODE 1 forms it below: sub-diagonal c_{i-1}
      // into the a slot, super-diagonal a_{i+1} into the c slot; across the
      // chunk's edges from global memory (c of the row before its first row,
      // a of the row after its last one where that row is in the system)
      T cprev = T(0), anext = T(0);
      if (active) {
        if (t > 0) cprev = wmc_elem<T>(S[2], t - 1, M - 1);
        else if (row_start > 0) cprev = gen.in[2][goff - 1];
        if (t + 1 < Rc) anext = wmc_elem<T>(S[0], t + 1, 0);
        else if (lead + rows_here == Rc * M && row_start + rows_here < nn) anext = gen.in[0][goff + rows_here];
      }
      __syncthreads();
      if (active) {
        T carry = cprev;
        T av[NV], an[NV];
        W::split(*reinterpret_cast<const typename W::V*>(S[0] + wmc_swz(t, 0)), av);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int off = wmc_swz(t, q);
          if (q < 7) W::split(*reinterpret_cast<const typename W::V*>(S[0] + wmc_swz(t, q + 1)), an);
          T cv[NV], sub[NV], sup[NV];
          W::split(*reinterpret_cast<const typename W::V*>(S[2] + off), cv);
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            sub[v] = v == 0 ? carry : cv[v - 1];
            sup[v] = v + 1 < NV ? av[v + 1] : (q < 7 ? an[0] : anext);
          }
          carry = cv[NV - 1];
          *reinterpret_cast<typename W::V*>(S[0] + off) = W::join(sub);
          *reinterpret_cast<typename W::V*>(S[2] + off) = W::join(sup);
#pragma unroll
          for (int v = 0; v < NV; ++v) av[v] = an[v];
        }
      }
      __syncthreads();
    }
  } else {
    if (t == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (t == 0) {
      mbar_arrive_expect_tx(bar, (unsigned)NA * (unsigned)Rc * 128u);
#pragma unroll
      for (int k = 0; k < NA; ++k) {
        const CUtensorMap* mp = &maps.m[packed ? 0 : mset + k];
        const int row = packed ? (j * 4 + k) * R : row0;
        tma_load_2d(S[k], mp, 0, row, bar);
      }
    }
    const bool ok = mbar_wait(bar, 0, err);
    if (!__syncthreads_and(ok)) return;
  }

  if constexpr (MODE == 1) {
    // A^T: sub-diagonal c_{i-1} into the a slot, super-diagonal a_{i+1} into
    // the c slot (the neighbours' boundary values are read before anyone
    // writes)
    const T cprev = (active && t > 0) ? wmc_elem<T>(S[2], t - 1, M - 1) : T(0);
    const T anext = (active && t + 1 < Rc) ? wmc_elem<T>(S[0], t + 1, 0) : T(0);
    __syncthreads();
    if (active) {
      T carry = cprev;
      T av[NV], an[NV];
      W::split(*reinterpret_cast<const typename W::V*>(S[0] + wmc_swz(t, 0)), av);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int off = wmc_swz(t, q);
        if (q < 7) W::split(*reinterpret_cast<const typename W::V*>(S[0] + wmc_swz(t, q + 1)), an);
        T cv[NV], sub[NV], sup[NV];
        W::split(*reinterpret_cast<const typename W::V*>(S[2] + off), cv);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          sub[v] = v == 0 ? carry : cv[v - 1];
          sup[v] = v + 1 < NV ? av[v + 1] : (q < 7 ? an[0] : anext);
        }
        carry = cv[NV - 1];
        *reinterpret_cast<typename W::V*>(S[0] + off) = W::join(sub);
        *reinterpret_cast<typename W::V*>(S[2] + off) = W::join(sup);
#pragma unroll
        for (int v = 0; v < NV; ++v) av[v] = an[v];
      }
    }
  }

  // ---- top-down elimination of the interior rows --------------------------
  T cp = T(0), dp = T(0), vp = T(0);  // c', d', v of the previous row
  T G = T(0), L = T(0), P = T(0);     // first-row relation
  T sa = T(0), sb = T(1), sc = T(0), sd = T(0);  // separator row
  if (active) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int off = wmc_swz(t, q);
      T va[NV], vb[NV], vc[NV], vd[NV];
      W::split(*reinterpret_cast<const typename W::V*>(S[0] + off), va);
      W::split(*reinterpret_cast<const typename W::V*>(S[1] + off), vb);
      W::split(*reinterpret_cast<const typename W::V*>(S[2] + off), vc);
      W::split(*reinterpret_cast<const typename W::V*>(S[3] + off), vd);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const int k = q * NV + v;
        const T a = (ch == 0 && t == 0 && k == 0) ? T(0) : va[v];  // a_0 is not read
        if (k < M - 1) {
          const T den = k == 0 ? vb[v] : fma(-a, cp, vb[v]);
          const T r = Div<T>(den).inv();
          const T ncp = vc[v] * r;
          const T ndp = (k == 0 ? vd[v] : fma(-a, dp, vd[v])) * r;
          const T nvp = (k == 0 ? a : -a * vp) * r;
          if (k == 0) {
            G = ndp;
            L = nvp;
            P = -ncp;
          } else {
            G = fma(P, ndp, G);
            L = fma(P, nvp, L);
            P = -P * ncp;
          }
          cp = ncp;
          dp = ndp;
          vp = nvp;
          va[v] = nvp;
          vb[v] = ncp;
          vd[v] = ndp;
        } else {
          sa = a;
          sb = vb[v];
          sc = (last_chunk && t == Rc - 1) ? T(0) : vc[v];  // c_{n-1} is not read
          sd = vd[v];
        }
      }
      *reinterpret_cast<typename W::V*>(S[0] + off) = W::join(va);
      *reinterpret_cast<typename W::V*>(S[1] + off) = W::join(vb);
      *reinterpret_cast<typename W::V*>(S[3] + off) = W::join(vd);
    }
    xg[t] = G;
    xp[t] = P;
    xl[t] = L;
  }
  if constexpr (MODE == 2) {
    // the partition's relations for the separators' system
    if (active) {
      T* o = ck.rel + (rel_base + t) * WMC_REL;
      o[0] = G;
      o[1] = P;
      o[2] = L;
      o[3] = vp;
      o[4] = cp;
      o[5] = dp;
      o[6] = sa;
      o[7] = sb;
      o[8] = sc;
      o[9] = sd;
    }
    return;
  }
  __syncthreads();
  // ---- the separators' tridiagonal system ---------------------------------
  if constexpr (MODE != 3) {
  T al = T(0), be = T(1), ga = T(0), de = T(0);
  if (active) {
    const T Gn = t + 1 < Rc ? xg[t + 1] : T(0);
    const T Pn = t + 1 < Rc ? xp[t + 1] : T(0);
    const T Ln = t + 1 < Rc ? xl[t + 1] : T(0);
    al = -sa * vp;
    be = fma(-sc, Ln, fma(-sa, cp, sb));
    ga = sc * Pn;
    de = fma(-sc, Gn, fma(-sa, dp, sd));
  }
  // parallel cyclic reduction: row t combines rows t - s and t + s.  Each
  // row publishes (a, 1/b, c, d): its reciprocal is formed once, by its
  // owner, instead of once by each of its two readers (the same value: x
  // is unchanged), which for FP64 saves three FP64 instructions per row and
  // step.
  T ib = active ? Div<T>(be).inv() : T(1);
  for (int s = 1; s < Rc; s <<= 1) {
    if (active) {
      ra[t] = al;
      rb[t] = ib;
      rc[t] = ga;
      rd[t] = de;
    }
    __syncthreads();
    if (active) {
      T a1 = T(0), i1 = T(1), c1 = T(0), d1 = T(0), a2 = T(0), i2 = T(1), c2 = T(0), d2 = T(0);
      if (t - s >= 0) {
        a1 = ra[t - s];
        i1 = rb[t - s];
        c1 = rc[t - s];
        d1 = rd[t - s];
      }
      if (t + s < Rc) {
        a2 = ra[t + s];
        i2 = rb[t + s];
        c2 = rc[t + s];
        d2 = rd[t + s];
      }
      const T k1 = al * i1;
      const T k2 = ga * i2;
      be = fma(-k2, a2, fma(-k1, c1, be));
      de = fma(-k2, d2, fma(-k1, d1, de));
      al = -k1 * a1;
      ga = -k2 * c2;
      ib = Div<T>(be).inv();
    }
    __syncthreads();
  }
  if (active) ys[t] = de * ib;
  }
  if constexpr (MODE == 3) {
    if (active) {
      const size_t g = y_base + t;
      ys[t] = ck.ysol[g];
      xl[t] = (ch > 0 || t > 0) ? ck.ysol[g - 1] : T(0);
    }
  }
  __syncthreads();
  // ---- bottom-up substitution ---------------------------------------------
  if (active) {
    const T y = ys[t];
    const T yl = MODE == 3 ? xl[t] : (t > 0 ? ys[t - 1] : T(0));
    T xn = y;
#pragma unroll
    for (int q = 7; q >= 0; --q) {
      const int off = wmc_swz(t, q);
      T va[NV], vb[NV], vd[NV];
      W::split(*reinterpret_cast<const typename W::V*>(S[0] + off), va);
      W::split(*reinterpret_cast<const typename W::V*>(S[1] + off), vb);
      W::split(*reinterpret_cast<const typename W::V*>(S[3] + off), vd);
#pragma unroll
      for (int v = NV - 1; v >= 0; --v) {
        const int k = q * NV + v;
        if (k == M - 1) {
          vd[v] = y;
        } else {
          xn = fma(-va[v], yl, fma(-vb[v], xn, vd[v]));
          vd[v] = xn;
        }
      }
      *reinterpret_cast<typename W::V*>(S[3] + off) = W::join(vd);
    }
  }
  if constexpr (MODE == 1) {
    // gradients: lambda (in the d slot) times the forward solution x
    if (active) {
      const T xprev = t > 0 ? wmc_elem<T>(S[4], t - 1, M - 1) : T(0);
      const T xnext = t + 1 < Rc ? wmc_elem<T>(S[4], t + 1, 0) : T(0);
      T carry = xprev;
      T xv[NV], xn[NV];
      W::split(*reinterpret_cast<const typename W::V*>(S[4] + wmc_swz(t, 0)), xv);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int off = wmc_swz(t, q);
        if (q < 7) W::split(*reinterpret_cast<const typename W::V*>(S[4] + wmc_swz(t, q + 1)), xn);
        T lam[NV], ga_[NV], gb_[NV], gc_[NV];
        W::split(*reinterpret_cast<const typename W::V*>(S[3] + off), lam);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const int i = t * M + q * NV + v;
          const T xl_ = v == 0 ? carry : xv[v - 1];
          const T xr_ = v + 1 < NV ? xv[v + 1] : (q < 7 ? xn[0] : xnext);
          ga_[v] = i > 0 ? -lam[v] * xl_ : T(0);
          gb_[v] = -lam[v] * xv[v];
          gc_[v] = i + 1 < nn ? -lam[v] * xr_ : T(0);
        }
        carry = xv[NV - 1];
        *reinterpret_cast<typename W::V*>(S[0] + off) = W::join(ga_);
        *reinterpret_cast<typename W::V*>(S[1] + off) = W::join(gb_);
        *reinterpret_cast<typename W::V*>(S[2] + off) = W::join(gc_);
#pragma unroll
        for (int v = 0; v < NV; ++v) xv[v] = xn[v];
      }
    }
  }
  if constexpr (GEN) {
    if (gen.info && t == 0 && (!CHUNKED || ch == 0)) gen.info[j] = 0;
    __syncthreads();
    if constexpr (TRANS) {
      // lambda and the gradients ga = -lambda x_{i-1}, gb = -lambda x_i,
      // gc = -lambda x_{i+1} (x of the forward solve in gen.in[4]).  The
      // x loads of U rows per thread are issued before any store (the
      // outputs could alias x as far as the compiler knows, which would
      // otherwise serialise one load latency per row).
      const T* __restrict__ xf = gen.in[4] + goff;
      T* __restrict__ o0 = gen.out[0] + goff;
      T* __restrict__ o1 = gen.out[1] + goff;
      T* __restrict__ o2 = gen.out[2] + goff;
      T* __restrict__ o3 = gen.out[3] + goff;
      auto al16 = [&](const T* q) {  // shared row 0's global address 16-byte aligned
        return ((reinterpret_cast<uintptr_t>(q) / sizeof(T) + (uintptr_t)(NV - lead)) % NV) == 0 &&
               reinterpret_cast<uintptr_t>(q) % sizeof(T) == 0;
      };
      if (al16(xf) && al16(o0) && al16(o1) && al16(o2) && al16(o3)) {
        // whole 16-byte units of rows: lambda from shared memory, x of the
        // unit and of the rows either side from global memory
        const int units = (lead + rows_here + NV - 1) / NV;
        for (int v = t; v < units; v += nt) {
          const int i = v * NV, j0 = i - lead, r0 = row_start + j0;
          if (j0 >= 0 && j0 + NV <= rows_here) {
            T lam[NV], xc[NV], g1[NV], g2[NV], g3[NV];
            W::split(*reinterpret_cast<const typename W::V*>(S[3] + wmc_swz(i / M, (i % M) / NV)), lam);
            W::split(__ldg(reinterpret_cast<const typename W::V*>(xf + j0)), xc);
            const T xl = r0 > 0 ? __ldg(xf + j0 - 1) : T(0);
            const T xr = r0 + NV < nn ? __ldg(xf + j0 + NV) : T(0);
#pragma unroll
            for (int e = 0; e < NV; ++e) {
              g1[e] = r0 + e > 0 ? -lam[e] * (e > 0 ? xc[e - 1] : xl) : T(0);
              g2[e] = -lam[e] * xc[e];
              g3[e] = r0 + e + 1 < nn ? -lam[e] * (e + 1 < NV ? xc[e + 1] : xr) : T(0);
            }
            *reinterpret_cast<typename W::V*>(o0 + j0) = W::join(lam);
            *reinterpret_cast<typename W::V*>(o1 + j0) = W::join(g1);
            *reinterpret_cast<typename W::V*>(o2 + j0) = W::join(g2);
            *reinterpret_cast<typename W::V*>(o3 + j0) = W::join(g3);
          } else {
            for (int e = 0; e < NV; ++e) {
              const int jj = j0 + e, r = row_start + jj;
              if (jj < 0 || jj >= rows_here) continue;
              const T l = wmc_elem<T>(S[3], (jj + lead) / M, (jj + lead) % M);
              o0[jj] = l;
              o1[jj] = r > 0 ? -l * __ldg(xf + jj - 1) : T(0);
              o2[jj] = -l * __ldg(xf + jj);
              o3[jj] = r + 1 < nn ? -l * __ldg(xf + jj + 1) : T(0);
            }
          }
        }
        return;
      }
      constexpr int U = 8;
      for (int i0 = t; i0 < rows_here; i0 += U * nt) {
        T xl_[U], xc_[U], xr_[U], lam[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 + u * nt, r = row_start + i;
          xl_[u] = xc_[u] = xr_[u] = lam[u] = T(0);
          if (i < rows_here) {
            if (r > 0) xl_[u] = __ldg(xf + i - 1);
            xc_[u] = __ldg(xf + i);
            if (r + 1 < nn) xr_[u] = __ldg(xf + i + 1);
            lam[u] = wmc_elem<T>(S[3], (i + lead) / M, (i + lead) % M);
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 + u * nt, r = row_start + i;
          if (i < rows_here) {
            o0[i] = lam[u];
            o1[i] = r > 0 ? -lam[u] * xl_[u] : T(0);
            o2[i] = -lam[u] * xc_[u];
            o3[i] = r + 1 < nn ? -lam[u] * xr_[u] : T(0);
          }
        }
      }
    } else {
      constexpr int NO = MODE == 1 ? 4 : 1;
#pragma unroll
      for (int k = 0; k < NO; ++k) {
        unsigned char* src = S[MODE == 1 ? k : 3];
        T* dst = gen.out[k] + goff;
        // whole 16-byte units where the rows' global addresses allow (shared
        // row i is the CTA's row i - lead)
        if (((reinterpret_cast<uintptr_t>(dst) / sizeof(T) + (uintptr_t)(NV - lead)) % NV) == 0 &&
            (reinterpret_cast<uintptr_t>(dst) % sizeof(T)) == 0) {
          const int units = (lead + rows_here + NV - 1) / NV;
          for (int v = t; v < units; v += nt) {
            const int i = v * NV, j0 = i - lead;
            const unsigned char* su = src + wmc_swz(i / M, (i % M) / NV);
            if (j0 >= 0 && j0 + NV <= rows_here) {
              *reinterpret_cast<uint4*>(dst + j0) = *reinterpret_cast<const uint4*>(su);
            } else {
              for (int e = 0; e < NV; ++e)
                if (j0 + e >= 0 && j0 + e < rows_here) dst[j0 + e] = reinterpret_cast<const T*>(su)[e];
            }
          }
        } else {
          for (int i = t; i < rows_here; i += nt) dst[i] = wmc_elem<T>(src, (i + lead) / M, (i + lead) % M);
        }
      }
    }
    return;
  }
  fence_async_smem();
  __syncthreads();
  if (t == 0) {
    if constexpr (MODE == 1) {
#pragma unroll
      for (int k = 0; k < 4; ++k) tma_store_2d(&maps.m[5 + k], 0, j * R, S[k]);
    } else {
      const int row = packed ? (j * 4 + 3) * R : row0;
      tma_store_2d(&maps.m[packed ? 0 : mset + 4], 0, row, S[3]);
    }
    bulk_commit();
    bulk_wait_read<0>();
  }
}

template <typename T, int MODE, bool GEN = false, bool TRANS = false>
__global__ void __launch_bounds__(WMC_MAX_R) wmc_kernel(const __grid_constant__ WmcMaps maps, int n, int R,
                                                        int packed, int* err, const WmcChunk<T> ck,
                                                        const WmcGen<T> gen) {
  if constexpr (GEN) {
    auto skipped = [&](int j) { return gen.kinds && gen.kinds[gen.kind_map ? gen.kind_map[j] : j] != gen.want; };
    if constexpr (MODE <= 1) {
      if (gen.ticket) {
        // resident CTAs drain one size bucket of a ragged batch
        __shared__ int s_item;
        for (;;) {
          if (threadIdx.x == 0) {
            const int k = atomicAdd(gen.ticket, 1);
            const int cnt = gen.dcount ? *(volatile const int*)gen.dcount : gen.count;
            s_item = k < cnt && (!err || *(volatile int*)err == 0) ? k : -1;
          }
          __syncthreads();
          const int k = s_item;
          __syncthreads();
          if (k < 0) break;
          if (skipped(gen.list ? gen.list[k] : k)) continue;
          wmc_body<T, MODE, GEN, TRANS>(maps, n, R, packed, err, ck, gen, k);
          __syncthreads();
        }
        return;
      }
      if (skipped(gen.list ? gen.list[blockIdx.x] : (int)blockIdx.x)) return;
    } else {
      if (skipped(ck.l_sys[ck.cl_li[blockIdx.x]])) return;
    }
  }
  wmc_body<T, MODE, GEN, TRANS>(maps, n, R, packed, err, ck, gen, blockIdx.x);
}

template <typename T>
bool wmc_eligible(int layout, int n) {
  constexpr int M = 128 / (int)sizeof(T);
  if (layout != CONTIG && layout != PACKED) return false;
  if (n % M != 0) return false;
  const int R = n / M;
  return R >= 8 && R <= WMC_MAX_R;
}

// the general staging: any n up to WMC_MAX_R 128-byte rows
template <typename T>
bool wmc_gen_eligible(int layout, int n) {
  constexpr int M = 128 / (int)sizeof(T);
  return (layout == CONTIG || layout == PACKED) && n >= 1 && n <= WMC_MAX_R * M;
}

template <typename T, int MODE>
static cudaError_t wmc_gen_launch(const WmcGen<T>& gen, int count, int Rmax, cudaStream_t s) {
  const int threads = (Rmax + 31) / 32 * 32;
  const size_t smem = wmc_smem_bytes<T>(Rmax, threads, MODE == 1 ? 5 : 4);
  cudaError_t e =
      cudaFuncSetAttribute(wmc_kernel<T, MODE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int grid = count;
  if (gen.ticket) {
    // a ticket-driven bucket: as many CTAs as stay resident at once
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, wmc_kernel<T, MODE, true>, threads, smem) ==
            cudaSuccess &&
        per > 0)
      grid = count < sms * per ? count : sms * per;
  }
  WmcMaps maps{};
  wmc_kernel<T, MODE, true><<<grid, threads, smem, s>>>(maps, 0, Rmax, 0, error_word(), WmcChunk<T>{}, gen);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_wmc(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                       cudaStream_t s, bool* used) {
  *used = false;
  if (batch <= 0) return cudaSuccess;
  if (!wmc_eligible<T>(layout, n)) {
    if (!wmc_gen_eligible<T>(layout, n)) return cudaSuccess;
    constexpr int M = 128 / (int)sizeof(T);
    WmcGen<T> gen{};
    const bool pk = layout == PACKED;
    if (pk && x != d) return cudaSuccess;
    gen.in[0] = a;
    gen.in[1] = pk ? a + n : b;
    gen.in[2] = pk ? a + 2 * (size_t)n : c;
    gen.in[3] = pk ? a + 3 * (size_t)n : d;
    gen.out[0] = pk ? const_cast<T*>(a) + 3 * (size_t)n : x;
    gen.stride = pk ? 4 * (long long)n : (long long)n;
    gen.n = n;
    cudaError_t e = wmc_gen_launch<T, 0>(gen, batch, (n + M - 1) / M, s);
    if (e == cudaSuccess) *used = true;
    return e;
  }
  constexpr int M = 128 / (int)sizeof(T);
  const int R = n / M;
  const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  WmcMaps maps;
  const bool packed = layout == PACKED;
  if (packed) {
    // one tensor over the whole packed batch: rows of 128 bytes, 4 R rows per system
    if (x != d) return cudaSuccess;
    if (!encode_tmap_2d(&maps.m[0], a, dt, sizeof(T), (uint64_t)M, (uint64_t)4 * R * (uint64_t)batch, 128, M, R,
                        CU_TENSOR_MAP_SWIZZLE_128B))
      return cudaSuccess;
  } else {
    const T* ptrs[5] = {a, b, c, d, x};
    for (int k = 0; k < 5; ++k)
      if (!encode_tmap_2d(&maps.m[k], ptrs[k], dt, sizeof(T), (uint64_t)M, (uint64_t)R * (uint64_t)batch, 128, M, R,
                          CU_TENSOR_MAP_SWIZZLE_128B))
        return cudaSuccess;
  }
  const int threads = (R + 31) / 32 * 32;
  const size_t smem = wmc_smem_bytes<T>(R, threads, 4);
  cudaError_t e = cudaFuncSetAttribute(wmc_kernel<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  wmc_kernel<T, 0><<<batch, threads, smem, s>>>(maps, n, R, packed ? 1 : 0, error_word(), WmcChunk<T>{}, WmcGen<T>{});
  e = cudaGetLastError();
  if (e == cudaSuccess) *used = true;
  return e;
}

template <typename T>
cudaError_t launch_wmc_adjoint(const T* a, const T* b, const T* c, const T* x, const T* xbar, T* ga, T* gb, T* gc,
                               T* gd, int n, int batch, cudaStream_t s, bool* used) {
  *used = false;
  if (batch <= 0) return cudaSuccess;
  if (!wmc_eligible<T>(CONTIG, n)) {
    if (!wmc_gen_eligible<T>(CONTIG, n)) return cudaSuccess;
    constexpr int M = 128 / (int)sizeof(T);
    WmcGen<T> gen{};
    const T* ins[5] = {a, b, c, xbar, x};
    T* outs[4] = {ga, gb, gc, gd};
    for (int k = 0; k < 5; ++k) gen.in[k] = ins[k];
    for (int k = 0; k < 4; ++k) gen.out[k] = outs[k];
    gen.stride = n;
    gen.n = n;
    cudaError_t e = wmc_gen_launch<T, 1>(gen, batch, (n + M - 1) / M, s);
    if (e == cudaSuccess) *used = true;
    return e;
  }
  constexpr int M = 128 / (int)sizeof(T);
  const int R = n / M;
  const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  WmcMaps maps;
  const T* ptrs[9] = {a, b, c, xbar, x, ga, gb, gc, gd};
  for (int k = 0; k < 9; ++k)
    if (!encode_tmap_2d(&maps.m[k], ptrs[k], dt, sizeof(T), (uint64_t)M, (uint64_t)R * (uint64_t)batch, 128, M, R,
                        CU_TENSOR_MAP_SWIZZLE_128B))
      return cudaSuccess;
  const int threads = (R + 31) / 32 * 32;
  const size_t smem = wmc_smem_bytes<T>(R, threads, 5);
  cudaError_t e = cudaFuncSetAttribute(wmc_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  wmc_kernel<T, 1><<<batch, threads, smem, s>>>(maps, n, R, 0, error_word(), WmcChunk<T>{}, WmcGen<T>{});
  e = cudaGetLastError();
  if (e == cudaSuccess) *used = true;
  return e;
}

template cudaError_t launch_wmc_adjoint<float>(const float*, const float*, const float*, const float*, const float*,
                                               float*, float*, float*, float*, int, int, cudaStream_t, bool*);
template cudaError_t launch_wmc_adjoint<double>(const double*, const double*, const double*, const double*,
                                                const double*, double*, double*, double*, double*, int, int,
                                                cudaStream_t, bool*);
// ---------------------------------------------------------------------------
// Long systems: chunks of WML_CHUNK_R partitions per CTA (MODE 2), the
// separators' system (one row per partition, padded to a shape the
// single-CTA kernel covers) assembled and solved by MODE 0, then the chunks
// again (MODE 3).  Traffic: the four inputs twice, x once, plus ~14 values
// per partition of workspace.

template <typename T>
static int wml_ppad(int Rt) {
  constexpr int M = 128 / (int)sizeof(T);
  int p = (Rt + M - 1) / M * M;
  return p < 8 * M ? 8 * M : p;
}

template <typename T>
bool wml_eligible(int layout, int n) {
  constexpr int M = 128 / (int)sizeof(T);
  if (layout != CONTIG || n % M != 0) return false;
  const int Rt = n / M;
  return Rt > WMC_MAX_R && wml_ppad<T>(Rt) <= WMC_MAX_R * M;  // longer than one CTA holds
}

template <typename T>
size_t wml_workspace_bytes(int n, int batch) {
  constexpr int M = 128 / (int)sizeof(T);
  const int Rt = n / M;
  const size_t rel = ((size_t)WMC_REL * Rt * batch * sizeof(T) + 255) / 256 * 256;
  const size_t red = ((size_t)wml_ppad<T>(Rt) * batch * sizeof(T) + 255) / 256 * 256;
  return rel + 4 * red;
}

template <typename T>
__global__ void __launch_bounds__(256) wml_assemble(const T* __restrict__ rel, T* al, T* be, T* ga, T* de, int Rt,
                                                    int Ppad, int batch) {
  const size_t total = (size_t)Ppad * (size_t)batch;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const size_t j = idx / (size_t)Ppad;
    const int p = (int)(idx % (size_t)Ppad);
    T a_ = T(0), b_ = T(1), g_ = T(0), d_ = T(0);
    if (p < Rt) {
      const T* o = rel + (j * Rt + p) * WMC_REL;
      const T* on = o + WMC_REL;
      const bool nx = p + 1 < Rt;
      const T Gn = nx ? on[0] : T(0), Pn = nx ? on[1] : T(0), Ln = nx ? on[2] : T(0);
      const T vL = o[3], cL = o[4], dL = o[5], sa = o[6], sb = o[7], sc = o[8], sd = o[9];
      a_ = -sa * vL;
      b_ = fma(-sc, Ln, fma(-sa, cL, sb));
      g_ = sc * Pn;
      d_ = fma(-sc, Gn, fma(-sa, dL, sd));
    }
    al[idx] = a_;
    be[idx] = b_;
    ga[idx] = g_;
    de[idx] = d_;
  }
}

template <typename T>
cudaError_t launch_wml(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch, void* work,
                       size_t work_bytes, cudaStream_t s, bool* used) {
  *used = false;
  if (!wml_eligible<T>(CONTIG, n) || batch <= 0 || !work || work_bytes < wml_workspace_bytes<T>(n, batch))
    return cudaSuccess;
  constexpr int M = 128 / (int)sizeof(T);
  const int Rt = n / M, R = WML_CHUNK_R;
  const int nchunks = (Rt + R - 1) / R;
  const int Rlast = Rt - (nchunks - 1) * R;
  const int Ppad = wml_ppad<T>(Rt);
  const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  WmcMaps maps;
  const T* ptrs[5] = {a, b, c, d, x};
  for (int set = 0; set < (Rlast != R ? 2 : 1); ++set)
    for (int k = 0; k < 5; ++k)
      if (!encode_tmap_2d(&maps.m[set * 5 + k], ptrs[k], dt, sizeof(T), (uint64_t)M, (uint64_t)Rt * (uint64_t)batch,
                          128, M, set ? Rlast : R, CU_TENSOR_MAP_SWIZZLE_128B))
        return cudaSuccess;
  char* p = static_cast<char*>(work);
  T* rel = reinterpret_cast<T*>(p);
  p += ((size_t)WMC_REL * Rt * batch * sizeof(T) + 255) / 256 * 256;
  const size_t red = ((size_t)Ppad * batch * sizeof(T) + 255) / 256 * 256;
  T* ra = reinterpret_cast<T*>(p);
  T* rb = reinterpret_cast<T*>(p + red);
  T* rc = reinterpret_cast<T*>(p + 2 * red);
  T* rd = reinterpret_cast<T*>(p + 3 * red);
  const size_t smem = wmc_smem_bytes<T>(R, R, 4);
  cudaError_t e = cudaFuncSetAttribute(wmc_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(wmc_kernel<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)nchunks * (unsigned)batch;
  WmcChunk<T> ck{nchunks, R, Rlast, Rt, Ppad, rel, rd};
  wmc_kernel<T, 2><<<grid, R, smem, s>>>(maps, n, R, 0, error_word(), ck, WmcGen<T>{});
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t total = (size_t)Ppad * batch;
  const unsigned ag = (unsigned)((total + 255) / 256 < (size_t)sms * 8 ? (total + 255) / 256 : (size_t)sms * 8);
  wml_assemble<T><<<ag, 256, 0, s>>>(rel, ra, rb, rc, rd, Rt, Ppad, batch);
  bool inner = false;
  e = launch_wmc<T>(CONTIG, ra, rb, rc, rd, rd, Ppad, batch, s, &inner);
  if (e != cudaSuccess) return e;
  if (!inner) return cudaErrorInvalidConfiguration;
  wmc_kernel<T, 3><<<grid, R, smem, s>>>(maps, n, R, 0, error_word(), ck, WmcGen<T>{});
  e = cudaGetLastError();
  if (e == cudaSuccess) *used = true;
  return e;
}

template bool wml_eligible<float>(int, int);
template bool wml_eligible<double>(int, int);
template size_t wml_workspace_bytes<float>(int, int);
template size_t wml_workspace_bytes<double>(int, int);
template cudaError_t launch_wml<float>(const float*, const float*, const float*, const float*, float*, int, int,
                                       void*, size_t, cudaStream_t, bool*);
template cudaError_t launch_wml<double>(const double*, const double*, const double*, const double*, double*, int,
                                        int, void*, size_t, cudaStream_t, bool*);

// Ragged batches: `count` systems list[0..count) of the packed arrays, each
// with n <= Rmax 128-byte rows (the caller groups systems by size).
template <typename T>
cudaError_t launch_wmc_ragged(int mode, const T* a, const T* b, const T* c, const T* d, const T* xf, T* o0, T* o1,
                              T* o2, T* o3, const long long* offsets, const int* list, int count, int Rmax, int* info,
                              cudaStream_t s, const BucketTicket* tk, const int* kind_map, const RaggedCheck* chk) {
  if (count <= 0) return cudaSuccess;
  if (Rmax < 1 || Rmax > WMC_MAX_R) return cudaErrorInvalidValue;
  WmcGen<T> gen{};
  if (tk) {
    gen.ticket = tk->ticket;
    gen.count = count;
    gen.dcount = tk->dcount;
    gen.kinds = tk->kinds;
    gen.want = tk->want;
    gen.kind_map = kind_map;
  }
  if (chk && mode == 0) gen.chk = *chk;
  gen.in[0] = a;
  gen.in[1] = b;
  gen.in[2] = c;
  gen.in[3] = d;
  gen.in[4] = xf;
  gen.out[0] = o0;
  gen.out[1] = o1;
  gen.out[2] = o2;
  gen.out[3] = o3;
  gen.offsets = offsets;
  gen.list = list;
  gen.info = info;
  return mode == 1 ? wmc_gen_launch<T, 1>(gen, count, Rmax, s) : wmc_gen_launch<T, 0>(gen, count, Rmax, s);
}

// Long systems of a ragged batch (more rows than one CTA holds), unpivoted:
// chunks of WML_CHUNK_R 128-byte rows per CTA (MODE 2), the separators'
// systems (one per long system, ragged) assembled and solved by the
// element-wise single-CTA kernel, then the chunks again (MODE 3).  mode 1:
// the adjoint, on A^T staged shifted, with the gradient epilogue.
template <typename T>
__global__ void __launch_bounds__(256) wml_assemble_ragged(const T* __restrict__ rel, T* al, T* be, T* ga, T* de,
                                                           const long long* __restrict__ roff, int L,
                                                           long long total) {
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = L;  // roff[lo] <= idx < roff[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (roff[mid] <= idx) lo = mid; else hi = mid;
    }
    const bool nx = idx + 1 < roff[lo + 1];
    const T* o = rel + idx * WMC_REL;
    const T* on = o + WMC_REL;
    const T Gn = nx ? on[0] : T(0), Pn = nx ? on[1] : T(0), Ln = nx ? on[2] : T(0);
    const T vL = o[3], cL = o[4], dL = o[5], sa = o[6], sb = o[7], sc = o[8], sd = o[9];
    al[idx] = -sa * vL;
    be[idx] = fma(-sc, Ln, fma(-sa, cL, sb));
    ga[idx] = sc * Pn;
    de[idx] = fma(-sc, Gn, fma(-sa, dL, sd));
  }
}

template <typename T>
size_t wml_ragged_workspace_elems(long long total_partitions) {
  return (size_t)(WMC_REL + 4) * (size_t)total_partitions;
}

template <typename T>
cudaError_t launch_wml_ragged(int mode, const T* a, const T* b, const T* c, const T* d, const T* xf, T* o0, T* o1,
                              T* o2, T* o3, const long long* offsets, const WmlRagged& lr, T* work, int* info,
                              cudaStream_t s, const unsigned char* kinds, const RaggedCheck* chk) {
  if (lr.L <= 0) return cudaSuccess;
  constexpr int M = 128 / (int)sizeof(T);
  const int R = lr.R;
  T* rel = work;
  T* ra = rel + (size_t)WMC_REL * lr.P;
  T* rb = ra + lr.P;
  T* rc = rb + lr.P;
  T* rd = rc + lr.P;
  WmcChunk<T> ck{};
  ck.nchunks = 1;
  ck.rel = rel;
  ck.ysol = rd;
  ck.cl_li = lr.cl_li;
  ck.cl_ch = lr.cl_ch;
  ck.l_sys = lr.l_sys;
  ck.roff = lr.roff;
  WmcGen<T> gen{};
  gen.offsets = offsets;
  gen.info = info;
  gen.in[0] = a;
  gen.in[1] = b;
  gen.in[2] = c;
  gen.in[3] = d;
  gen.in[4] = xf;
  gen.out[0] = o0;
  gen.out[1] = o1;
  gen.out[2] = o2;
  gen.out[3] = o3;
  gen.kinds = kinds;  // (systems marked for pivoting are skipped)
  gen.want = 1;
  WmcGen<T> gen2 = gen;  // MODE 2 of a forward solve checks the rows it stages
  if (chk && mode == 0) gen2.chk = *chk;
  const size_t smem = wmc_smem_bytes<T>(R, R, 4);
  WmcMaps maps{};
  cudaError_t e;
  if (mode == 1) {
    e = cudaFuncSetAttribute(wmc_kernel<T, 2, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(wmc_kernel<T, 3, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    wmc_kernel<T, 2, true, true><<<lr.C, R, smem, s>>>(maps, 0, R, 0, error_word(), ck, gen);
  } else {
    e = cudaFuncSetAttribute(wmc_kernel<T, 2, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(wmc_kernel<T, 3, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    wmc_kernel<T, 2, true, false><<<lr.C, R, smem, s>>>(maps, 0, R, 0, error_word(), ck, gen2);
  }
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = (lr.P + 255) / 256;
  const unsigned ag = (unsigned)(blocks < (long long)sms * 8 ? blocks : (long long)sms * 8);
  wml_assemble_ragged<T><<<ag, 256, 0, s>>>(rel, ra, rb, rc, rd, lr.roff, lr.L, lr.P);
  BucketTicket sk;
  sk.kinds = kinds;
  sk.want = 1;
  e = launch_wmc_ragged<T>(0, ra, rb, rc, rd, nullptr, rd, nullptr, nullptr, nullptr, lr.roff, nullptr, lr.L,
                           (lr.Pmax + M - 1) / M, nullptr, s, kinds ? &sk : nullptr, lr.l_sys);
  if (e != cudaSuccess) return e;
  if (mode == 1)
    wmc_kernel<T, 3, true, true><<<lr.C, R, smem, s>>>(maps, 0, R, 0, error_word(), ck, gen);
  else
    wmc_kernel<T, 3, true, false><<<lr.C, R, smem, s>>>(maps, 0, R, 0, error_word(), ck, gen);
  return cudaGetLastError();
}

template size_t wml_ragged_workspace_elems<float>(long long);
template size_t wml_ragged_workspace_elems<double>(long long);
template cudaError_t launch_wml_ragged<float>(int, const float*, const float*, const float*, const float*,
                                              const float*, float*, float*, float*, float*, const long long*,
                                              const WmlRagged&, float*, int*, cudaStream_t,
                                              const unsigned char*, const RaggedCheck*);
template cudaError_t launch_wml_ragged<double>(int, const double*, const double*, const double*, const double*,
                                               const double*, double*, double*, double*, double*, const long long*,
                                               const WmlRagged&, double*, int*, cudaStream_t,
                                               const unsigned char*, const RaggedCheck*);

template cudaError_t launch_wmc_ragged<float>(int, const float*, const float*, const float*, const float*,
                                              const float*, float*, float*, float*, float*, const long long*,
                                              const int*, int, int, int*, cudaStream_t, const BucketTicket*,
                                              const int*, const RaggedCheck*);
template cudaError_t launch_wmc_ragged<double>(int, const double*, const double*, const double*, const double*,
                                               const double*, double*, double*, double*, double*, const long long*,
                                               const int*, int, int, int*, cudaStream_t, const BucketTicket*,
                                               const int*, const RaggedCheck*);
template bool wmc_gen_eligible<float>(int, int);
template bool wmc_gen_eligible<double>(int, int);
template bool wmc_eligible<float>(int, int);
template bool wmc_eligible<double>(int, int);
template cudaError_t launch_wmc<float>(int, const float*, const float*, const float*, const float*, float*, int, int,
                                       cudaStream_t, bool*);
template cudaError_t launch_wmc<double>(int, const double*, const double*, const double*, const double*, double*,
                                        int, int, cudaStream_t, bool*);

}  // namespace tdg
