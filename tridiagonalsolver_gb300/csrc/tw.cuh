// Framework for two-ended thread-per-system sweeps over TMA-staged tiles.
//
// A CTA owns 32 systems (one per lane) and runs two warps: warp 0 sweeps
// rows [0, m) top-down, warp 1 sweeps rows [m, n) bottom-up ("burn at both
// ends"), the warps meet in a small solve on rows m-1 and m, and then each
// sweeps back outward.  Both sweeps stream tiles of R rows x 32 systems
// (4 KB) through a ring of STAGES slots per warp; every slot holds four tile
// buffers.  Which global array feeds or receives which buffer in each phase
// is declared by the operation (Op) in four small tables; the Op supplies
// the per-tile arithmetic.  Ops whose step finishes a row of the previous
// tile (pivoted elimination looks one row ahead) set DELAY_F / DELAY_B and
// the stores of a tile then trail by one tile.
//
// Ring protocol (per warp, lane 0 issues all TMA):
//   slot k % STAGES holds tile k of the warp's order; its mbarrier counts the
//   bytes of every fill; the lane-wise parity of each slot lives in a
//   register mask.  A slot is refilled only after the bulk store that reads
//   it has finished reading (cp.async.bulk.wait_group.read).  After the
//   forward phase the last STAGES tiles stay resident for the back phase.
#pragma once

#include "common.cuh"
#include "tma.cuh"

namespace tdg {

template <typename T, int L>
struct TileGeom {
  static constexpr int R = 128 / (int)sizeof(T);  // rows per tile
  static constexpr int S = 32;                      // systems per tile
  static constexpr int ELEMS = R * S;
  static constexpr int BYTES = ELEMS * (int)sizeof(T);

  // Address of (row r, system s) in a tile buffer.  CONTIG tiles are
  // [system][row] with the TMA 128-byte swizzle (16-byte chunk index XOR
  // system%8), INTERLEAVED tiles are [row][system].
  __device__ static __forceinline__ T* at(T* base, int r, int s) {
    if (L == INTERLEAVED) return base + r * S + s;
    const int rb = r * (int)sizeof(T);
    const int off = s * 128 + ((((rb >> 4) ^ (s & 7)) << 4) | (rb & 15));
    return reinterpret_cast<T*>(reinterpret_cast<char*>(base) + off);
  }
  __device__ static __forceinline__ int cx(int t, int sb) { return L == INTERLEAVED ? sb * S : t * R; }
  __device__ static __forceinline__ int cy(int t, int sb) { return L == INTERLEAVED ? t * R : sb * S; }
};

// Division helper.  FP64: x/k = x r0 (1 + e + e^2) with r0 the MUFU seed and
// e = 1 - k r0, which keeps the dependent chain at one MUFU + three FMAs
// (the quotient x r0 is formed in parallel).  FP32: MUFU reciprocal.
template <typename T>
struct Div;
template <>
struct Div<double> {
  double r0, t;
  __device__ __forceinline__ explicit Div(double k) {
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(k));
    const double e = fma(-k, r0, 1.0);
    t = fma(e, e, e);
  }
  __device__ __forceinline__ double div(double x) const {
    const double q = x * r0;
    return fma(q, t, q);
  }
  __device__ __forceinline__ double inv() const { return fma(r0, t, r0); }
};
template <>
struct Div<float> {
  float r;
  __device__ __forceinline__ explicit Div(float k) { r = rcp(k); }
  __device__ __forceinline__ float div(float x) const { return x * r; }
  __device__ __forceinline__ float inv() const { return r; }
};

constexpr int TW_MAXMAP = 11;

// Buffer tables: for each warp (top, bottom) and tile buffer 0..3, the index
// of the tensor map that feeds or receives it, packed 4 bits per entry
// (15 = none).
constexpr unsigned long long tw_e(int x) { return x < 0 ? 15ull : (unsigned long long)x; }
constexpr unsigned long long tw_table(int t0, int t1, int t2, int t3, int b0, int b1, int b2, int b3) {
  return tw_e(t0) | tw_e(t1) << 4 | tw_e(t2) << 8 | tw_e(t3) << 12 | tw_e(b0) << 16 | tw_e(b1) << 20 |
         tw_e(b2) << 24 | tw_e(b3) << 28;
}
__host__ __device__ constexpr int tw_entry(unsigned long long tab, int w, int b) {
  return (int)((tab >> ((w * 4 + b) * 4)) & 15ull);
}
struct TwMaps {
  CUtensorMap m[TW_MAXMAP];
};

template <typename T, int L, int STAGES>
struct TwSmem {
  using G = TileGeom<T, L>;
  struct alignas(1024) Slot {
    T buf[4][G::ELEMS];
  };
  Slot slot[2][STAGES];
  uint64_t bar[2][STAGES];
  T meet[2][8][32];  // per warp, up to 8 values per lane exchanged at the meeting
  int dead[2];
};

template <typename T, int L, int STAGES>
constexpr size_t tw_smem_bytes() {
  return sizeof(TwSmem<T, L, STAGES>) + 1024;  // + alignment slack
}

// Per-lane view of one tile slot.
template <typename T, int L>
struct TileRef {
  T* buf[4];
  __device__ __forceinline__ T& operator()(int k, int r, int lane) const {
    return *TileGeom<T, L>::at(buf[k], r, lane);
  }
};

// ---------------------------------------------------------------------------
// The kernel skeleton.  Op must provide:
//   static constexpr unsigned long long FLOAD, FSTORE, BLOAD, BRES, BSTORE;
//       (tw_table: map index per warp and buffer, -1 = none)
//       (BRES: loads needed even for tiles still resident after phase F)
//   static constexpr bool DELAY_F, DELAY_B;
//   struct State;  struct Args;
//   fwd(w, State&, cur, prev, t, k, K, lane, j, n, m, Args)   -- phase F tile
//   meet(w, State&, T* mine[8] (write), T* top[8], T* bot[8], lane, j, n, m, Args)
//     is split in two: meet_put (before the CTA barrier) and meet_get (after).
//   back(w, State&, cur, prev, t, k, K, lane, j, n, m, Args) -- phase B tile
//   back_finish(w, State&, tile0, lane, j, n, m, Args)      -- pending rows
template <typename T, int L, int STAGES, class Op>
__global__ void __launch_bounds__(64, 1)
    tw_kernel(const __grid_constant__ TwMaps maps, const typename Op::Args args, int n, int batch, int* err) {
  using G = TileGeom<T, L>;
  using Sm = TwSmem<T, L, STAGES>;
  extern __shared__ unsigned char smem_raw[];
  Sm& sm = *reinterpret_cast<Sm*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int sb = blockIdx.x;
  const int j = sb * 32 + lane;  // this lane's system (may be >= batch)
  const int T_ = (n + G::R - 1) / G::R;
  // split on a tile boundary that is also a multiple of 32 rows (pivot words)
  int tm = T_ / 2;
  if (G::R < 32) tm &= ~(32 / G::R - 1);
  const int m = tm * G::R;
  const int K = w == 0 ? tm : T_ - tm;
  auto tile_of = [&](int k) { return w == 0 ? k : T_ - 1 - k; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&sm.bar[0][s], 1);
      mbar_init(&sm.bar[1][s], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();

  auto ref = [&](int q) {
    TileRef<T, L> r;
#pragma unroll
    for (int b = 0; b < 4; ++b) r.buf[b] = sm.slot[w][q].buf[b];
    return r;
  };
  auto issue_loads = [&](unsigned long long tab, int k, int q) {
    int cnt = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) cnt += tw_entry(tab, w, b) != 15;
    if (cnt == 0) return false;
    const int t = tile_of(k);
    mbar_arrive_expect_tx(&sm.bar[w][q], cnt * G::BYTES);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int e = tw_entry(tab, w, b);
      if (e != 15) tma_load_2d(sm.slot[w][q].buf[b], &maps.m[e], G::cx(t, sb), G::cy(t, sb), &sm.bar[w][q]);
    }
    return true;
  };
  auto issue_stores = [&](unsigned long long tab, int k, int q) {
    const int t = tile_of(k);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int e = tw_entry(tab, w, b);
      if (e != 15) tma_store_2d(&maps.m[e], G::cx(t, sb), G::cy(t, sb), sm.slot[w][q].buf[b]);
    }
    bulk_commit();
  };
  auto has = [&](unsigned long long tab) {
    int c = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) c += tw_entry(tab, w, b) != 15;
    return c > 0;
  };

  typename Op::State st;
  Op::init(w, st, lane, j, n, m, args);
  unsigned parity = 0;
  bool dead = false;

  if (lane == 0)
    for (int k = 0; k < K && k < STAGES; ++k) issue_loads(Op::FLOAD, k, k);

  // ---- phase F: toward the middle
  for (int k = 0; k < K; ++k) {
    const int q = k % STAGES;
    bool ok = dead ? false : mbar_wait(&sm.bar[w][q], (parity >> q) & 1u, err);
    parity ^= 1u << q;
    dead = !__all_sync(FULL, ok);
    if (dead) break;
    Op::fwd(w, st, ref(q), ref((k + STAGES - 1) % STAGES), tile_of(k), k, K, lane, j, n, m, args);
    fence_async_smem();
    __syncwarp();
    if (lane == 0) {
      if (!Op::DELAY_F) {
        issue_stores(Op::FSTORE, k, q);
        if (k >= 1 && k - 1 + STAGES < K) {
          bulk_wait_read<1>();
          issue_loads(Op::FLOAD, k - 1 + STAGES, (k - 1) % STAGES);
        }
      } else {
        if (k >= 1) issue_stores(Op::FSTORE, k - 1, (k - 1) % STAGES);
        if (k >= 2 && k - 2 + STAGES < K) {
          bulk_wait_read<1>();
          issue_loads(Op::FLOAD, k - 2 + STAGES, (k - 2) % STAGES);
        }
      }
    }
  }
  if (lane == 0) {
    if (Op::DELAY_F && K >= 1 && !dead) issue_stores(Op::FSTORE, K - 1, (K - 1) % STAGES);
    bulk_wait_all();
    fence_async_global();
  }
  __syncwarp();

  // ---- meet: both warps always arrive, also after a timeout
  Op::meet_put(w, st, sm.meet[w], lane, j, n, m, args);
  if (lane == 0) sm.dead[w] = dead ? 1 : 0;
  __syncthreads();
  dead = sm.dead[0] || sm.dead[1];
  Op::meet_get(w, st, sm.meet[0], sm.meet[1], lane, j, n, m, args);

  // loads the back phase needs even for resident tiles
  const bool need_res = has(Op::BRES);
  if (lane == 0 && !dead && need_res)
    for (int k = K - 1; k >= 0 && k >= K - STAGES; --k) issue_loads(Op::BRES, k, k % STAGES);

  // ---- phase B: outward
  for (int k = K - 1; k >= 0 && !dead; --k) {
    const int q = k % STAGES;
    const bool resident = k >= K - STAGES;
    if (!resident || need_res) {
      bool ok = mbar_wait(&sm.bar[w][q], (parity >> q) & 1u, err);
      parity ^= 1u << q;
      dead = !__all_sync(FULL, ok);
      if (dead) break;
    }
    Op::back(w, st, ref(q), ref((k + 1) % STAGES), tile_of(k), k, K, lane, j, n, m, args);
    fence_async_smem();
    __syncwarp();
    if (lane == 0) {
      if (!Op::DELAY_B) {
        issue_stores(Op::BSTORE, k, q);
        const int kp = k + 1;
        if (kp <= K - 1 && kp - STAGES >= 0) {
          bulk_wait_read<1>();
          issue_loads(Op::BLOAD, kp - STAGES, kp % STAGES);
        }
      } else {
        if (k + 1 <= K - 1) issue_stores(Op::BSTORE, k + 1, (k + 1) % STAGES);
        const int kp = k + 2;
        if (kp <= K - 1 && kp - STAGES >= 0) {
          bulk_wait_read<1>();
          issue_loads(Op::BLOAD, kp - STAGES, kp % STAGES);
        }
      }
    }
  }
  if (Op::DELAY_B && K >= 1 && !dead) {
    Op::back_finish(w, st, ref(0), lane, j, n, m, args);
    fence_async_smem();
    __syncwarp();
    if (lane == 0) issue_stores(Op::BSTORE, 0, 0);
  }
  if (lane == 0) bulk_wait_all();
}

}  // namespace tdg
