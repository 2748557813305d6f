// Two-ended TMA-staged sweeps (see tw.cuh): Thomas, partial-pivoting
// elimination, and the adjoint of the pivoted solve, for the CONTIG and
// INTERLEAVED layouts.
//
// Reference: Thomas_kernel, Tridiagonal_CUDA/tridiagonal_basic.cu:4-30; the
// pivoted sweep follows LAPACK ?gtsv, the algorithm of the reference's MKL
// row (Tridiagonal_AVX512/tridiagonal_basic.cpp:131-143).
#include "kernels.h"
#include "tw.cuh"

namespace tdg {

// Rows of a tile are processed in chunks of CH: chunk c+1 is read from shared
// memory before the arithmetic of chunk c, so load latency stays off the
// recurrence.
constexpr int CH = 8;

template <typename T, int L>
struct Rows4 {
  T v[4][CH];
  template <class Ref, class RowFn>
  __device__ __forceinline__ void load(const Ref& cur, int c0, int lane, RowFn row) {
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = row(c0 + u);
#pragma unroll
      for (int b = 0; b < 4; ++b) v[b][u] = cur(b, r, lane);
    }
  }
};

// ===========================================================================
// Thomas.  Maps: 0 a, 1 b, 2 c, 3 d.
//   top    (rows < m):  c'_i = c_i / k_i, d'_i = (d_i - a_i d'_{i-1}) / k_i,
//                       k_i = b_i - a_i c'_{i-1};   x_i = d'_i - c'_i x_{i+1}
//   bottom (rows >= m): a''_i = a_i / k_i, d''_i = (d_i - c_i d''_{i+1}) / k_i,
//                       k_i = b_i - c_i a''_{i+1};  x_i = d''_i - a''_i x_{i-1}
//   meet: x_{m-1} = (d'_{m-1} - c'_{m-1} d''_m) / (1 - c'_{m-1} a''_m),
//         x_m = d''_m - a''_m x_{m-1}.
// c'/a'' go to c and d'/d'' to d (the reference's in-place contract), then
// d is overwritten with x.
template <typename T, int L>
struct ThomasOp {
  using G = TileGeom<T, L>;
  using Ref = TileRef<T, L>;
  static constexpr unsigned long long FLOAD = tw_table(0, 1, 2, 3, 0, 1, 2, 3);
  static constexpr unsigned long long FSTORE = tw_table(-1, -1, 2, 3, -1, -1, 2, 3);
  static constexpr unsigned long long BLOAD = tw_table(-1, -1, 2, 3, -1, -1, 2, 3);
  static constexpr unsigned long long BRES = tw_table(-1, -1, -1, -1, -1, -1, -1, -1);
  static constexpr unsigned long long BSTORE = tw_table(-1, -1, -1, 3, -1, -1, -1, 3);
  static constexpr bool DELAY_F = false, DELAY_B = false;
  struct Args {
    int batch;
  };
  struct State {
    T cp, dp, x, xm1, xm;
  };
  static __device__ __forceinline__ void init(int, State& s, int, int, int, int, const Args&) {
    s.cp = T(0);
    s.dp = T(0);
  }
  static __device__ __forceinline__ void fwd(int w, State& s, const Ref& cur, const Ref&, int t, int, int, int lane,
                                             int, int n, int, const Args&) {
    constexpr int R = G::R;
    auto row = [&](int idx) { return w == 0 ? idx : R - 1 - idx; };
    Rows4<T, L> X, NX;
    X.load(cur, 0, lane, row);
#pragma unroll
    for (int c0 = 0; c0 < R; c0 += CH) {
      if (c0 + CH < R) NX.load(cur, c0 + CH, lane, row);
      T oc[CH], od[CH];
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int i = t * R + row(c0 + u);
        if (w == 0) {
          const T ai = i == 0 ? T(0) : X.v[0][u];
          const Div<T> q(fma(-ai, s.cp, X.v[1][u]));
          s.cp = q.div(X.v[2][u]);
          s.dp = q.div(fma(-ai, s.dp, X.v[3][u]));
        } else if (i < n) {
          const T ai = i == 0 ? T(0) : X.v[0][u];
          const T ci = i == n - 1 ? T(0) : X.v[2][u];
          const Div<T> q(fma(-ci, s.cp, X.v[1][u]));
          s.cp = q.div(ai);
          s.dp = q.div(fma(-ci, s.dp, X.v[3][u]));
        }
        oc[u] = s.cp;
        od[u] = s.dp;
      }
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int r = row(c0 + u);
        cur(2, r, lane) = oc[u];
        cur(3, r, lane) = od[u];
      }
      if (c0 + CH < R) X = NX;
    }
  }
  static __device__ __forceinline__ void meet_put(int, State& s, T (*mine)[32], int lane, int, int, int,
                                                  const Args&) {
    mine[0][lane] = s.cp;
    mine[1][lane] = s.dp;
  }
  static __device__ __forceinline__ void meet_get(int w, State& s, T (*top)[32], T (*bot)[32], int lane, int, int,
                                                  int, const Args&) {
    const T cm1 = top[0][lane], dm1 = top[1][lane];  // 0, 0 when the top half is empty
    const T am = bot[0][lane], dm = bot[1][lane];
    const Div<T> q(fma(-cm1, am, T(1)));
    s.xm1 = q.div(fma(-cm1, dm, dm1));
    s.xm = fma(-am, s.xm1, dm);
    s.x = w == 0 ? s.xm1 : s.xm;
  }
  static __device__ __forceinline__ void back(int w, State& s, const Ref& cur, const Ref&, int t, int, int, int lane,
                                              int, int n, int m, const Args&) {
    constexpr int R = G::R;
    auto row = [&](int idx) { return w == 0 ? R - 1 - idx : idx; };
#pragma unroll
    for (int c0 = 0; c0 < R; c0 += CH) {
      T C[CH], D[CH], ox[CH];
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int r = row(c0 + u);
        C[u] = cur(2, r, lane);
        D[u] = cur(3, r, lane);
      }
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int i = t * R + row(c0 + u);
        if (w == 0) {
          s.x = (i == m - 1) ? s.xm1 : fma(-C[u], s.x, D[u]);
        } else if (i < n) {
          s.x = (i == m) ? s.xm : fma(-C[u], s.x, D[u]);
        }
        ox[u] = s.x;
      }
#pragma unroll
      for (int u = 0; u < CH; ++u) cur(3, row(c0 + u), lane) = ox[u];
    }
  }
  static __device__ __forceinline__ void back_finish(int, State&, const Ref&, int, int, int, int, const Args&) {}
};

// ===========================================================================
// Shared pieces of the pivoted sweeps.

// One elimination step with partial pivoting.  The carried row is
// (u0 on the pivot unknown, u1 on the next one, rhs); the incoming row has
// `sub` on the pivot unknown, `dg` on the next, `far` one further, rhs `dn`.
// Rows are swapped when |u0| < |sub| (LAPACK's rule: ties keep the rows).
// The finished row is (U0 = p, U1, U2 = sw ? far : 0, RHS); the carried row
// becomes the reduced incoming row.  Returns the swap bit.
template <typename T>
struct PivStep {
  T mlt, rinv, U1, RHS;
  bool sw, singular;
  __device__ __forceinline__ void run(T& u0, T& u1, T& rhs, T sub, T dg, T far, T dn) {
    sw = !abs_ge(u0, sub);
    const T p = sw ? sub : u0;
    const T q = sw ? u0 : sub;
    singular = is_zero(p);
    const Div<T> dv(p);
    mlt = dv.div(q);
    rinv = dv.inv();
    U1 = sw ? dg : u1;
    RHS = sw ? dn : rhs;
    const T nu0 = fma(-mlt, sw ? dg : u1, sw ? u1 : dg);
    const T nu1 = sw ? -mlt * far : far;
    const T nrhs = fma(-mlt, sw ? dn : rhs, sw ? rhs : dn);
    u0 = nu0;
    u1 = nu1;
    rhs = nrhs;
  }
  // factor only (no right-hand side), with the swap given
  __device__ __forceinline__ void refactor(T& u0, T& u1, T sub, T dg, T far, bool s) {
    sw = s;
    const T p = sw ? sub : u0;
    const T q = sw ? u0 : sub;
    const Div<T> dv(p);
    mlt = dv.div(q);
    rinv = dv.inv();
    U1 = sw ? dg : u1;
    const T nu0 = fma(-mlt, sw ? dg : u1, sw ? u1 : dg);
    const T nu1 = sw ? -mlt * far : far;
    u0 = nu0;
    u1 = nu1;
  }
};

// Pivot record writer: bit i%32 of word i/32; word w of system j at
// piv[w*batch + j].  A lane keeps the word it is filling in a register.
struct BitWriter {
  int cw;
  unsigned word;
  __device__ __forceinline__ void init() {
    cw = -1;
    word = 0;
  }
  __device__ __forceinline__ void flush(unsigned* piv, int j, int batch) {
    if (cw >= 0 && j < batch) piv[(size_t)cw * batch + j] = word;
  }
  __device__ __forceinline__ void set(unsigned* piv, int i, bool b, int j, int batch) {
    const int wi = i >> 5;
    if (wi != cw) {
      flush(piv, j, batch);
      cw = wi;
      word = 0;
    }
    word |= (unsigned)b << (i & 31);
  }
};

struct BitReader {
  int cw;
  unsigned word;
  __device__ __forceinline__ void init() { cw = -1; word = 0; }
  __device__ __forceinline__ bool get(const unsigned* piv, int i, int j, int batch) {
    const int wi = i >> 5;
    if (wi != cw) {
      cw = wi;
      word = j < batch ? piv[(size_t)wi * batch + j] : 0u;
    }
    return (word >> (i & 31)) & 1u;
  }
};

// ===========================================================================
// Pivoted solve.  Maps: 0 a, 1 b, 2 c, 3 d (rhs in, x out), 4 w1 (U1),
// 5 w2 (1/U0).  Top warp: step finishing row i with row i+1 (sub = a_{i+1},
// far = c_{i+1}); bottom warp: the mirror image (sub = c_{i-1},
// far = a_{i-1}).  A finished row keeps (U1, 1/U0, RHS) in buffers
// (0 | 2), 1, 3 of its tile; the top keeps c and the bottom keeps a in the
// remaining buffer for U2 in the back sweep.  Meeting: the two carried rows
// form a 2x2 system on (x_{m-1}, x_m), solved with partial pivoting; its
// swap is recorded as bit m-1.
template <typename T, int L>
struct GtsvOp {
  using G = TileGeom<T, L>;
  using Ref = TileRef<T, L>;
  static constexpr unsigned long long FLOAD = tw_table(0, 1, 2, 3, 0, 1, 2, 3);
  static constexpr unsigned long long FSTORE = tw_table(4, 5, -1, 3, -1, 5, 4, 3);
  static constexpr unsigned long long BLOAD = tw_table(4, 5, 2, 3, 0, 5, 4, 3);
  static constexpr unsigned long long BRES = tw_table(-1, -1, -1, -1, -1, -1, -1, -1);
  static constexpr unsigned long long BSTORE = tw_table(-1, -1, -1, 3, -1, -1, -1, 3);
  static constexpr bool DELAY_F = true, DELAY_B = false;
  struct Args {
    unsigned* piv;
    int* info;
    int batch;
  };
  struct State {
    T u0, u1, rhs;      // carried (unfinished) row
    T x, x2, keep;      // back sweep: x of the previous two rows, kept c/a of the previous row
    T xm1, xm;
    int bad;
    BitWriter bw;
    BitReader br;
  };
  static __device__ __forceinline__ void init(int, State& s, int, int, int, int, const Args&) {
    s.u0 = T(1);
    s.u1 = T(0);
    s.rhs = T(0);
    s.bad = 0;
    s.bw.init();
    s.br.init();
  }
  static __device__ __forceinline__ void fwd(int w, State& s, const Ref& cur, const Ref& prev, int t, int, int,
                                             int lane, int j, int n, int, const Args& g) {
    constexpr int R = G::R;
    auto row = [&](int idx) { return w == 0 ? idx : R - 1 - idx; };
    Rows4<T, L> X, NX;
    X.load(cur, 0, lane, row);
#pragma unroll
    for (int c0 = 0; c0 < R; c0 += CH) {
      if (c0 + CH < R) NX.load(cur, c0 + CH, lane, row);
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int idx = c0 + u;
        const int r = row(idx);
        const int i = t * R + r;  // incoming row
        if (w == 0) {
          if (i == 0) {
            s.u0 = X.v[1][u];
            s.u1 = X.v[2][u];
            s.rhs = X.v[3][u];
          } else {
            PivStep<T> ps;
            ps.run(s.u0, s.u1, s.rhs, X.v[0][u], X.v[1][u], X.v[2][u], X.v[3][u]);
            if (ps.singular && s.bad == 0) s.bad = i;  // finished row i-1 -> k+1 = i
            const Ref& dst = idx > 0 ? cur : prev;
            const int rr = idx > 0 ? r - 1 : R - 1;
            dst(0, rr, lane) = ps.U1;
            dst(1, rr, lane) = ps.rinv;
            dst(3, rr, lane) = ps.RHS;
            s.bw.set(g.piv, i - 1, ps.sw, j, g.batch);
          }
        } else if (i < n) {
          const T ai = i == 0 ? T(0) : X.v[0][u];
          if (i == n - 1) {
            s.u0 = X.v[1][u];
            s.u1 = ai;
            s.rhs = X.v[3][u];
          } else {
            PivStep<T> ps;
            ps.run(s.u0, s.u1, s.rhs, X.v[2][u], X.v[1][u], ai, X.v[3][u]);
            if (ps.singular && s.bad == 0) s.bad = i + 2;  // finished row i+1
            const Ref& dst = idx > 0 ? cur : prev;
            const int rr = idx > 0 ? r + 1 : 0;
            dst(2, rr, lane) = ps.U1;
            dst(1, rr, lane) = ps.rinv;
            dst(3, rr, lane) = ps.RHS;
            s.bw.set(g.piv, i + 1, ps.sw, j, g.batch);
          }
        }
      }
      if (c0 + CH < R) X = NX;
    }
  }
  static __device__ __forceinline__ void meet_put(int w, State& s, T (*mine)[32], int lane, int, int, int m,
                                                  const Args&) {
    const bool empty = (w == 0 && m == 0);  // no top rows: x_{-1} = 0
    mine[0][lane] = empty ? T(1) : s.u0;
    mine[1][lane] = empty ? T(0) : s.u1;
    mine[2][lane] = empty ? T(0) : s.rhs;
    mine[3][lane] = T(s.bad);
  }
  static __device__ __forceinline__ void meet_get(int w, State& s, T (*top)[32], T (*bot)[32], int lane, int j,
                                                  int n, int m, const Args& g) {
    // rows: top (u0t x_{m-1} + u1t x_m = rt), bottom (u1b x_{m-1} + u0b x_m = rb)
    const T u0t = top[0][lane], u1t = top[1][lane], rt = top[2][lane];
    const T u0b = bot[0][lane], u1b = bot[1][lane], rb = bot[2][lane];
    const bool gsw = !abs_ge(u0t, u1b);
    const T p0 = gsw ? u1b : u0t, p1 = gsw ? u0b : u1t, pr = gsw ? rb : rt;  // pivot row
    const T o0 = gsw ? u0t : u1b, o1 = gsw ? u1t : u0b, orr = gsw ? rt : rb;  // other row
    const Div<T> dp(p0);
    const T l = dp.div(o0);
    const T q0 = fma(-l, p1, o1);
    const T rq = fma(-l, pr, orr);
    const Div<T> dq(q0);
    s.xm = dq.div(rq);
    s.xm1 = dp.div(fma(-p1, s.xm, pr));
    const bool sing = is_zero(p0) || is_zero(q0);
    if (w == 0) {
      if (m > 0) {
        s.bw.set(g.piv, m - 1, gsw, j, g.batch);
        s.bw.flush(g.piv, j, g.batch);
      }
      const int bt = (int)top[3][lane], bb = (int)bot[3][lane];
      if (g.info && j < g.batch) g.info[j] = bt ? bt : (sing ? (m > 0 ? m : 1) : bb);
      s.x = s.xm1;  // x_{i+1} for row m-2
      s.x2 = s.xm;  // x_{i+2}
    } else {
      s.bw.flush(g.piv, j, g.batch);
      s.x = s.xm;   // x_{i-1} for row m+1
      s.x2 = s.xm1; // x_{i-2}
    }
    (void)n;
  }
  static __device__ __forceinline__ void back(int w, State& s, const Ref& cur, const Ref&, int t, int, int, int lane,
                                              int j, int n, int m, const Args& g) {
    constexpr int R = G::R;
    auto row = [&](int idx) { return w == 0 ? R - 1 - idx : idx; };
#pragma unroll
    for (int c0 = 0; c0 < R; c0 += CH) {
      Rows4<T, L> X;
      X.load(cur, c0, lane, row);
      T ox[CH];
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int i = t * R + row(c0 + u);
        if (w == 0) {
          // buffers: 0 U1, 1 1/U0, 2 c (kept), 3 RHS
          if (i == m - 1) {
            ox[u] = s.xm1;
          } else {
            const bool sw = s.br.get(g.piv, i, j, g.batch);
            const T u2 = sw ? s.keep : T(0);  // c_{i+1}
            const T xi = fma(-u2, s.x2, fma(-X.v[0][u], s.x, X.v[3][u])) * X.v[1][u];
            s.x2 = s.x;
            s.x = xi;
            ox[u] = xi;
          }
          s.keep = X.v[2][u];
        } else if (i < n) {
          // buffers: 0 a (kept), 1 1/U0, 2 U1, 3 RHS
          if (i == m) {
            ox[u] = s.xm;
          } else {
            const bool sw = s.br.get(g.piv, i, j, g.batch);
            const T u2 = sw ? s.keep : T(0);  // a_{i-1}
            const T xi = fma(-u2, s.x2, fma(-X.v[2][u], s.x, X.v[3][u])) * X.v[1][u];
            s.x2 = s.x;
            s.x = xi;
            ox[u] = xi;
          }
          s.keep = i == 0 ? T(0) : X.v[0][u];
        } else {
          ox[u] = T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < CH; ++u) cur(3, row(c0 + u), lane) = ox[u];
    }
  }
  static __device__ __forceinline__ void back_finish(int, State&, const Ref&, int, int, int, int, const Args&) {}
};

// ===========================================================================
// Adjoint of the pivoted solve.  Maps: 0 a, 1 b, 2 c, 3 g (= xbar), 4 w1
// (z spill), 5 w2 (multiplier spill), 6 x, 7 gd, 8 ga, 9 gb, 10 gc.
// With E A = W (E: the elimination steps of both halves and the meeting, W
// twisted triangular), A^T lambda = g is W^T z = g, lambda = E^T z.
// Phase F re-factors with the recorded pivots and solves the top part of
// W^T z = g top-down and the bottom part bottom-up (spilling z and the
// multipliers); the meeting closes z_{m-1}, z_m and applies the meeting
// step's transpose; phase B applies the transposed steps outward, which
// finishes lambda_i one row behind, and emits the gradients.
template <typename T, int L>
struct AdjOp {
  using G = TileGeom<T, L>;
  using Ref = TileRef<T, L>;
  static constexpr unsigned long long FLOAD = tw_table(0, 1, 2, 3, 0, 1, 2, 3);
  static constexpr unsigned long long FSTORE = tw_table(4, 5, -1, -1, 4, 5, -1, -1);
  static constexpr unsigned long long BLOAD = tw_table(4, 5, 6, -1, 4, 5, 6, -1);
  static constexpr unsigned long long BRES = tw_table(-1, -1, 6, -1, -1, -1, 6, -1);
  static constexpr unsigned long long BSTORE = tw_table(7, 8, 9, 10, 7, 8, 9, 10);
  static constexpr bool DELAY_F = true, DELAY_B = true;
  struct Args {
    const unsigned* piv;
    const T* x;  // for the two rows next to the meeting
    int batch;
    int n;
  };
  struct State {
    T u0, u1, gcur;        // carried row and its g
    T z1, z2;              // z one and two rows back
    T P1, P2, P2b;         // U1 one row back, U2 one and two rows back
    T lam;                 // carried lambda entry
    T x1, x2;              // x one and two rows back
    BitReader br;
  };
  static __device__ __forceinline__ size_t off(int i, int j, const Args& g) {
    return idx<L>(i, j, g.n, g.batch);
  }
  static __device__ __forceinline__ void init(int, State& s, int, int, int, int, const Args&) {
    s.u0 = T(1);
    s.u1 = T(0);
    s.gcur = T(0);
    s.z1 = s.z2 = s.P1 = s.P2 = s.P2b = T(0);
    s.br.init();
  }
  static __device__ __forceinline__ void fwd(int w, State& s, const Ref& cur, const Ref& prev, int t, int, int,
                                             int lane, int j, int n, int, const Args& g) {
    constexpr int R = G::R;
    auto row = [&](int idx) { return w == 0 ? idx : R - 1 - idx; };
    Rows4<T, L> X, NX;
    X.load(cur, 0, lane, row);
#pragma unroll
    for (int c0 = 0; c0 < R; c0 += CH) {
      if (c0 + CH < R) NX.load(cur, c0 + CH, lane, row);
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int idx = c0 + u;
        const int r = row(idx);
        const int i = t * R + r;  // incoming row
        const bool first = w == 0 ? (i == 0) : (i == n - 1);
        if (w == 1 && i >= n) continue;
        const T ai = i == 0 ? T(0) : X.v[0][u];
        if (first) {
          s.u0 = X.v[1][u];
          s.u1 = w == 0 ? X.v[2][u] : ai;
          s.gcur = X.v[3][u];
          continue;
        }
        const int fin = w == 0 ? i - 1 : i + 1;  // row being finished
        const bool sw = s.br.get(g.piv, fin, j, g.batch);
        PivStep<T> ps;
        if (w == 0)
          ps.refactor(s.u0, s.u1, ai, X.v[1][u], X.v[2][u], sw);
        else
          ps.refactor(s.u0, s.u1, X.v[2][u], X.v[1][u], ai, sw);
        const T U2 = sw ? (w == 0 ? X.v[2][u] : ai) : T(0);
        // z_fin = (g_fin - U1_{prev} z_{prev} - U2_{prev2} z_{prev2}) / U0_fin
        const T z = fma(-s.P2b, s.z2, fma(-s.P1, s.z1, s.gcur)) * ps.rinv;
        const Ref& dst = idx > 0 ? cur : prev;
        const int rr = idx > 0 ? (w == 0 ? r - 1 : r + 1) : (w == 0 ? R - 1 : 0);
        dst(0, rr, lane) = z;
        dst(1, rr, lane) = ps.mlt;
        s.z2 = s.z1;
        s.z1 = z;
        s.P2b = s.P2;
        s.P2 = U2;
        s.P1 = ps.U1;
        s.gcur = X.v[3][u];
      }
      if (c0 + CH < R) X = NX;
    }
  }
  // Meeting data per lane: 0 u0, 1 u1, 2 g, 3 s1 (partial sum entering the
  // far row: top U1 z + U2 z for row m-1; bottom V2 z for row m-1),
  // 4 s2 (partial sum entering the near-other row).
  static __device__ __forceinline__ void meet_put(int w, State& s, T (*mine)[32], int lane, int, int, int m,
                                                  const Args&) {
    const bool empty = (w == 0 && m == 0);
    mine[0][lane] = empty ? T(1) : s.u0;
    mine[1][lane] = empty ? T(0) : s.u1;
    mine[2][lane] = empty ? T(0) : s.gcur;
    if (w == 0) {
      mine[3][lane] = empty ? T(0) : fma(s.P1, s.z1, s.P2b * s.z2);  // into z_{m-1}
      mine[4][lane] = empty ? T(0) : s.P2 * s.z1;                    // into z_m
    } else {
      mine[3][lane] = s.P2 * s.z1;                    // into z_{m-1}: V2_{m+1} z_{m+1}
      mine[4][lane] = fma(s.P1, s.z1, s.P2b * s.z2);  // into z_m: V1_{m+1} z_{m+1} + V2_{m+2} z_{m+2}
    }
  }
  static __device__ __forceinline__ void meet_get(int w, State& s, T (*top)[32], T (*bot)[32], int lane, int j,
                                                  int n, int m, const Args& g) {
    const T u0t = top[0][lane], u1t = top[1][lane], gt = top[2][lane], st1 = top[3][lane], st2 = top[4][lane];
    const T u0b = bot[0][lane], u1b = bot[1][lane], gb_ = bot[2][lane], sb1 = bot[3][lane], sb2 = bot[4][lane];
    const bool gsw = m > 0 ? s.br.get(g.piv, m - 1, j, g.batch) : false;
    const T p0 = gsw ? u1b : u0t, p1 = gsw ? u0b : u1t;
    const T o0 = gsw ? u0t : u1b, o1 = gsw ? u1t : u0b;
    const Div<T> dp(p0);
    const T l = dp.div(o0);
    const T q0 = fma(-l, p1, o1);
    // W^T rows m-1 and m
    const T zm1 = dp.div(gt - st1 - sb1);
    const T zm = (gb_ - st2 - sb2 - p1 * zm1) * Div<T>(q0).inv();
    // meeting step transposed: v_{m-1} -= l v_m, then swap
    T vm1 = fma(-l, zm, zm1), vm = zm;
    if (gsw) {
      const T tmp = vm1;
      vm1 = vm;
      vm = tmp;
    }
    s.lam = w == 0 ? vm1 : vm;
    // x next to the meeting (the other half's row)
    if (w == 0) {
      s.x2 = (m > 0 && j < g.batch) ? g.x[off(m, j, g)] : T(0);  // x_m
    } else {
      s.x2 = (m > 0 && j < g.batch) ? g.x[off(m - 1, j, g)] : T(0);  // x_{m-1}
    }
    s.br.init();
    (void)n;
  }
  // Phase B.  Top (rows upward from m-1): step i (i <= m-2) applies
  // E_i^T to entries (i, i+1), which finalises lambda_{i+1}; its gradients
  // go to row i+1.  Bottom (rows downward from m): step i (i >= m+1) applies
  // F_i^T to (i, i-1) and finalises lambda_{i-1}.
  static __device__ __forceinline__ void back(int w, State& s, const Ref& cur, const Ref& prev, int t, int, int,
                                              int lane, int j, int n, int m, const Args& g) {
    constexpr int R = G::R;
    auto row = [&](int idx) { return w == 0 ? R - 1 - idx : idx; };
#pragma unroll
    for (int c0 = 0; c0 < R; c0 += CH) {
      T Z[CH], M[CH], XX[CH];
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int r = row(c0 + u);
        Z[u] = cur(0, r, lane);
        M[u] = cur(1, r, lane);
        XX[u] = cur(2, r, lane);
      }
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        const int idx = c0 + u;
        const int r = row(idx);
        const int i = t * R + r;
        if (w == 1 && i >= n) continue;
        const bool first = w == 0 ? (i == m - 1) : (i == m);
        if (first) {
          s.x1 = XX[u];
          continue;
        }
        const bool sw = s.br.get(g.piv, i, j, g.batch);
        const T v = fma(-M[u], s.lam, Z[u]);
        const T lam_done = sw ? v : s.lam;  // final entry of the row finished now
        s.lam = sw ? s.lam : v;
        // the finished row is i+1 (top) or i-1 (bottom): the previous row in
        // processing order; neighbours: x(prev) = x1, x(prev's far side) = x2,
        // x(this row) = XX[u]
        const T xnear = XX[u], xrow = s.x1, xfar = s.x2;
        const T ga = w == 0 ? -lam_done * xnear : -lam_done * xfar;
        const T gcv = w == 0 ? -lam_done * xfar : -lam_done * xnear;
        const Ref& dst = idx > 0 ? cur : prev;
        const int rr = idx > 0 ? (w == 0 ? r + 1 : r - 1) : (w == 0 ? 0 : R - 1);
        const int fin = w == 0 ? i + 1 : i - 1;
        dst(0, rr, lane) = lam_done;
        dst(1, rr, lane) = fin == 0 ? T(0) : ga;
        dst(2, rr, lane) = -lam_done * xrow;
        dst(3, rr, lane) = fin == n - 1 ? T(0) : gcv;
        s.x2 = s.x1;
        s.x1 = xnear;
      }
    }
  }
  // the last row in processing order (row 0 for the top, row n-1 for the
  // bottom) takes the carried lambda
  static __device__ __forceinline__ void back_finish(int w, State& s, const Ref& tile0, int lane, int, int n, int,
                                                     const Args&) {
    constexpr int R = G::R;
    const int i = w == 0 ? 0 : n - 1;
    const int r = i - (w == 0 ? 0 : ((n - 1) / R) * R);
    const T lam = s.lam;
    tile0(0, r, lane) = lam;
    tile0(1, r, lane) = (w == 0 || i == 0) ? T(0) : -lam * s.x2;  // ga = -lam x_{i-1}
    tile0(2, r, lane) = -lam * s.x1;                              // gb = -lam x_i
    tile0(3, r, lane) = (w == 1 || i == n - 1) ? T(0) : -lam * s.x2;  // gc = -lam x_{i+1}
  }
};

// ===========================================================================
// Host side.

static CUtensorMapDataType tmap_type(const float*) { return CU_TENSOR_MAP_DATA_TYPE_FLOAT32; }
static CUtensorMapDataType tmap_type(const double*) { return CU_TENSOR_MAP_DATA_TYPE_FLOAT64; }

template <typename T, int L>
static bool make_map(CUtensorMap* m, const T* p, int n, int batch) {
  using G = TileGeom<T, L>;
  if (L == INTERLEAVED)
    return encode_tmap_2d(m, p, tmap_type(p), sizeof(T), (uint64_t)batch, (uint64_t)n, (uint64_t)batch * sizeof(T),
                          G::S, G::R, CU_TENSOR_MAP_SWIZZLE_NONE);
  return encode_tmap_2d(m, p, tmap_type(p), sizeof(T), (uint64_t)n, (uint64_t)batch, (uint64_t)n * sizeof(T), G::R,
                        G::S, CU_TENSOR_MAP_SWIZZLE_128B);
}

constexpr int TW_STAGES = 6;

template <typename T, int L, class Op>
static cudaError_t launch_tw(const TwMaps& maps, const typename Op::Args& args, int n, int batch, cudaStream_t s) {
  const size_t smem = tw_smem_bytes<T, L, TW_STAGES>();
  cudaError_t e = cudaFuncSetAttribute(tw_kernel<T, L, TW_STAGES, Op>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((batch + 31) / 32);
  tw_kernel<T, L, TW_STAGES, Op><<<grid, 64, smem, s>>>(maps, args, n, batch, error_word());
  return cudaGetLastError();
}

template <typename T, int L>
static bool maps_for(TwMaps& maps, std::initializer_list<const T*> ptrs, int n, int batch) {
  int k = 0;
  for (const T* p : ptrs) {
    if (!make_map<T, L>(&maps.m[k++], p, n, batch)) return false;
  }
  return true;
}

template <typename T>
cudaError_t launch_thomas_tw(int layout, T* a, T* b, T* c, T* d, int n, int batch, cudaStream_t s, bool* used) {
  *used = false;
  TwMaps maps;
  if (layout == INTERLEAVED) {
    if (!maps_for<T, INTERLEAVED>(maps, {a, b, c, d}, n, batch)) return cudaSuccess;
    *used = true;
    return launch_tw<T, INTERLEAVED, ThomasOp<T, INTERLEAVED>>(maps, {batch}, n, batch, s);
  }
  if (layout == CONTIG) {
    if (!maps_for<T, CONTIG>(maps, {a, b, c, d}, n, batch)) return cudaSuccess;
    *used = true;
    return launch_tw<T, CONTIG, ThomasOp<T, CONTIG>>(maps, {batch}, n, batch, s);
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t launch_gtsv_tw(int layout, const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv,
                           int* info, int n, int batch, cudaStream_t s, bool* used) {
  *used = false;
  TwMaps maps;
  if (layout == INTERLEAVED) {
    if (!maps_for<T, INTERLEAVED>(maps, {a, b, c, d, w1, w2}, n, batch)) return cudaSuccess;
    *used = true;
    return launch_tw<T, INTERLEAVED, GtsvOp<T, INTERLEAVED>>(maps, {piv, info, batch}, n, batch, s);
  }
  if (layout == CONTIG) {
    if (!maps_for<T, CONTIG>(maps, {a, b, c, d, w1, w2}, n, batch)) return cudaSuccess;
    *used = true;
    return launch_tw<T, CONTIG, GtsvOp<T, CONTIG>>(maps, {piv, info, batch}, n, batch, s);
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t launch_gtsv_adjoint_tw(int layout, const T* a, const T* b, const T* c, const T* x, const unsigned* piv,
                                   const T* g, T* ga, T* gb, T* gc, T* gd, T* wz, T* wm, int n, int batch,
                                   cudaStream_t s, bool* used) {
  *used = false;
  TwMaps maps;
  if (layout == INTERLEAVED) {
    if (!maps_for<T, INTERLEAVED>(maps, {a, b, c, g, wz, wm, x, gd, ga, gb, gc}, n, batch)) return cudaSuccess;
    *used = true;
    return launch_tw<T, INTERLEAVED, AdjOp<T, INTERLEAVED>>(maps, {piv, x, batch, n}, n, batch, s);
  }
  if (layout == CONTIG) {
    if (!maps_for<T, CONTIG>(maps, {a, b, c, g, wz, wm, x, gd, ga, gb, gc}, n, batch)) return cudaSuccess;
    *used = true;
    return launch_tw<T, CONTIG, AdjOp<T, CONTIG>>(maps, {piv, x, batch, n}, n, batch, s);
  }
  return cudaSuccess;
}

#define INST(T)                                                                                                   \
  template cudaError_t launch_thomas_tw<T>(int, T*, T*, T*, T*, int, int, cudaStream_t, bool*);                   \
  template cudaError_t launch_gtsv_tw<T>(int, const T*, const T*, const T*, T*, T*, T*, unsigned*, int*, int, int, \
                                         cudaStream_t, bool*);                                                    \
  template cudaError_t launch_gtsv_adjoint_tw<T>(int, const T*, const T*, const T*, const T*, const unsigned*,    \
                                                 const T*, T*, T*, T*, T*, T*, T*, int, int, cudaStream_t, bool*);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
