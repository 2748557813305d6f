// Thread-per-system sweeps: Thomas, Gaussian elimination with partial
// pivoting ("gtsv"), and the adjoint of the pivoted solve.
//
// One thread owns one system and walks it top-down then bottom-up, the
// fewest floating-point operations per equation of any method (Thomas: 8
// FP64 ops, pivoted: 10).  On GB300 that matters: FP64 runs at ~1/50 of the
// FP32 rate and these kernels are FP64-pipe bound at large batch.  In the
// INTERLEAVED layout a warp reads 32 consecutive systems per row, one
// coalesced 256-byte (FP64) line per array; loads run UNROLL rows ahead of
// the dependent recurrence through a register double buffer.
//
// Reference: Thomas_kernel, Tridiagonal_CUDA/tridiagonal_basic.cu:4-30 (one
// thread per system, layout 0).  The pivoted sweep restates LAPACK ?gtsv,
// the reference's only pivoting solver (MKL row,
// Tridiagonal_AVX512/tridiagonal_basic.cpp:131-143).
#include "common.cuh"
#include "kernels.h"

namespace tdg {

// ---------------------------------------------------------------------------
// Thomas: forward sweep stores c' into c and d' into d, back sweep overwrites
// d with x (the reference's in-place contract).

template <typename T, int L, int U>
__global__ void __launch_bounds__(128) thomas_seq_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                         T* __restrict__ c, T* __restrict__ d, int n, int batch) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  T na[U], nb[U], nc[U], nd[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (u < n) {
      size_t o = idx<L>(u, j, n, batch);
      na[u] = (u == 0) ? T(0) : ld_stream(a + o);
      nb[u] = ld_stream(b + o);
      nc[u] = ld_stream(c + o);
      nd[u] = ld_stream(d + o);
    }
  }
  T cp = T(0), dp = T(0);
  for (int i0 = 0; i0 < n; i0 += U) {
    T ra[U], rb[U], rc[U], rd[U];
#pragma unroll
    for (int u = 0; u < U; ++u) { ra[u] = na[u]; rb[u] = nb[u]; rc[u] = nc[u]; rd[u] = nd[u]; }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int i = i0 + U + u;
      if (i < n) {
        size_t o = idx<L>(i, j, n, batch);
        na[u] = ld_stream(a + o);
        nb[u] = ld_stream(b + o);
        nc[u] = ld_stream(c + o);
        nd[u] = ld_stream(d + o);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int i = i0 + u;
      if (i < n) {
        T k = fma(-ra[u], cp, rb[u]);
        T r = rcp(k);
        cp = rc[u] * r;
        dp = fma(-ra[u], dp, rd[u]) * r;
        size_t o = idx<L>(i, j, n, batch);
        st_keep(c + o, cp);
        st_keep(d + o, dp);
      }
    }
  }
  // back sweep: x_i = d'_i - c'_i x_{i+1}
  T x = dp;  // x_{n-1} = d'_{n-1}, already stored
  int top = n - 2;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    int i = top - u;
    if (i >= 0) {
      size_t o = idx<L>(i, j, n, batch);
      nc[u] = ld_keep(c + o);
      nd[u] = ld_keep(d + o);
    }
  }
  for (int i0 = top; i0 >= 0; i0 -= U) {
    T rc[U], rd[U];
#pragma unroll
    for (int u = 0; u < U; ++u) { rc[u] = nc[u]; rd[u] = nd[u]; }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int i = i0 - U - u;
      if (i >= 0) {
        size_t o = idx<L>(i, j, n, batch);
        nc[u] = ld_keep(c + o);
        nd[u] = ld_keep(d + o);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int i = i0 - u;
      if (i >= 0) {
        x = fma(-rc[u], x, rd[u]);
        st_stream(d + idx<L>(i, j, n, batch), x);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Pivoted elimination.  Step i compares the running pivot u0 (row i) with the
// sub-diagonal a_{i+1}; when |u0| < |a_{i+1}| rows i and i+1 are interchanged
// (LAPACK's rule: ties keep the rows).  The finished row i is kept as
//   RHS_i -> d[i], U1_i -> w1[i], 1/U0_i -> w2[i]
// (w1, w2: n * batch elements each, indexed by sidx, for every layout),
// and its second super-diagonal U2_i equals c_{i+1} when the rows were
// swapped, else 0, so only the pivot bit is stored (bit i%32 of word i/32,
// word w of system j at piv[w*batch + j]).  a, b, c are not modified.
// info[j] (optional) receives 0 or k+1 for the first zero pivot U0_k.

template <typename T, int L, int U>
__global__ void __launch_bounds__(128) gtsv_seq_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                       const T* __restrict__ c, T* __restrict__ d,
                                                       T* __restrict__ w1, T* __restrict__ w2,
                                                       unsigned* __restrict__ piv, int* __restrict__ info, int n,
                                                       int batch, const int* __restrict__ mask) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  if (mask && !mask[j]) {  // (masked launch: only the marked systems)
    if (info) info[j] = 0;
    return;
  }
  // row i carried as (u0, u1, rhs); the next row is read from memory
  size_t o0 = idx<L>(0, j, n, batch);
  T u0 = ld_stream(b + o0), u1 = (n > 1) ? ld_stream(c + o0) : T(0), rhs = ld_stream(d + o0);
  int bad = 0;
  unsigned word = 0;
  T na[U], nb[U], nc[U], nd[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    int i = 1 + u;
    if (i < n) {
      size_t o = idx<L>(i, j, n, batch);
      na[u] = ld_stream(a + o);
      nb[u] = ld_stream(b + o);
      nc[u] = (i + 1 < n) ? ld_stream(c + o) : T(0);
      nd[u] = ld_stream(d + o);
    }
  }
  for (int i0 = 0; i0 + 1 < n; i0 += U) {
    T ra[U], rb[U], rc[U], rd[U];
#pragma unroll
    for (int u = 0; u < U; ++u) { ra[u] = na[u]; rb[u] = nb[u]; rc[u] = nc[u]; rd[u] = nd[u]; }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int i = i0 + 1 + U + u;
      if (i < n) {
        size_t o = idx<L>(i, j, n, batch);
        na[u] = ld_stream(a + o);
        nb[u] = ld_stream(b + o);
        nc[u] = (i + 1 < n) ? ld_stream(c + o) : T(0);
        nd[u] = ld_stream(d + o);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u;  // finishing row i, next row i+1 = (ra, rb, rc, rd)[u]
      if (i + 1 < n) {
        const bool sw = !abs_ge(u0, ra[u]);
        const T p = sw ? ra[u] : u0;
        const T q = sw ? u0 : ra[u];
        if (is_zero(p) && bad == 0) bad = i + 1;
        const T r = rcp(p);
        const T m = q * r;
        const T U1 = sw ? rb[u] : u1;
        const T R = sw ? rd[u] : rhs;
        const T nu0 = fma(-m, sw ? rb[u] : u1, sw ? u1 : rb[u]);
        const T nu1 = sw ? -m * rc[u] : rc[u];
        const T nrhs = fma(-m, sw ? rd[u] : rhs, sw ? rhs : rd[u]);
        const size_t so = sidx<L>(i, j, n, batch);
        st_keep(d + idx<L>(i, j, n, batch), R);
        st_keep(w1 + so, U1);
        st_keep(w2 + so, r);
        word |= (unsigned)sw << (i & 31);
        if ((i & 31) == 31) {
          if (piv) piv[(size_t)(i >> 5) * batch + j] = word;
          word = 0;
        }
        u0 = nu0;
        u1 = nu1;
        rhs = nrhs;
      }
    }
  }
  // last row; flush the pivot word of the last step (n-2) unless full
  if (is_zero(u0) && bad == 0) bad = n;
  if (piv && n >= 2 && ((n - 2) & 31) != 31) piv[(size_t)((n - 2) >> 5) * batch + j] = word;
  const T rl = rcp(u0);
  T x1 = rhs * rl;  // x_{n-1}
  st_stream(d + idx<L>(n - 1, j, n, batch), x1);
  if (info) info[j] = bad;
  // back substitution: x_i = (RHS_i - U1_i x_{i+1} - U2_i x_{i+2}) / U0_i
  T x2 = T(0);  // x_{i+2}
  unsigned wcur = 0;
  int wloaded = -1;
  for (int i = n - 2; i >= 0; --i) {
    size_t o = idx<L>(i, j, n, batch);
    const int w = i >> 5;
    if (w != wloaded) {
      wcur = piv[(size_t)w * batch + j];
      wloaded = w;
    }
    // U2_i = c_{i+1} when row i was swapped; only read when needed
    T u2 = T(0);
    const bool sw = (wcur >> (i & 31)) & 1u;
    if (sw && i + 2 < n) u2 = ld_stream(c + idx<L>(i + 1, j, n, batch));
    const size_t so = sidx<L>(i, j, n, batch);
    T R = ld_keep(d + o), U1v = ld_keep(w1 + so), rv = ld_keep(w2 + so);
    T x0 = fma(-U1v, x1, R);
    x0 = fma(-u2, x2, x0) * rv;
    st_stream(d + o, x0);
    x2 = x1;
    x1 = x0;
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the pivoted solve: lambda = A^{-T} xbar, grads of L = <xbar, x>.
// Top-down: re-factor A with the forward sweep's pivot bits (bit-identical
// factors) and solve U^T z = xbar on the fly; spill z and the multipliers m.
// Bottom-up: lambda = E_0^T ... E_{n-2}^T z (z_i -= m_i z_{i+1}, then swap
// entries i, i+1 if rows were interchanged at step i), emitting
//   gd_i = lambda_i, ga_i = -lambda_i x_{i-1}, gb_i = -lambda_i x_i,
//   gc_i = -lambda_i x_{i+1}.

template <typename T, int L>
__global__ void __launch_bounds__(128) gtsv_adjoint_seq_kernel(
    const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c, const T* __restrict__ x,
    const unsigned* __restrict__ piv, const T* __restrict__ g, T* __restrict__ ga, T* __restrict__ gb,
    T* __restrict__ gc, T* __restrict__ gd, T* __restrict__ wz, T* __restrict__ wm, int n, int batch) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= batch) return;
  size_t o0 = idx<L>(0, j, n, batch);
  T u0 = ld_stream(b + o0), u1 = (n > 1) ? ld_stream(c + o0) : T(0);
  // U^T z = g: z_i = (g_i - U1_{i-1} z_{i-1} - U2_{i-2} z_{i-2}) / U0_i
  T z1 = T(0), z2 = T(0);      // z_{i-1}, z_{i-2}
  T U1p = T(0), U2p = T(0), U2pp = T(0);  // U1_{i-1}, U2_{i-1}, U2_{i-2}
  unsigned wcur = 0;
  for (int i = 0; i < n; ++i) {
    size_t o = idx<L>(i, j, n, batch);
    T U0, U1, U2 = T(0), m = T(0), r;
    if (i + 1 < n) {
      if ((i & 31) == 0) wcur = piv[(size_t)(i >> 5) * batch + j];
      const bool sw = (wcur >> (i & 31)) & 1u;
      size_t on = idx<L>(i + 1, j, n, batch);
      T an = ld_stream(a + on), bn = ld_stream(b + on), cn = (i + 2 < n) ? ld_stream(c + on) : T(0);
      const T p = sw ? an : u0;
      const T q = sw ? u0 : an;
      r = rcp(p);
      m = q * r;
      U0 = p;
      U1 = sw ? bn : u1;
      U2 = sw ? cn : T(0);
      const T nu0 = fma(-m, sw ? bn : u1, sw ? u1 : bn);
      const T nu1 = sw ? -m * cn : cn;
      u0 = nu0;
      u1 = nu1;
    } else {
      U0 = u0;
      U1 = T(0);
      r = rcp(U0);
    }
    (void)U0;
    T s = ld_stream(g + o);
    s = fma(-U1p, z1, s);
    s = fma(-U2pp, z2, s);
    T z = s * r;
    const size_t so = sidx<L>(i, j, n, batch);
    st_keep(wz + so, z);
    st_keep(wm + so, m);
    z2 = z1;
    z1 = z;
    U2pp = U2p;
    U2p = U2;
    U1p = U1;
  }
  // bottom-up
  T carry = z1;  // entry n-1, final unless step n-2 swaps
  T xi1 = ld_stream(x + idx<L>(n - 1, j, n, batch));  // x_{i+1}
  T xi2 = T(0);                                        // x_{i+2}
  for (int i = n - 2; i >= 0; --i) {
    size_t o = idx<L>(i, j, n, batch);
    if (((i & 31) == 31) || i == n - 2) wcur = piv[(size_t)(i >> 5) * batch + j];
    const bool sw = (wcur >> (i & 31)) & 1u;
    const size_t so = sidx<L>(i, j, n, batch);
    T zi = ld_keep(wz + so), mi = ld_keep(wm + so);
    T ni = fma(-mi, carry, zi);
    T lam1 = sw ? ni : carry;  // final lambda_{i+1}
    carry = sw ? carry : ni;
    T xi = ld_stream(x + o);
    size_t o1 = idx<L>(i + 1, j, n, batch);
    st_stream(gd + o1, lam1);
    st_stream(ga + o1, -lam1 * xi);
    st_stream(gb + o1, -lam1 * xi1);
    st_stream(gc + o1, (i + 2 < n) ? -lam1 * xi2 : T(0));
    xi2 = xi1;
    xi1 = xi;
  }
  // row 0
  st_stream(gd + o0, carry);
  st_stream(ga + o0, T(0));
  st_stream(gb + o0, -carry * xi1);
  st_stream(gc + o0, (n > 1) ? -carry * xi2 : T(0));
}

// ---------------------------------------------------------------------------
// Launchers.

static inline int seq_block(int batch) {
  // Few systems: one warp per block so the warps spread over all SMs.
  return batch <= 32 * 152 * 2 ? 32 : 128;
}

template <typename T, int L>
cudaError_t launch_thomas_seq_l(T* a, T* b, T* c, T* d, int n, int batch, cudaStream_t s) {
  int tpb = seq_block(batch);
  dim3 grid((batch + tpb - 1) / tpb);
  thomas_seq_kernel<T, L, 8><<<grid, tpb, 0, s>>>(a, b, c, d, n, batch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_thomas_seq(int layout, T* a, T* b, T* c, T* d, int n, int batch, cudaStream_t s) {
  switch (layout) {
    case CONTIG: return launch_thomas_seq_l<T, CONTIG>(a, b, c, d, n, batch, s);
    case PACKED: return launch_thomas_seq_l<T, PACKED>(a, b, c, d, n, batch, s);
    case INTERLEAVED: return launch_thomas_seq_l<T, INTERLEAVED>(a, b, c, d, n, batch, s);
  }
  return cudaErrorInvalidValue;
}

template <typename T, int L>
cudaError_t launch_gtsv_seq_l(const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv, int* info,
                              int n, int batch, cudaStream_t s, const int* mask = nullptr) {
  int tpb = seq_block(batch);
  dim3 grid((batch + tpb - 1) / tpb);
  gtsv_seq_kernel<T, L, 4><<<grid, tpb, 0, s>>>(a, b, c, d, w1, w2, piv, info, n, batch, mask);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gtsv_seq_masked(int layout, const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv,
                                   int* info, int n, int batch, const int* mask, cudaStream_t s) {
  if (layout == INTERLEAVED) return launch_gtsv_seq_l<T, INTERLEAVED>(a, b, c, d, w1, w2, piv, info, n, batch, s, mask);
  return launch_gtsv_seq_l<T, CONTIG>(a, b, c, d, w1, w2, piv, info, n, batch, s, mask);
}

template <typename T>
cudaError_t launch_gtsv_seq(int layout, const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv,
                            int* info, int n, int batch, cudaStream_t s) {
  switch (layout) {
    case CONTIG: return launch_gtsv_seq_l<T, CONTIG>(a, b, c, d, w1, w2, piv, info, n, batch, s);
    case PACKED: return launch_gtsv_seq_l<T, PACKED>(a, b, c, d, w1, w2, piv, info, n, batch, s);
    case INTERLEAVED: return launch_gtsv_seq_l<T, INTERLEAVED>(a, b, c, d, w1, w2, piv, info, n, batch, s);
  }
  return cudaErrorInvalidValue;
}

template <typename T, int L>
cudaError_t launch_gtsv_adjoint_l(const T* a, const T* b, const T* c, const T* x, const unsigned* piv, const T* g,
                                  T* ga, T* gb, T* gc, T* gd, T* wz, T* wm, int n, int batch, cudaStream_t s) {
  int tpb = seq_block(batch);
  dim3 grid((batch + tpb - 1) / tpb);
  gtsv_adjoint_seq_kernel<T, L><<<grid, tpb, 0, s>>>(a, b, c, x, piv, g, ga, gb, gc, gd, wz, wm, n, batch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gtsv_adjoint(int layout, const T* a, const T* b, const T* c, const T* x, const unsigned* piv,
                                const T* g, T* ga, T* gb, T* gc, T* gd, T* wz, T* wm, int n, int batch,
                                cudaStream_t s) {
  switch (layout) {
    case CONTIG: return launch_gtsv_adjoint_l<T, CONTIG>(a, b, c, x, piv, g, ga, gb, gc, gd, wz, wm, n, batch, s);
    case PACKED: return launch_gtsv_adjoint_l<T, PACKED>(a, b, c, x, piv, g, ga, gb, gc, gd, wz, wm, n, batch, s);
    case INTERLEAVED:
      return launch_gtsv_adjoint_l<T, INTERLEAVED>(a, b, c, x, piv, g, ga, gb, gc, gd, wz, wm, n, batch, s);
  }
  return cudaErrorInvalidValue;
}

#define INST(T)                                                                                                  \
  template cudaError_t launch_thomas_seq<T>(int, T*, T*, T*, T*, int, int, cudaStream_t);                        \
  template cudaError_t launch_gtsv_seq_masked<T>(int, const T*, const T*, const T*, T*, T*, T*, unsigned*, int*, \
                                                 int, int, const int*, cudaStream_t);                              \
  template cudaError_t launch_gtsv_seq<T>(int, const T*, const T*, const T*, T*, T*, T*, unsigned*, int*, int,   \
                                          int, cudaStream_t);                                                    \
  template cudaError_t launch_gtsv_adjoint<T>(int, const T*, const T*, const T*, const T*, const unsigned*,      \
                                              const T*, T*, T*, T*, T*, T*, T*, int, int, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tdg
