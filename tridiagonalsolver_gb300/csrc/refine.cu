// Kernels of the mixed-precision refined solve: FP64 inputs, FP32 pivoted
// solves, FP64 residuals.
//
//   narrow:   a, b, c, d (FP64) -> FP32 copies
//   residual: x_new = x_old + dx (FP64), r = d - A x_new (FP64) -> FP32
//   update:   x_out = x_old + dx
//
// On GB300 the FP64 pipe (and with it cvt.f32.f64 / cvt.f64.f32) runs at
// ~1/50 of the FP32 rate, so the conversions here use the integer pipe: an
// FP64 -> FP32 narrowing is the IEEE 754 round-to-nearest-even of the 52-bit
// significand to 23 bits done on the bit pattern, and FP32 -> FP64 widening
// is exact (re-biased exponent, significand shifted by 29).  Only zeros,
// infinities, NaNs and values outside the FP32 normal range take the
// hardware conversion.  The FP64 pipe then carries only the residual's three
// FMAs and the update's add per row.
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace tdg {

// The hardware conversions of the rare cases sit in functions of their own
// (inlined, they made the residual pass keep the FP64 pipe busier than its
// FMAs and adds account for: 159 -> 118 us per 8.4 M rows).
__device__ __noinline__ float narrow_rare(double v) { return __double2float_rn(v); }
__device__ __noinline__ double widen_rare(float f) { return (double)f; }

__device__ __forceinline__ float narrow_rn(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  const int e32 = e - 1023 + 127;
  if (e == 0) return __uint_as_float(sign);  // zero, or an FP64 subnormal (rounds to zero in FP32)
  if (e32 >= 1 && e32 <= 254) {
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 of the 52 significand bits
    const unsigned half = (lo >> 28) & 1u;                    // first dropped bit
    const unsigned rest = lo & 0x0fffffffu;                   // the other 28 dropped bits
    unsigned r = sign | ((unsigned)e32 << 23) | m;
    r += half & ((rest != 0u) | (m & 1u));  // ties to even; a carry rolls into the exponent (up to inf)
    return __uint_as_float(r);
  }
  return narrow_rare(v);  // inf, NaN, overflow, FP32 subnormal range
}

__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  if (e == 0u || e == 255u) return widen_rare(f);  // FP32 subnormal, inf, NaN
  const unsigned hi = (u & 0x80000000u) | ((e + 1023u - 127u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// a, b, c, d -> FP32, two elements per thread and array when the arrays are
// 16-byte aligned (checked on the host), else one.
template <bool VEC>
__global__ void __launch_bounds__(256) narrow4_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                      const double* __restrict__ c, const double* __restrict__ d,
                                                      float* __restrict__ a32, float* __restrict__ b32,
                                                      float* __restrict__ c32, float* __restrict__ d32,
                                                      size_t count) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (VEC) {
    const size_t pairs = count / 2;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < pairs; p += stride) {
      const double2 va = __ldg(reinterpret_cast<const double2*>(a) + p);
      const double2 vb = __ldg(reinterpret_cast<const double2*>(b) + p);
      const double2 vc = __ldg(reinterpret_cast<const double2*>(c) + p);
      const double2 vd = __ldg(reinterpret_cast<const double2*>(d) + p);
      reinterpret_cast<float2*>(a32)[p] = make_float2(narrow_rn(va.x), narrow_rn(va.y));
      reinterpret_cast<float2*>(b32)[p] = make_float2(narrow_rn(vb.x), narrow_rn(vb.y));
      reinterpret_cast<float2*>(c32)[p] = make_float2(narrow_rn(vc.x), narrow_rn(vc.y));
      reinterpret_cast<float2*>(d32)[p] = make_float2(narrow_rn(vd.x), narrow_rn(vd.y));
    }
    if ((count & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
      const size_t k = count - 1;
      a32[k] = narrow_rn(a[k]);
      b32[k] = narrow_rn(b[k]);
      c32[k] = narrow_rn(c[k]);
      d32[k] = narrow_rn(d[k]);
    }
  } else {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
      a32[k] = narrow_rn(a[k]);
      b32[k] = narrow_rn(b[k]);
      c32[k] = narrow_rn(c[k]);
      d32[k] = narrow_rn(d[k]);
    }
  }
}

// Row i of system j lives at j*n + i (CONTIG) or i*batch + j (INTERLEAVED);
// the neighbours of a row are one element (CONTIG) or one row of the batch
// (INTERLEAVED) away.  The grid walks (outer, inner) tiles: outer = system
// for CONTIG, row for INTERLEAVED; inner is the unit-stride index.  CONTIG:
// a warp holds 32 consecutive rows of one system and x_new of the rows
// beside a lane's comes by shuffles (lanes 0 and 31 form their outer
// neighbour), so each row's x_old + dx is formed once: 4 FP64 instructions
// per row.  INTERLEAVED forms the neighbours' x again (3 more).
template <int L>
__global__ void __launch_bounds__(256) residual_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                       const double* __restrict__ c, const double* __restrict__ d,
                                                       const double* __restrict__ xold, const float* __restrict__ dx,
                                                       double* __restrict__ xnew, float* __restrict__ r32, int n,
                                                       int batch) {
  const int inner_len = L == INTERLEAVED ? batch : n;
  const int outer_len = L == INTERLEAVED ? n : batch;
  const size_t nb = (size_t)(L == INTERLEAVED ? batch : 1);  // distance to the neighbouring row
  auto xat = [&](size_t q) { return (xold ? xold[q] : 0.0) + widen(dx[q]); };
  const int lane = threadIdx.x & 31;
  for (int o = blockIdx.y; o < outer_len; o += gridDim.y) {
    // (warp-uniform trip count: the shuffles need every lane)
    for (int t0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); t0 < inner_len; t0 += gridDim.x * blockDim.x) {
      const int t = t0 + lane;
      const bool in = t < inner_len;
      const size_t k = (size_t)o * inner_len + t;
      const int i = L == INTERLEAVED ? o : t;  // row index within the system
      const double xi = in ? xat(k) : 0.0;
      double xm, xp;
      if (L == INTERLEAVED) {
        xm = in && i > 0 ? xat(k - nb) : 0.0;
        xp = in && i < n - 1 ? xat(k + nb) : 0.0;
      } else {
        xm = __shfl_up_sync(0xffffffffu, xi, 1);
        xp = __shfl_down_sync(0xffffffffu, xi, 1);
        if (lane == 0 && in && i > 0) xm = xat(k - 1);
        if ((lane == 31 || t + 1 == inner_len) && in && i < n - 1) xp = xat(k + 1);
      }
      if (in) {
        double r = fma(-__ldg(b + k), xi, __ldg(d + k));
        if (i > 0) r = fma(-__ldg(a + k), xm, r);
        if (i < n - 1) r = fma(-__ldg(c + k), xp, r);
        xnew[k] = xi;
        r32[k] = narrow_rn(r);
      }
    }
  }
}

// CONTIG with n a multiple of 4 and 16-byte aligned arrays: a warp holds
// 128 consecutive rows of one system, lane l rows 4l .. 4l+3 (16-byte
// loads), so the rows' x_old + dx are formed once by full-warp instructions
// and only the two rows beyond the warp's tile are formed again by one lane.
__global__ void __launch_bounds__(256) residual4_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                        const double* __restrict__ c, const double* __restrict__ d,
                                                        const double* __restrict__ xold, const float* __restrict__ dx,
                                                        double* __restrict__ xnew, float* __restrict__ r32, int n,
                                                        int batch) {
  const int lane = threadIdx.x & 31;
  auto xat = [&](size_t q) { return (xold ? xold[q] : 0.0) + widen(dx[q]); };
  for (int o = blockIdx.y; o < batch; o += gridDim.y) {
    for (int t0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) * 4; t0 < n; t0 += gridDim.x * blockDim.x * 4) {
      const int i0 = t0 + 4 * lane;  // (warp-uniform trip count: the shuffles need every lane)
      const bool in = i0 < n;       // (n % 4 == 0: a lane's four rows are all in or all out)
      const size_t k = (size_t)o * n + i0;
      double x[4] = {0.0, 0.0, 0.0, 0.0};
      if (in) {
        const float4 v = *reinterpret_cast<const float4*>(dx + k);
        const float dv[4] = {v.x, v.y, v.z, v.w};
        double xo[4] = {0.0, 0.0, 0.0, 0.0};
        if (xold) {
          const double2 p0 = *reinterpret_cast<const double2*>(xold + k);
          const double2 p1 = *reinterpret_cast<const double2*>(xold + k + 2);
          xo[0] = p0.x; xo[1] = p0.y; xo[2] = p1.x; xo[3] = p1.y;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = xo[u] + widen(dv[u]);
      }
      double xm = __shfl_up_sync(0xffffffffu, x[3], 1);
      double xp = __shfl_down_sync(0xffffffffu, x[0], 1);
      if (lane == 0 && in && i0 > 0) xm = xat(k - 1);
      if (lane == 31 && in && i0 + 4 < n) xp = xat(k + 4);
      if (in) {
        const double2 a0 = __ldg(reinterpret_cast<const double2*>(a + k)), a1 = __ldg(reinterpret_cast<const double2*>(a + k + 2));
        const double2 b0 = __ldg(reinterpret_cast<const double2*>(b + k)), b1 = __ldg(reinterpret_cast<const double2*>(b + k + 2));
        const double2 c0 = __ldg(reinterpret_cast<const double2*>(c + k)), c1 = __ldg(reinterpret_cast<const double2*>(c + k + 2));
        const double2 d0 = __ldg(reinterpret_cast<const double2*>(d + k)), d1 = __ldg(reinterpret_cast<const double2*>(d + k + 2));
        const double av[4] = {a0.x, a0.y, a1.x, a1.y}, bv[4] = {b0.x, b0.y, b1.x, b1.y};
        const double cv[4] = {c0.x, c0.y, c1.x, c1.y}, dvv[4] = {d0.x, d0.y, d1.x, d1.y};
        float rr[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u;
          const double left = u > 0 ? x[u - 1] : xm, right = u < 3 ? x[u + 1] : xp;
          double r = fma(-bv[u], x[u], dvv[u]);
          if (i > 0) r = fma(-av[u], left, r);
          if (i < n - 1) r = fma(-cv[u], right, r);
          rr[u] = narrow_rn(r);
        }
        *reinterpret_cast<double2*>(xnew + k) = make_double2(x[0], x[1]);
        *reinterpret_cast<double2*>(xnew + k + 2) = make_double2(x[2], x[3]);
        *reinterpret_cast<float4*>(r32 + k) = make_float4(rr[0], rr[1], rr[2], rr[3]);
      }
    }
  }
}

__global__ void __launch_bounds__(256) update_kernel(const double* __restrict__ xold, const float* __restrict__ dx,
                                                     double* xout, size_t count) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride)
    xout[k] = (xold ? xold[k] : 0.0) + widen(dx[k]);
}

static int grid_for(size_t work, int threads) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (work + threads - 1) / threads;
  const size_t cap = (size_t)sms * 8;
  return (int)(want < cap ? (want ? want : 1) : cap);
}

cudaError_t launch_narrow4(const double* a, const double* b, const double* c, const double* d, float* a32,
                           float* b32, float* c32, float* d32, size_t count, cudaStream_t s) {
  const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                     reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(d) |
                     reinterpret_cast<uintptr_t>(a32) | reinterpret_cast<uintptr_t>(b32) |
                     reinterpret_cast<uintptr_t>(c32) | reinterpret_cast<uintptr_t>(d32)) &
                    15u) == 0;
  if (vec)
    narrow4_kernel<true><<<grid_for(count / 2, 256), 256, 0, s>>>(a, b, c, d, a32, b32, c32, d32, count);
  else
    narrow4_kernel<false><<<grid_for(count, 256), 256, 0, s>>>(a, b, c, d, a32, b32, c32, d32, count);
  return cudaGetLastError();
}

cudaError_t launch_residual(int layout, const double* a, const double* b, const double* c, const double* d,
                            const double* xold, const float* dx, double* xnew, float* r32, int n, int batch,
                            cudaStream_t s) {
  const int inner = layout == INTERLEAVED ? batch : n;
  const int outer = layout == INTERLEAVED ? n : batch;
  const int threads = 256;
  const int gx = (inner + threads - 1) / threads;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int gy_cap = (sms * 8 + gx - 1) / gx;
  const int gy = outer < gy_cap ? outer : (gy_cap < 65535 ? gy_cap : 65535);
  dim3 grid(gx, gy > 0 ? gy : 1);
  const bool vec4 = layout == CONTIG && n % 4 == 0 &&
                    ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c) |
                      reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(xold) |
                      reinterpret_cast<uintptr_t>(dx) | reinterpret_cast<uintptr_t>(xnew) |
                      reinterpret_cast<uintptr_t>(r32)) & 15u) == 0;
  if (vec4) {
    const int gx4 = (n / 4 + threads - 1) / threads;
    const int gy4_cap = (sms * 8 + gx4 - 1) / gx4;
    const int gy4 = outer < gy4_cap ? outer : (gy4_cap < 65535 ? gy4_cap : 65535);
    residual4_kernel<<<dim3(gx4, gy4 > 0 ? gy4 : 1), threads, 0, s>>>(a, b, c, d, xold, dx, xnew, r32, n, batch);
  } else if (layout == INTERLEAVED) {
    residual_kernel<INTERLEAVED><<<grid, threads, 0, s>>>(a, b, c, d, xold, dx, xnew, r32, n, batch);
  } else {
    residual_kernel<CONTIG><<<grid, threads, 0, s>>>(a, b, c, d, xold, dx, xnew, r32, n, batch);
  }
  return cudaGetLastError();
}

cudaError_t launch_update(const double* xold, const float* dx, double* xout, size_t count, cudaStream_t s) {
  update_kernel<<<grid_for(count, 256), 256, 0, s>>>(xold, dx, xout, count);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Ragged batches: one warp per RAGGED_ROW_CHUNK rows of the packed arrays,
// whatever systems they belong to (a warp per system would leave the longest
// systems' warps running long after the rest), 32 rows per step, lane l on
// row r0 + l.  The system boundaries inside a step come from the offsets
// themselves: lane l reads offsets[s + 1 + l] (s = the system holding r0)
// and a reduction over the warp gives the masks of the step's first and
// last rows, so a_0, c_{n-1} (TRANS: c_{-1}, a_n) of a system are never
// read.  x of the neighbouring rows travels by shuffles (lane 0 takes the
// previous step's lane 31, lane 31 loads row r0 + 32).  TRANS: the
// coefficients of A^T (sub-diagonal c_{i-1}, super-diagonal a_{i+1}).

// Masks of the first / last rows of their systems among rows [r0, r0 + 32)
// (bit l: row r0 + l), s the system holding r0; s moves on to the system
// holding r0 + 32.  Sizes are >= 1, so the boundaries increase strictly and
// at most 32 of them lie in (r0, r0 + 32].
__device__ __forceinline__ void ragged_step_masks(const RaggedRows& rr, long long r0, int& s, unsigned& first,
                                                  unsigned& last) {
  const int lane = threadIdx.x & 31;
  const int q = s + 1 + lane;
  const long long v = q <= rr.batch ? __ldg(rr.offsets + q) : 0x7fffffffffffffffll;
  const bool f_in = v < r0 + 32, l_in = v <= r0 + 32;  // (v > r0: s holds r0)
  const unsigned f = __reduce_or_sync(0xffffffffu, f_in ? 1u << (int)(v - r0) : 0u);
  last = __reduce_or_sync(0xffffffffu, l_in ? 1u << (int)(v - 1 - r0) : 0u);
  first = f | (__ldg(rr.offsets + s) == r0 ? 1u : 0u);
  s += __popc(__ballot_sync(0xffffffffu, l_in));
}

// The warp's chunk: rows [*begin, *end), its first system in *s; false for a
// warp past the last row.
__device__ __forceinline__ bool ragged_chunk(const RaggedRows& rr, long long* begin, long long* end, int* s) {
  const long long k = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  *begin = k * RAGGED_ROW_CHUNK;
  if (*begin >= rr.rows) return false;
  *end = min(rr.rows, *begin + RAGGED_ROW_CHUNK);
  *s = __ldg(rr.chunk_sys + k);
  return true;
}

// a, b, c, rhs -> FP32 copies of A (TRANS: of A^T) and of the right-hand side
template <bool TRANS>
__global__ void __launch_bounds__(256) ragged_narrow_kernel(const double* __restrict__ a,
                                                            const double* __restrict__ b,
                                                            const double* __restrict__ c,
                                                            const double* __restrict__ rhs, float* __restrict__ a32,
                                                            float* __restrict__ b32, float* __restrict__ c32,
                                                            float* __restrict__ r32, const RaggedRows rr) {
  long long begin, end;
  int s;
  if (!ragged_chunk(rr, &begin, &end, &s)) return;
  const int lane = threadIdx.x & 31;
  for (long long r0 = begin; r0 < end; r0 += 32) {
    unsigned fm, lm;
    ragged_step_masks(rr, r0, s, fm, lm);
    const long long r = r0 + lane;
    if (r < end) {
      const bool first = (fm >> lane) & 1u, last = (lm >> lane) & 1u;
      const double lo = first ? 0.0 : (TRANS ? __ldg(c + r - 1) : __ldg(a + r));
      const double up = last ? 0.0 : (TRANS ? __ldg(a + r + 1) : __ldg(c + r));
      a32[r] = narrow_rn(lo);
      b32[r] = narrow_rn(__ldg(b + r));
      c32[r] = narrow_rn(up);
      r32[r] = narrow_rn(__ldg(rhs + r));
    }
  }
}

// x_new = x_old + dx (x_old may be NULL: zero), r = rhs - A x_new (FP64,
// stored as FP32); TRANS: r = rhs - A^T x_new.
template <bool TRANS>
__global__ void __launch_bounds__(256) ragged_residual_kernel(
    const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
    const double* __restrict__ rhs, const double* __restrict__ xold, const float* __restrict__ dx,
    double* __restrict__ xnew, float* __restrict__ r32, const RaggedRows rr) {
  long long begin, end;
  int s;
  if (!ragged_chunk(rr, &begin, &end, &s)) return;
  const int lane = threadIdx.x & 31;
  auto xat = [&](long long k) { return xold ? __ldg(xold + k) + widen(__ldg(dx + k)) : widen(__ldg(dx + k)); };
  // x of the row before the chunk (read only where that row is in the same system)
  double xlast = begin > 0 && __ldg(rr.offsets + s) < begin ? xat(begin - 1) : 0.0;
  for (long long r0 = begin; r0 < end; r0 += 32) {
    unsigned fm, lm;
    ragged_step_masks(rr, r0, s, fm, lm);
    const long long r = r0 + lane;
    const bool in = r < end, first = (fm >> lane) & 1u, last = (lm >> lane) & 1u;
    const double xi = in ? xat(r) : 0.0;
    double xm = __shfl_up_sync(0xffffffffu, xi, 1);
    if (lane == 0) xm = xlast;
    double xp = __shfl_down_sync(0xffffffffu, xi, 1);
    if (lane == 31 && in && !last) xp = xat(r + 1);
    if (in) {
      const double lo = first ? 0.0 : (TRANS ? __ldg(c + r - 1) : __ldg(a + r));
      const double up = last ? 0.0 : (TRANS ? __ldg(a + r + 1) : __ldg(c + r));
      double res = fma(-__ldg(b + r), xi, __ldg(rhs + r));
      res = fma(-lo, xm, res);
      res = fma(-up, xp, res);
      xnew[r] = xi;
      r32[r] = narrow_rn(res);
    }
    xlast = __shfl_sync(0xffffffffu, xi, 31);
  }
}

// Gradients of the adjoint from lambda and the forward solution x:
// ga_i = -lambda_i x_{i-1} (0 at a system's first row), gb_i = -lambda_i
// x_i, gc_i = -lambda_i x_{i+1} (0 at its last row).
__global__ void __launch_bounds__(256) ragged_gradient_kernel(const double* __restrict__ lam,
                                                              const double* __restrict__ x, double* __restrict__ ga,
                                                              double* __restrict__ gb, double* __restrict__ gc,
                                                              const RaggedRows rr) {
  long long begin, end;
  int s;
  if (!ragged_chunk(rr, &begin, &end, &s)) return;
  const int lane = threadIdx.x & 31;
  double xlast = begin > 0 && __ldg(rr.offsets + s) < begin ? __ldg(x + begin - 1) : 0.0;
  for (long long r0 = begin; r0 < end; r0 += 32) {
    unsigned fm, lm;
    ragged_step_masks(rr, r0, s, fm, lm);
    const long long r = r0 + lane;
    const bool in = r < end, first = (fm >> lane) & 1u, last = (lm >> lane) & 1u;
    const double xi = in ? __ldg(x + r) : 0.0;
    double xm = __shfl_up_sync(0xffffffffu, xi, 1);
    if (lane == 0) xm = xlast;
    double xp = __shfl_down_sync(0xffffffffu, xi, 1);
    if (lane == 31 && in && !last) xp = __ldg(x + r + 1);
    if (in) {
      const double l = -__ldg(lam + r);
      ga[r] = first ? 0.0 : l * xm;
      gb[r] = l * xi;
      gc[r] = last ? 0.0 : l * xp;
    }
    xlast = __shfl_sync(0xffffffffu, xi, 31);
  }
}

// The refinement steps restricted to the systems solved with pivoting
// (kinds[s] == 0; every system when kinds is NULL), on x in place.
//
// ragged_sel: the system of row r0 + lane is s0 (the one holding r0) plus
// the system starts in (r0, r0 + lane]; a warp whose chunk lies inside one
// unselected system returns at once.
__device__ __forceinline__ bool ragged_sel_skip(const RaggedRows& rr, const unsigned char* kinds, int s,
                                                long long end) {
  return kinds && __ldg(kinds + s) != 0 && __ldg(rr.offsets + s + 1) >= end;
}
__device__ __forceinline__ int ragged_lane_sys(int s0, unsigned first) {
  const int lane = threadIdx.x & 31;
  const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
  return s0 + __popc(first & upto & ~1u);
}

// r = rhs - A x (TRANS: A^T) as FP32, on the rows of the selected systems.
// A step with no selected row is skipped: the x of its last row is then
// needed by no later row (a selected row that is not its system's first has
// its predecessor in the same, selected system).
template <bool TRANS>
__global__ void __launch_bounds__(256) ragged_residual_sel_kernel(
    const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
    const double* __restrict__ rhs, const double* __restrict__ x, float* __restrict__ r32,
    const unsigned char* __restrict__ kinds, const RaggedRows rr) {
  long long begin, end;
  int s;
  if (!ragged_chunk(rr, &begin, &end, &s)) return;
  if (ragged_sel_skip(rr, kinds, s, end)) return;
  const int lane = threadIdx.x & 31;
  double xlast = begin > 0 && __ldg(rr.offsets + s) < begin ? __ldg(x + begin - 1) : 0.0;
  for (long long r0 = begin; r0 < end; r0 += 32) {
    const int s0 = s;
    unsigned fm, lm;
    ragged_step_masks(rr, r0, s, fm, lm);
    const long long r = r0 + lane;
    const bool in = r < end, first = (fm >> lane) & 1u, last = (lm >> lane) & 1u;
    const bool sel = in && (!kinds || __ldg(kinds + ragged_lane_sys(s0, fm)) == 0);
    if (!__any_sync(0xffffffffu, sel)) continue;
    const double xi = in ? __ldg(x + r) : 0.0;
    double xm = __shfl_up_sync(0xffffffffu, xi, 1);
    if (lane == 0) xm = xlast;
    double xp = __shfl_down_sync(0xffffffffu, xi, 1);
    if (lane == 31 && in && !last) xp = __ldg(x + r + 1);
    if (sel) {
      const double lo = first ? 0.0 : (TRANS ? __ldg(c + r - 1) : __ldg(a + r));
      const double up = last ? 0.0 : (TRANS ? __ldg(a + r + 1) : __ldg(c + r));
      double res = fma(-__ldg(b + r), xi, __ldg(rhs + r));
      res = fma(-lo, xm, res);
      res = fma(-up, xp, res);
      r32[r] = narrow_rn(res);
    }
    xlast = __shfl_sync(0xffffffffu, xi, 31);
  }
}

// x += dx on the rows of the selected systems
__global__ void __launch_bounds__(256) ragged_update_sel_kernel(double* __restrict__ x, const float* __restrict__ dx,
                                                                const unsigned char* __restrict__ kinds,
                                                                const RaggedRows rr) {
  long long begin, end;
  int s;
  if (!ragged_chunk(rr, &begin, &end, &s)) return;
  if (ragged_sel_skip(rr, kinds, s, end)) return;
  const int lane = threadIdx.x & 31;
  for (long long r0 = begin; r0 < end; r0 += 32) {
    const int s0 = s;
    unsigned fm, lm;
    ragged_step_masks(rr, r0, s, fm, lm);
    const long long r = r0 + lane;
    if (r < end && (!kinds || __ldg(kinds + ragged_lane_sys(s0, fm)) == 0)) x[r] += widen(__ldg(dx + r));
  }
}

static int ragged_grid(const RaggedRows& rr) {
  const long long chunks = (rr.rows + RAGGED_ROW_CHUNK - 1) / RAGGED_ROW_CHUNK;
  return (int)((chunks + 7) / 8);  // eight warps (chunks) per 256-thread block
}

cudaError_t launch_ragged_narrow(bool trans, const double* a, const double* b, const double* c, const double* rhs,
                                 float* a32, float* b32, float* c32, float* r32, const RaggedRows& rr,
                                 cudaStream_t s) {
  if (rr.rows <= 0) return cudaSuccess;
  if (trans)
    ragged_narrow_kernel<true><<<ragged_grid(rr), 256, 0, s>>>(a, b, c, rhs, a32, b32, c32, r32, rr);
  else
    ragged_narrow_kernel<false><<<ragged_grid(rr), 256, 0, s>>>(a, b, c, rhs, a32, b32, c32, r32, rr);
  return cudaGetLastError();
}

cudaError_t launch_ragged_residual(bool trans, const double* a, const double* b, const double* c, const double* rhs,
                                   const double* xold, const float* dx, double* xnew, float* r32,
                                   const RaggedRows& rr, cudaStream_t s) {
  if (rr.rows <= 0) return cudaSuccess;
  if (trans)
    ragged_residual_kernel<true><<<ragged_grid(rr), 256, 0, s>>>(a, b, c, rhs, xold, dx, xnew, r32, rr);
  else
    ragged_residual_kernel<false><<<ragged_grid(rr), 256, 0, s>>>(a, b, c, rhs, xold, dx, xnew, r32, rr);
  return cudaGetLastError();
}

cudaError_t launch_ragged_residual_sel(bool trans, const double* a, const double* b, const double* c,
                                       const double* rhs, const double* x, float* r32, const unsigned char* kinds,
                                       const RaggedRows& rr, cudaStream_t s) {
  if (rr.rows <= 0) return cudaSuccess;
  if (trans)
    ragged_residual_sel_kernel<true><<<ragged_grid(rr), 256, 0, s>>>(a, b, c, rhs, x, r32, kinds, rr);
  else
    ragged_residual_sel_kernel<false><<<ragged_grid(rr), 256, 0, s>>>(a, b, c, rhs, x, r32, kinds, rr);
  return cudaGetLastError();
}

cudaError_t launch_ragged_update_sel(double* x, const float* dx, const unsigned char* kinds, const RaggedRows& rr,
                                     cudaStream_t s) {
  if (rr.rows <= 0) return cudaSuccess;
  ragged_update_sel_kernel<<<ragged_grid(rr), 256, 0, s>>>(x, dx, kinds, rr);
  return cudaGetLastError();
}

cudaError_t launch_ragged_gradient(const double* lam, const double* x, double* ga, double* gb, double* gc,
                                   const RaggedRows& rr, cudaStream_t s) {
  if (rr.rows <= 0) return cudaSuccess;
  ragged_gradient_kernel<<<ragged_grid(rr), 256, 0, s>>>(lam, x, ga, gb, gc, rr);
  return cudaGetLastError();
}

// Conversion check used by the tests: out[k] = narrow_rn(in[k]) and
// back[k] = widen(out[k]).
__global__ void convert_probe_kernel(const double* in, float* out, double* back, size_t count) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x) {
    const float f = narrow_rn(in[k]);
    out[k] = f;
    back[k] = widen(f);
  }
}

cudaError_t launch_convert_probe(const double* in, float* out, double* back, size_t count, cudaStream_t s) {
  convert_probe_kernel<<<grid_for(count, 256), 256, 0, s>>>(in, out, back, count);
  return cudaGetLastError();
}

}  // namespace tdg
