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
  return __double2float_rn(v);  // inf, NaN, overflow, FP32 subnormal range
}

__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  if (e == 0u || e == 255u) return (double)f;  // FP32 subnormal, inf, NaN
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
// for CONTIG, row for INTERLEAVED; inner is the unit-stride index.
template <int L>
__global__ void __launch_bounds__(256) residual_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                       const double* __restrict__ c, const double* __restrict__ d,
                                                       const double* __restrict__ xold, const float* __restrict__ dx,
                                                       double* __restrict__ xnew, float* __restrict__ r32, int n,
                                                       int batch) {
  const int inner_len = L == INTERLEAVED ? batch : n;
  const int outer_len = L == INTERLEAVED ? n : batch;
  const size_t nb = (size_t)(L == INTERLEAVED ? batch : 1);  // distance to the neighbouring row
  for (int o = blockIdx.y; o < outer_len; o += gridDim.y) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < inner_len; t += gridDim.x * blockDim.x) {
      const size_t k = (size_t)o * inner_len + t;
      const int i = L == INTERLEAVED ? o : t;  // row index within the system
      auto xat = [&](size_t q) { return (xold ? xold[q] : 0.0) + widen(dx[q]); };
      const double xi = xat(k);
      double r = fma(-__ldg(b + k), xi, __ldg(d + k));
      if (i > 0) r = fma(-__ldg(a + k), xat(k - nb), r);
      if (i < n - 1) r = fma(-__ldg(c + k), xat(k + nb), r);
      xnew[k] = xi;
      r32[k] = narrow_rn(r);
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
  if (layout == INTERLEAVED)
    residual_kernel<INTERLEAVED><<<grid, threads, 0, s>>>(a, b, c, d, xold, dx, xnew, r32, n, batch);
  else
    residual_kernel<CONTIG><<<grid, threads, 0, s>>>(a, b, c, d, xold, dx, xnew, r32, n, batch);
  return cudaGetLastError();
}

cudaError_t launch_update(const double* xold, const float* dx, double* xout, size_t count, cudaStream_t s) {
  update_kernel<<<grid_for(count, 256), 256, 0, s>>>(xold, dx, xout, count);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Ragged batches (system s = rows [offsets[s], offsets[s+1])): one warp per
// system, grid-stride over the systems, lane l holding row i0 + l; the
// neighbouring rows' values travel by shuffles (the row before a 32-row
// step by the previous step's lane 31, the row after it by one more load),
// so every row's x is formed once.  a_0 and c_{n-1} of a system are not
// read.  TRANS: the coefficients of A^T (sub-diagonal c_{i-1},
// super-diagonal a_{i+1}).

__device__ __forceinline__ int ragged_warps() { return (int)(gridDim.x * blockDim.x / 32); }

// a, b, c, rhs -> FP32 copies of A (TRANS: of A^T) and of the right-hand side
template <bool TRANS>
__global__ void __launch_bounds__(256) ragged_narrow_kernel(const double* __restrict__ a,
                                                            const double* __restrict__ b,
                                                            const double* __restrict__ c,
                                                            const double* __restrict__ rhs, float* a32, float* b32,
                                                            float* c32, float* r32, const long long* offsets,
                                                            int batch) {
  const int lane = threadIdx.x & 31;
  for (int s = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32); s < batch; s += ragged_warps()) {
    const long long base = offsets[s], n = offsets[s + 1] - base;
    for (long long i = lane; i < n; i += 32) {
      const long long k = base + i;
      const double lo = i > 0 ? (TRANS ? __ldg(c + k - 1) : __ldg(a + k)) : 0.0;
      const double up = i < n - 1 ? (TRANS ? __ldg(a + k + 1) : __ldg(c + k)) : 0.0;
      a32[k] = narrow_rn(lo);
      b32[k] = narrow_rn(__ldg(b + k));
      c32[k] = narrow_rn(up);
      r32[k] = narrow_rn(__ldg(rhs + k));
    }
  }
}

// x_new = x_old + dx (x_old may be NULL: zero), r = rhs - A x_new (FP64,
// stored as FP32); TRANS: r = rhs - A^T x_new.
template <bool TRANS>
__global__ void __launch_bounds__(256) ragged_residual_kernel(
    const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
    const double* __restrict__ rhs, const double* __restrict__ xold, const float* __restrict__ dx,
    double* __restrict__ xnew, float* __restrict__ r32, const long long* __restrict__ offsets, int batch) {
  const int lane = threadIdx.x & 31;
  auto xat = [&](long long k) { return xold ? __ldg(xold + k) + widen(__ldg(dx + k)) : widen(__ldg(dx + k)); };
  for (int s = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32); s < batch; s += ragged_warps()) {
    const long long base = offsets[s], n = offsets[s + 1] - base;
    double xlast = 0.0;  // x of the row before this step
    for (long long i0 = 0; i0 < n; i0 += 32) {
      const long long i = i0 + lane, k = base + i;
      const bool in = i < n;
      const double xi = in ? xat(k) : 0.0;
      double xm = __shfl_up_sync(0xffffffffu, xi, 1);
      if (lane == 0) xm = xlast;
      double xp = __shfl_down_sync(0xffffffffu, xi, 1);
      if (lane == 31 && i + 1 < n) xp = xat(k + 1);
      if (in) {
        const double lo = i > 0 ? (TRANS ? __ldg(c + k - 1) : __ldg(a + k)) : 0.0;
        const double up = i < n - 1 ? (TRANS ? __ldg(a + k + 1) : __ldg(c + k)) : 0.0;
        double r = fma(-__ldg(b + k), xi, __ldg(rhs + k));
        r = fma(-lo, xm, r);
        r = fma(-up, xp, r);
        xnew[k] = xi;
        r32[k] = narrow_rn(r);
      }
      xlast = __shfl_sync(0xffffffffu, xi, 31);
    }
  }
}

// Gradients of the adjoint from lambda and the forward solution x:
// ga_i = -lambda_i x_{i-1} (0 at a system's first row), gb_i = -lambda_i
// x_i, gc_i = -lambda_i x_{i+1} (0 at its last row).
__global__ void __launch_bounds__(256) ragged_gradient_kernel(const double* __restrict__ lam,
                                                              const double* __restrict__ x, double* ga, double* gb,
                                                              double* gc, const long long* __restrict__ offsets,
                                                              int batch) {
  const int lane = threadIdx.x & 31;
  for (int s = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32); s < batch; s += ragged_warps()) {
    const long long base = offsets[s], n = offsets[s + 1] - base;
    double xlast = 0.0;
    for (long long i0 = 0; i0 < n; i0 += 32) {
      const long long i = i0 + lane, k = base + i;
      const bool in = i < n;
      const double xi = in ? __ldg(x + k) : 0.0;
      double xm = __shfl_up_sync(0xffffffffu, xi, 1);
      if (lane == 0) xm = xlast;
      double xp = __shfl_down_sync(0xffffffffu, xi, 1);
      if (lane == 31 && i + 1 < n) xp = __ldg(x + k + 1);
      if (in) {
        const double l = -__ldg(lam + k);
        ga[k] = i > 0 ? l * xm : 0.0;
        gb[k] = l * xi;
        gc[k] = i < n - 1 ? l * xp : 0.0;
      }
      xlast = __shfl_sync(0xffffffffu, xi, 31);
    }
  }
}

static int ragged_grid(int batch) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int want = (batch + 7) / 8;  // eight warps per 256-thread block
  return want < sms * 8 ? (want > 0 ? want : 1) : sms * 8;
}

cudaError_t launch_ragged_narrow(bool trans, const double* a, const double* b, const double* c, const double* rhs,
                                 float* a32, float* b32, float* c32, float* r32, const long long* offsets, int batch,
                                 cudaStream_t s) {
  if (trans)
    ragged_narrow_kernel<true><<<ragged_grid(batch), 256, 0, s>>>(a, b, c, rhs, a32, b32, c32, r32, offsets, batch);
  else
    ragged_narrow_kernel<false><<<ragged_grid(batch), 256, 0, s>>>(a, b, c, rhs, a32, b32, c32, r32, offsets, batch);
  return cudaGetLastError();
}

cudaError_t launch_ragged_residual(bool trans, const double* a, const double* b, const double* c, const double* rhs,
                                   const double* xold, const float* dx, double* xnew, float* r32,
                                   const long long* offsets, int batch, cudaStream_t s) {
  if (trans)
    ragged_residual_kernel<true><<<ragged_grid(batch), 256, 0, s>>>(a, b, c, rhs, xold, dx, xnew, r32, offsets, batch);
  else
    ragged_residual_kernel<false><<<ragged_grid(batch), 256, 0, s>>>(a, b, c, rhs, xold, dx, xnew, r32, offsets,
                                                                     batch);
  return cudaGetLastError();
}

cudaError_t launch_ragged_gradient(const double* lam, const double* x, double* ga, double* gb, double* gc,
                                   const long long* offsets, int batch, cudaStream_t s) {
  ragged_gradient_kernel<<<ragged_grid(batch), 256, 0, s>>>(lam, x, ga, gb, gc, offsets, batch);
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
