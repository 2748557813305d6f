// Shared device helpers for the batched tridiagonal kernels (sm_103a).
//
// Conventions used by every kernel in this directory:
//   * a system is   a_i x_{i-1} + b_i x_i + c_i x_{i+1} = d_i,  i = 0..n-1;
//     a_0 and c_{n-1} are never read (treated as 0).
//   * layouts (the reference's numbering, Tridiagonal_CUDA/helpers.h:17,
//     plus one new):
//       CONTIG      (0)  a[j*n + i]           system-major, the reference's layout 0
//       PACKED      (1)  base[j*4n + k*n + i] with k = 0..3 for a,b,c,d
//                        (BPLG layout, Tridiagonal_CUDA/utils.cu:255-260)
//       INTERLEAVED (2)  a[i*batch + j]       batch-fastest, coalesced for a
//                        thread-per-system sweep
//   * FP64 arithmetic on GB300 runs at ~1/50 of the FP32 rate, while the
//     MUFU reciprocal approximation and integer ops run at full rate.  The
//     FP64 paths therefore take reciprocals from rcp.approx.ftz.f64 refined
//     by one third-order Newton step (3 FP64 FMAs) and compare magnitudes on
//     the integer bit patterns.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tdg {

enum Layout : int { CONTIG = 0, PACKED = 1, INTERLEAVED = 2 };

// Element offset of row i of system j for array k (0..3 = a,b,c,d) relative
// to that array's base pointer.  For PACKED all four arrays share one base
// pointer (the caller passes the same pointer four times, offset by k*n).
template <int L>
__host__ __device__ __forceinline__ size_t idx(int i, int j, int n, int batch) {
  if (L == INTERLEAVED) return (size_t)i * (size_t)batch + (size_t)j;
  if (L == PACKED) return (size_t)j * 4u * (size_t)n + (size_t)i;
  return (size_t)j * (size_t)n + (size_t)i;
}

// Element offset of row i of system j in a kernel's own scratch array of
// n * batch elements: batch-fastest for interleaved inputs (so the scratch
// accesses coalesce like the inputs'), system-major otherwise.  Never the
// packed stride: packed systems are 4n elements apart, which would run past
// an n * batch array.
template <int L>
__host__ __device__ __forceinline__ size_t sidx(int i, int j, int n, int batch) {
  return L == INTERLEAVED ? idx<INTERLEAVED>(i, j, n, batch) : idx<CONTIG>(i, j, n, batch);
}

// ---------------------------------------------------------------------------
// Reciprocals.

// 1/x in FP64: MUFU seed (rcp.approx.ftz.f64), then one third-order
// Newton-Raphson step r <- r (1 + e + e^2) with e = 1 - x r, which cubes the
// seed's relative error (the classical iterative reciprocal refinement, e.g.
// Markstein, "IA-64 and Elementary Functions", 2000).  x = 0 gives NaN/Inf.
__device__ __forceinline__ double rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  e = fma(e, e, e);
  return fma(r, e, r);
}

// 1/x in FP32: the MUFU approximation (at most 1 ulp from the rounded
// reciprocal), the same class of division the reference's GPU kernels use
// by default (div.approx.ftz.f32, Tridiagonal_CUDA/intrin.h:56-61).
__device__ __forceinline__ float rcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// v when k, else +0, as a select the compiler cannot see through: an FMA
// whose operand is a selected constant zero may otherwise be split into the
// two cases (a separate multiply or add on the FP64 pipe for the zero one).
__device__ __forceinline__ double keep_if(bool k, double v) {
  double r;
  asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\tselp.f64 %0, %1, 0d0000000000000000, p;\n\t}"
      : "=d"(r)
      : "d"(v), "r"((unsigned)k));
  return r;
}
__device__ __forceinline__ float keep_if(bool k, float v) {
  float r;
  asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\tselp.f32 %0, %1, 0f00000000, p;\n\t}"
      : "=f"(r)
      : "f"(v), "r"((unsigned)k));
  return r;
}

// The IEEE bit pattern of x through a move the compiler cannot see through,
// so that tests written on it stay integer instructions: a test it
// recognises (== 0 after dropping the sign, exponent all ones) may otherwise
// be turned back into a floating-point compare, which for FP64 takes a slot
// of the FP64 pipe.
__device__ __forceinline__ unsigned long long bits_of(double x) {
  unsigned long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ unsigned bits_of(float x) {
  unsigned r;
  asm("mov.b32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// |x| >= |y| on the IEEE bit patterns (integer pipe; NaN compares as large).
__device__ __forceinline__ bool abs_ge(double x, double y) {
  return (bits_of(x) & 0x7fffffffffffffffull) >= (bits_of(y) & 0x7fffffffffffffffull);
}
__device__ __forceinline__ bool abs_ge(float x, float y) {
  return (bits_of(x) & 0x7fffffffu) >= (bits_of(y) & 0x7fffffffu);
}

__device__ __forceinline__ bool is_zero(double x) { return (bits_of(x) << 1) == 0ull; }
__device__ __forceinline__ bool is_zero(float x) { return (bits_of(x) << 1) == 0u; }

// FP32 bounds of |x| formed on the integer pipe: mag_below(x) <= |x| <=
// mag_above(x) (FP64: the mantissa truncated to 23 bits, and the next float
// up; exponents beyond the FP32 range clamp to 0 / FLT_MIN / FLT_MAX / inf
// the safe way).
__device__ __forceinline__ float mag_below(float v) { return fabsf(v); }
__device__ __forceinline__ float mag_above(float v) { return fabsf(v); }
__device__ __forceinline__ float mag_below(double v) {
  const unsigned long long u = bits_of(v) & 0x7fffffffffffffffull;
  const int e = (int)(u >> 52) - 1023 + 127;
  if (e <= 0) return 0.0f;
  if (e >= 255) return 3.4028234663852886e38f;
  return __uint_as_float(((unsigned)e << 23) | (unsigned)((u >> 29) & 0x7fffffu));
}
__device__ __forceinline__ float mag_above(double v) {
  const unsigned long long u = bits_of(v) & 0x7fffffffffffffffull;
  const int e = (int)(u >> 52) - 1023 + 127;
  if (u == 0ull) return 0.0f;
  if (e <= 0) return 1.17549435e-38f;
  if (e >= 255) return __int_as_float(0x7f800000);
  return __uint_as_float((((unsigned)e << 23) | (unsigned)((u >> 29) & 0x7fffffu)) + 1u);
}

// Row i strictly diagonally dominant: |b_i| > |a_i| + |c_i| (the caller
// passes 0 for a_0 and c_{n-1}).  FP32 compares the values themselves; FP64
// compares the FP32 bounds above with the sum rounded up, so it never
// accepts a row that is not dominant (and keeps the test off the FP64 pipe).
template <typename T>
__device__ __forceinline__ bool dominant_row(T a, T b, T c) {
  const float off = mag_above(a) + mag_above(c);
  const float bound = sizeof(T) == 8 ? __uint_as_float(__float_as_uint(off) + 1u) : off;
  return mag_below(b) > bound;
}

// ---------------------------------------------------------------------------
// Streaming memory access with cache hints.  Inputs that are read once go
// through the read-only path and are marked evict-first; values re-read soon
// (forward-sweep intermediates) use the default policy.

template <typename T>
__device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }
template <typename T>
__device__ __forceinline__ T ld_keep(const T* p) { return __ldcg(p); }
template <typename T>
__device__ __forceinline__ void st_stream(T* p, T v) { __stcs(p, v); }
template <typename T>
__device__ __forceinline__ void st_keep(T* p, T v) { __stcg(p, v); }

// ---------------------------------------------------------------------------
// Warp helpers.
constexpr unsigned FULL = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T shfl(T v, int lane) { return __shfl_sync(FULL, v, lane); }
template <typename T>
__device__ __forceinline__ T shfl_up(T v, int d) { return __shfl_up_sync(FULL, v, d); }
template <typename T>
__device__ __forceinline__ T shfl_down(T v, int d) { return __shfl_down_sync(FULL, v, d); }

}  // namespace tdg
