/*
 * Pre-included when compiling the reference's Tridiagonal_AVX512 kernels with
 * GCC (oracle/Makefile, target `ref`).  It defines the include guard of the
 * reference's vec.h so that header is skipped: its operator overloads on
 * __m512/__m512d are ICC-only (GCC has them built in) and its default FP32
 * division uses AVX-512ER, which this CPU lacks.  The three helpers the
 * kernels call are given here with the reference's -DDIV semantics: IEEE
 * division, zero-masked IEEE division, and -(a*b) as a fused negated
 * multiply-add with zero.
 */
#ifndef TRIDIAG_REF_VEC_SHIM_H
#define TRIDIAG_REF_VEC_SHIM_H
#define VEC_H_INCLUDED
#include <immintrin.h>

static inline __m512d div(__m512d a, __m512d b) { return _mm512_div_pd(a, b); }
static inline __m512 div(__m512 a, __m512 b) { return _mm512_div_ps(a, b); }
static inline __m512d maskz_div(__mmask8 m, __m512d a, __m512d b) { return _mm512_maskz_div_pd(m, a, b); }
static inline __m512 maskz_div(__mmask16 m, __m512 a, __m512 b) { return _mm512_maskz_div_ps(m, a, b); }
static inline __m512d nmul(__m512d a, __m512d b) { return _mm512_fnmadd_pd(a, b, _mm512_setzero_pd()); }
static inline __m512 nmul(__m512 a, __m512 b) { return _mm512_fnmadd_ps(a, b, _mm512_setzero_ps()); }
#endif
