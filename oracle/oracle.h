/*
 * CPU oracle for the batched tridiagonal solve (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's CPU solvers plus an FP64 pivoted
 * elimination.  Only the test suite, the smoke check and the CPU-baseline leg
 * of bench.py may load this library, and only as the checker of the CUDA
 * library's results; the product path never calls into it.
 *
 * Data layout is the reference's "layout 0": four arrays a, b, c, d of
 * n*batch elements, system j occupying [j*n, (j+1)*n).  a[j*n] and
 * c[j*n+n-1] are ignored (treated as 0).  Every solver is in place like the
 * reference: a and b are preserved, c may be overwritten, d receives x.
 *
 * Parity is pinned: tests/golden holds outputs of the reference's own CPU
 * kernels (built from Tridiagonal_AVX512/ by oracle/Makefile) and the tests
 * require the solvers below to reproduce them bit for bit.
 */
#ifndef TRIDIAG_ORACLE_H
#define TRIDIAG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Number of OpenMP threads the oracle uses (<=0: all available). */
void orc_set_threads(int n);
int orc_get_threads(void);

/* Thomas algorithm, Tridiagonal_AVX512/tridiagonal_basic.cpp:6-27. */
void orc_thomas_f32(float *a, float *b, float *c, float *d, int n, int batch);
void orc_thomas_f64(double *a, double *b, double *c, double *d, int n, int batch);

/* Cyclic reduction with `levels` odd/even levels, then Thomas, then
 * back-substitution: Tridiagonal_AVX512/tridiagonal_basic.cpp:29-128
 * (the reference instantiates levels = 7).  Needs n % 2^levels == 0.
 * Returns 0, or -1 on bad arguments / allocation failure. */
int orc_cr_f32(float *a, float *b, float *c, float *d, int n, int batch, int levels);
int orc_cr_f64(double *a, double *b, double *c, double *d, int n, int batch, int levels);

/* PCR-pThomas: `steps` PCR steps (strides 1,2,..,2^(steps-1)) decouple the
 * system into W = 2^steps interleaved chains, each solved by Thomas.
 * Tridiagonal_AVX512/tridiagonal_d_avx512.cpp:419-646 (PCR3_double: steps 3,
 * PCR2_double: steps 2), tridiagonal_s_avx512.cpp:502-785 (PCR4_single:
 * steps 4, PCR3_single: steps 3).  Any n >= 1. */
int orc_pcr_f32(float *a, float *b, float *c, float *d, int n, int batch, int steps);
int orc_pcr_f64(double *a, double *b, double *c, double *d, int n, int batch, int steps);

/* WM-pGE (unpivoted): `rounds` rounds of pairwise block merging reduce each
 * block of B = 2^rounds equations to spike form, then a sequential Gaussian
 * elimination across blocks stores normalised c', d' and a back sweep per
 * block recovers x.  half = 0: WM3_double (rounds 3), WM4_single (rounds 4)
 * (tridiagonal_d_avx512.cpp:74-241, tridiagonal_s_avx512.cpp:86-287);
 * half = 1: WM2_double (rounds 2), WM3_single (rounds 3), where the
 * elimination runs over pairs of blocks and the first block of a pair is
 * not normalised before use (tridiagonal_d_avx512.cpp:243-416,
 * tridiagonal_s_avx512.cpp:290-499).
 * Needs n % B == 0 (half = 0) or n % 2B == 0 (half = 1). */
int orc_wm_f32(float *a, float *b, float *c, float *d, int n, int batch, int rounds, int half);
int orc_wm_f64(double *a, double *b, double *c, double *d, int n, int batch, int rounds, int half);

/* Gaussian elimination with partial pivoting (adjacent-row interchange,
 * second super-diagonal fill), then back substitution: the algorithm of
 * LAPACK ?gtsv that the reference's MKL row calls
 * (Tridiagonal_AVX512/tridiagonal_basic.cpp:131-143).  a, b, c are
 * overwritten with the factors.  Returns 0, or k+1 if U(k,k) == 0 in the
 * first failing system (that system's d is left unsolved). */
int orc_gtsv_f32(float *a, float *b, float *c, float *d, int n, int batch);
int orc_gtsv_f64(double *a, double *b, double *c, double *d, int n, int batch);

/* Block tridiagonal systems with 2 x 2 blocks (no reference counterpart):
 * A_i x_{i-1} + B_i x_i + C_i x_{i+1} = d_i, blocks row-major, block (i, j)
 * at a[(j*n + i)*4], right-hand side at d[(j*n + i)*2].  gbsv = partial
 * pivoting over the scalar band (the LAPACK ?gbsv algorithm, kl = ku = 3);
 * thomas = block Thomas with 2 x 2 inverses, no pivoting.  x is returned in
 * d; a, b, c are not modified; infos[j] (may be NULL) = 0 or the first
 * zero-pivot scalar column (gbsv) / singular block row (thomas), 1-based.
 * Returns the code of the first failing system, or 0. */
int orc_block2_gbsv_f32(const float *a, const float *b, const float *c, float *d, int *infos, int n, int batch);
int orc_block2_gbsv_f64(const double *a, const double *b, const double *c, double *d, int *infos, int n, int batch);
int orc_block2_thomas_f32(const float *a, const float *b, const float *c, float *d, int *infos, int n, int batch);
int orc_block2_thomas_f64(const double *a, const double *b, const double *c, double *d, int *infos, int n,
                          int batch);

/* Adjoint of x = A^{-1} d for L = sum(xbar * x) in FP64: lambda = A^{-T} xbar
 * from the pivoted LU of A, then grad_d = lambda, grad_a_i = -lambda_i x_{i-1},
 * grad_b_i = -lambda_i x_i, grad_c_i = -lambda_i x_{i+1}.  Inputs are not
 * modified.  x is the solution of the forward solve.  Returns 0 or k+1 on a
 * zero pivot. */
int orc_adjoint_f64(const double *a, const double *b, const double *c, const double *x,
                    const double *xbar, double *ga, double *gb, double *gc, double *gd,
                    int n, int batch);

/* r = d - A x per system in FP64 (compensated dot product). */
void orc_residual_f64(const double *a, const double *b, const double *c, const double *d,
                      const double *x, double *r, int n, int batch);

/* Normwise backward error per system:
 * eta_j = ||d - A x||_inf / (||A||_inf ||x||_inf + ||d||_inf), in FP64.
 * Writes batch values into eta; returns the maximum over systems. */
double orc_backward_error_f64(const double *a, const double *b, const double *c,
                              const double *d, const double *x, double *eta, int n, int batch);

/* The reference driver's error statistics of x against xref over `size`
 * elements: mean |e|, RMS, max |e| (a NaN wins the max), index of the max.
 * Tridiagonal_AVX512/check.c:52-163, Tridiagonal_CUDA/utils.cu:28-219.
 * stats[0..2] = mean, rms, max. Returns the argmax. */
int orc_check_f64(const double *x, const double *xref, int size, double *stats);

#ifdef __cplusplus
}
#endif
#endif
