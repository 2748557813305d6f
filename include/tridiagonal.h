/*
 * Batched tridiagonal solvers for one NVIDIA GB300 (sm_103a): C ABI of
 * libtridiag.so.
 *
 * Part 1 keeps the solver entry points of the reference's
 * Tridiagonal_CUDA/tridiagonal.h (NIC0NIC0NI/TridiagonalSolver) with the same
 * names, signatures and contract, so the reference's driver links against
 * this library unchanged:
 *   - all pointers are DEVICE pointers allocated by the caller;
 *   - layout 0: a, b, c, d hold n_batch systems of n_eqt rows, system j in
 *     [j*n_eqt, (j+1)*n_eqt); a[j*n_eqt] and c[j*n_eqt+n_eqt-1] are unused;
 *   - in place: a and b are preserved, c may be overwritten, d receives x;
 *   - synchronous: each call returns after the solve completed
 *     (cudaDeviceSynchronize, as the reference's wrappers do).
 * The reference's entry points return void; the status of the last call on
 * the calling thread is available from tridiag_last_status().
 *
 * Part 2 adds int-returning entry points (0 = success, TRIDIAG_ERR_* else)
 * that take a layout, an algorithm and a CUDA stream (cudaStream_t passed as
 * void*; NULL = legacy default stream).  They are asynchronous: they return
 * after enqueueing work on the stream.
 */
#ifndef TRIDIAGONAL_H_INCLUDED
#define TRIDIAGONAL_H_INCLUDED 1

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Part 1: the reference's entry points (Tridiagonal_CUDA/tridiagonal.h).    */

/* cuSPARSE gtsv2StridedBatch, the reference's vendor row -- replaces
 * Tridiagonal_CUDA/tridiagonal.h:8-12 (Tridiagonal_CUDA/tridiagonal_basic.cu:
 * 207-246): NVIDIA's library solve with the same init (handle + library
 * workspace, returns 0 or an error) / synchronous solve / final protocol.
 * Status of the last cuSparse_* call: tridiag_vendor_last_status(). */
int cuSparse_init_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
int cuSparse_init_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void cuSparse_final(void);
void cuSparse_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void cuSparse_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
int tridiag_vendor_last_status(void);

/* BPLG -- replaces Tridiagonal_CUDA/tridiagonal.h:14-17 (FP32, packed
 * layout 1: [batch][a|b|c|d][n] at a_gbl; b_gbl, c_gbl, d_gbl are ignored,
 * x lands in the d rows).  Served by this library's kernels: BPLG_WM ->
 * WM-pGE, BPLG_CR and BPLG_LF -> CR-PCR, BPLG_PCR -> PCR-pThomas. */
void BPLG_WM(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void BPLG_LF(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void BPLG_CR(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void BPLG_PCR(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);

/* WM-pGE (partitioned Gaussian elimination, reduced interface system by
 * PCR) -- replaces Tridiagonal_CUDA/tridiagonal.h:32,37,42,47
 * (WM{5,4}_{shmem,reg}; kernels Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:
 * 17-884).  One kernel family serves all four variants of each precision:
 * systems that fit one warp (n <= 1024 FP32, 512 FP64) run the on-chip
 * version without pivoting, as the reference does; longer systems run the
 * partitioned solve with partial pivoting inside each partition (one CTA,
 * or a cluster of up to 8 CTAs, per system: up to 65536 rows FP32 / 27648
 * FP64), beyond that the Thomas sweep. */
void WM5_shmem_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void WM4_shmem_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void WM5_reg_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void WM4_reg_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void WM5_shmem_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void WM4_shmem_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void WM5_reg_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void WM4_reg_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);

/* PCR-pThomas (5 PCR steps split the system into 32 interleaved chains,
 * each solved by Thomas) -- replaces Tridiagonal_CUDA/tridiagonal.h:33-34,
 * 38-39,43-44,48-49 (PCR{5,4}_{shmem,reg}; kernels
 * Tridiagonal_CUDA/tridiagonal_wm_pcr.cu:886-1431).  One on-chip kernel
 * serves all four variants of each precision. */
void PCR5_shmem_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void PCR4_shmem_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void PCR5_reg_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void PCR4_reg_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void PCR5_shmem_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void PCR4_shmem_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void PCR5_reg_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void PCR4_reg_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);

/* CR -- replaces Tridiagonal_CUDA/tridiagonal.h:24-28 (global-memory cyclic
 * reduction, Tridiagonal_CUDA/tridiagonal_basic.cu:32-204) and the
 * register-packed CR_reg{4,8,16} of tridiagonal.h:50-55
 * (Tridiagonal_CUDA/tridiagonal_onchip.cu:218-820).  All run the on-chip
 * CR-PCR hybrid (cyclic reduction in registers, warp PCR on the reduced
 * rows).  It needs no scratch: CR_init_* validates the sizes and returns 0
 * without allocating, CR_final does nothing. */
int CR_init_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
int CR_init_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void CR_final(void);
void CR_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void CR_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void CR_reg4_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void CR_reg8_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void CR_reg16_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);
void CR_reg4_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void CR_reg8_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void CR_reg16_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);

/* naive Thomas -- replaces Tridiagonal_CUDA/tridiagonal.h:20-21 (kernel
 * Tridiagonal_CUDA/tridiagonal_basic.cu:4-30, wrappers :171-190). */
void Thomas_single(float *a_gbl, float *b_gbl, float *c_gbl, float *d_gbl, int n_eqt, int n_batch);
void Thomas_double(double *a_gbl, double *b_gbl, double *c_gbl, double *d_gbl, int n_eqt, int n_batch);

/* ------------------------------------------------------------------------ */
/* Part 2: extensions (no counterpart in the reference unless stated).       */

/* status codes */
#define TRIDIAG_SUCCESS 0
#define TRIDIAG_ERR_INVALID_VALUE 1 /* bad size, null pointer, unknown layout/algorithm */
#define TRIDIAG_ERR_NOT_SUPPORTED 2 /* valid but unsupported combination */
#define TRIDIAG_ERR_CUDA 3          /* a CUDA runtime call or launch failed */
#define TRIDIAG_ERR_WORKSPACE 4     /* workspace missing or too small */
#define TRIDIAG_ERR_SINGULAR 5      /* a zero pivot was met (see info arrays) */
#define TRIDIAG_ERR_TIMEOUT 6       /* a bounded device-side wait gave up */

/* layouts: 0 and 1 are the reference's (Tridiagonal_CUDA/helpers.h:17);
 * 2 is new: row i of system j at [i*n_batch + j] in each of a, b, c, d. */
#define TRIDIAG_LAYOUT_CONTIGUOUS 0
#define TRIDIAG_LAYOUT_PACKED 1
#define TRIDIAG_LAYOUT_INTERLEAVED 2

/* algorithms */
#define TRIDIAG_ALGO_AUTO 0
#define TRIDIAG_ALGO_THOMAS 1 /* unpivoted, one thread per system */
#define TRIDIAG_ALGO_CR 2     /* CR-PCR hybrid, one warp per system */
#define TRIDIAG_ALGO_PCR 3    /* PCR-pThomas, one warp per system */
#define TRIDIAG_ALGO_WM 4     /* WM-pGE, one warp per system, unpivoted */
#define TRIDIAG_ALGO_GTSV 5   /* partial pivoting: PGE for n >= 512 where it fits, else one thread per system */
#define TRIDIAG_ALGO_PGE 6    /* WM-pGE with partial pivoting inside partitions, one CTA per system */
#define TRIDIAG_ALGO_PARTITION 7 /* partition method without pivoting: one CTA per system for n <= 8192 FP32 /
                                    4096 FP64 (contiguous / packed, any n); chunks of 4096 / 2048 rows per CTA for
                                    longer systems whose n is a multiple of 32 / 16 (contiguous, up to 262144 /
                                    65536) */

/* Status of the last library call made by the calling host thread. */
int tridiag_last_status(void);
/* Static description of a status code. */
const char *tridiag_status_string(int status);
/* Library version as major*10000 + minor*100 + patch. */
int tridiag_version(void);
/* First error a kernel recorded on the device since the last reset (0 if
 * none; TRIDIAG_ERR_TIMEOUT when a bounded wait gave up).  Synchronous. */
int tridiag_device_error(int reset);

/* In-place solve with the reference's contract (c may be overwritten, d <- x)
 * in any layout.  For TRIDIAG_LAYOUT_PACKED pass the packed base pointer as
 * a and NULL for b, c, d.  TRIDIAG_ALGO_GTSV allocates its workspace with
 * cudaMallocAsync on `stream`.  The unpivoted algorithms (AUTO, THOMAS, CR,
 * PCR, PARTITION) assume systems that need no pivoting (e.g. diagonally
 * dominant); AUTO picks TRIDIAG_ALGO_PARTITION where it applies and n > 1024,
 * else Thomas; CR and PCR beyond one warp's reach use PARTITION where it
 * applies.  WM keeps the pivoted partitioned solve beyond one warp. */
int tridiag_solve_single(int algo, int layout, float *a, float *b, float *c, float *d, int n_eqt, int n_batch,
                         void *stream);
int tridiag_solve_double(int algo, int layout, double *a, double *b, double *c, double *d, int n_eqt,
                         int n_batch, void *stream);

/* Out-of-place solve: a, b, c, d are read only, x receives the solution.
 * TRIDIAG_ALGO_WM runs the on-chip WM-pGE where the shape allows (contiguous
 * layout), the pivoted partitioned solve beyond it; AUTO runs the
 * unpivoted TRIDIAG_ALGO_PARTITION where it applies and n > 1024, else as WM
 * (CR and PCR beyond one warp: PARTITION where it applies).  These need no
 * workspace; shapes none of them covers, and TRIDIAG_ALGO_THOMAS / GTSV, use
 * `work` of tridiag_solve_out_workspace_size() bytes.  The packed layout is
 * not supported here. */
size_t tridiag_solve_out_workspace_size(int precision, int algo, int layout, int n_eqt, int n_batch);
int tridiag_solve_out_single(int algo, int layout, const float *a, const float *b, const float *c, const float *d,
                             float *x, void *work, size_t work_bytes, int n_eqt, int n_batch, void *stream);
int tridiag_solve_out_double(int algo, int layout, const double *a, const double *b, const double *c,
                             const double *d, double *x, void *work, size_t work_bytes, int n_eqt, int n_batch,
                             void *stream);

/* Out-of-place solve with a, b, c, d and x in HOST memory (no counterpart in
 * the reference, whose test harness, Tridiagonal_CUDA/utils.cu:259-281,
 * copies each array to the device before the call).  The batch streams
 * through device buffers in chunks of `chunk` systems (0: about 96 MB of
 * inputs per chunk; interleaved batches in one piece, as 2-D copies of
 * chunks move far below the link's rate): host -> device copies, the solve of
 * tridiag_solve_out_* with `algo`, device -> host copy of x, on three
 * streams of the library's own, so that the copies of one chunk overlap the
 * solve of another; the streams and a ring of three chunk buffers persist per
 * device (grown on demand) and are shared by all such calls, so that calls
 * made from independent caller streams keep the host link busy back to back.
 * Layouts: contiguous and interleaved (2-D copies).  Ordered after the work
 * queued on `stream`; work queued on `stream` afterwards runs after x is
 * complete in host memory.  Returns once the copies are queued: x is valid
 * after `stream` is synchronised.  Page-locked host memory moves at the
 * link's rate; pageable memory works but the driver stages it. */
int tridiag_solve_host_single(int algo, int layout, const float *a, const float *b, const float *c, const float *d,
                              float *x, int n_eqt, int n_batch, int chunk, void *stream);
int tridiag_solve_host_double(int algo, int layout, const double *a, const double *b, const double *c,
                              const double *d, double *x, int n_eqt, int n_batch, int chunk, void *stream);

/* Bytes of workspace tridiag_gtsv_* needs (precision: 0 = single, 1 = double). */
size_t tridiag_gtsv_workspace_size(int precision, int layout, int n_eqt, int n_batch);
/* Bytes of the pivot record written by tridiag_gtsv_* (one bit per row). */
size_t tridiag_pivot_record_size(int n_eqt, int n_batch);

/* Gaussian elimination with partial pivoting (the algorithm of LAPACK ?gtsv,
 * the reference's MKL row: Tridiagonal_AVX512/tridiagonal_basic.cpp:131-143).
 * a, b, c are read only; d holds the right-hand side on entry and x on exit.
 * pivots (may be NULL) receives the pivot record for tridiag_gtsv_adjoint_*;
 * info (may be NULL) receives per system 0 or k+1 for the first zero pivot
 * U(k,k).  work: tridiag_gtsv_workspace_size() bytes.  With a pivot record:
 * one thread per system (two from both ends where the layout allows).
 * Without one, from n = 512 on: the partitioned solve with partial pivoting
 * inside partitions (one CTA or a cluster per system; contiguous FP64 from
 * 12288 rows and any longer contiguous system in chunks of 4224 rows, one CTA
 * each), which checks every result's backward error and hands a system that
 * misses it to the sequential solve.  Layout 1 (packed): a is the packed base
 * pointer (b and c are ignored) and d points at the right-hand-side rows of
 * system 0 with the packed stride 4n between systems (a + 3n solves in place). */
int tridiag_gtsv_single(int layout, const float *a, const float *b, const float *c, float *d,
                        unsigned int *pivots, int *info, void *work, size_t work_bytes, int n_eqt, int n_batch,
                        void *stream);
int tridiag_gtsv_double(int layout, const double *a, const double *b, const double *c, double *d,
                        unsigned int *pivots, int *info, void *work, size_t work_bytes, int n_eqt, int n_batch,
                        void *stream);

/* Adjoint of x = A^{-1} d for a scalar loss with dL/dx = xbar: solves
 * A^T lambda = xbar reusing the pivots of the forward tridiag_gtsv_* call
 * (the factors are recomputed from a, b, c with those pivots, bit-identical
 * to the forward factorisation), then writes
 *   gd = lambda, ga_i = -lambda_i x_{i-1}, gb_i = -lambda_i x_i,
 *   gc_i = -lambda_i x_{i+1}   (ga_0 = gc_{n-1} = 0).
 * x is the forward solution.  work: tridiag_gtsv_workspace_size() bytes. */
int tridiag_gtsv_adjoint_single(int layout, const float *a, const float *b, const float *c, const float *x,
                                const unsigned int *pivots, const float *xbar, float *ga, float *gb, float *gc,
                                float *gd, void *work, size_t work_bytes, int n_eqt, int n_batch, void *stream);
int tridiag_gtsv_adjoint_double(int layout, const double *a, const double *b, const double *c, const double *x,
                                const unsigned int *pivots, const double *xbar, double *ga, double *gb,
                                double *gc, double *gd, void *work, size_t work_bytes, int n_eqt, int n_batch,
                                void *stream);

/* Mixed-precision refined solve (no counterpart in the reference): FP64
 * arrays in and out, the eliminations in FP32.  a, b, c, d are converted to
 * FP32 once, x0 is the FP32 partial-pivoting solve, and each of `iters`
 * refinement steps forms r = d - A x in FP64 and adds the FP32 solve of
 * A dx = r.  Two steps bring the normwise backward error to the FP64 level
 * for condition numbers up to ~1e7.  Layouts: contiguous or interleaved.
 * a, b, c, d are read only; x receives the solution; info (may be NULL) as
 * tridiag_gtsv_*, from the FP32 factorisation.  iters in [0, 8].
 * work: tridiag_refine_workspace_size() bytes. */
size_t tridiag_refine_workspace_size(int layout, int n_eqt, int n_batch);
int tridiag_refine_double(int layout, const double *a, const double *b, const double *c, const double *d,
                          double *x, int iters, int *info, void *work, size_t work_bytes, int n_eqt, int n_batch,
                          void *stream);
/* The same with a choice of FP32 solver: TRIDIAG_ALGO_GTSV (or AUTO; partial
 * pivoting, as tridiag_refine_double) or TRIDIAG_ALGO_PARTITION (the
 * unpivoted partition method, for systems that need no pivoting such as
 * diagonally dominant ones; contiguous layout where its kernels cover the
 * shape, else the Thomas sweep; info is set to 0). */
int tridiag_refine_ex_double(int algo, int layout, const double *a, const double *b, const double *c,
                             const double *d, double *x, int iters, int *info, void *work, size_t work_bytes,
                             int n_eqt, int n_batch, void *stream);

/* FP64 -> FP32 narrowing (round to nearest even) and FP32 -> FP64 widening
 * as the refined solve performs them on the integer pipe: out[k] = (float)
 * in[k], back[k] = (double)out[k].  For tests of that conversion. */
int tridiag_convert_check(const double *in, float *out, double *back, size_t count, void *stream);

/* WM-pGE with partial pivoting inside each partition, the system staged in
 * shared memory of one CTA (n up to 8960 FP32 / 4736 FP64) or of a cluster
 * of 2, 4 or 8 CTAs (n up to 65536 FP32 / 27648 FP64); contiguous or packed
 * layout, n >= 65, else TRIDIAG_ERR_NOT_SUPPORTED.  The NT threads of a CTA
 * each eliminate one partition (three right-hand sides);
 * the separator system is solved by PCR, or with partial pivoting when
 * PCR's result fails a backward-error check; results whose separator rows
 * miss the residual bound and then an exact backward-error check are
 * refined in the kernel (FP64 residual, up to two correction passes) and,
 * if that does not reach the bound, recomputed by a sequential
 * partial-pivoting solve (clusters: info = n + 1 instead).  a, b, c, d are
 * read only (x may alias d); info (may be NULL) as tridiag_gtsv_*. */
int tridiag_pge_single(int layout, const float *a, const float *b, const float *c, const float *d, float *x,
                       int *info, int n_eqt, int n_batch, void *stream);
int tridiag_pge_double(int layout, const double *a, const double *b, const double *c, const double *d, double *x,
                       int *info, int n_eqt, int n_batch, void *stream);

/* Adjoint through the partitioned solve (no pivot record needed): solves
 * A^T lambda = xbar with tridiag_pge_* on the transposed coefficients
 * (sub-diagonal c_{i-1}, super-diagonal a_{i+1}) and writes gd = lambda,
 * ga_i = -lambda_i x_{i-1}, gb_i = -lambda_i x_i, gc_i = -lambda_i x_{i+1}
 * (ga_0 = gc_{n-1} = 0); x is the forward solution.  Sizes as tridiag_pge_*;
 * info (may be NULL) refers to A^T. */
int tridiag_pge_adjoint_single(int layout, const float *a, const float *b, const float *c, const float *x,
                               const float *xbar, float *ga, float *gb, float *gc, float *gd, int *info, int n_eqt,
                               int n_batch, void *stream);
int tridiag_pge_adjoint_double(int layout, const double *a, const double *b, const double *c, const double *x,
                               const double *xbar, double *ga, double *gb, double *gc, double *gd, int *info,
                               int n_eqt, int n_batch, void *stream);

/* Adjoint through the unpivoted partition method (TRIDIAG_ALGO_PARTITION;
 * no counterpart in the reference): solves A^T lambda = xbar with the
 * partition kernel on the transposed coefficients and writes the gradients
 * as tridiag_pge_adjoint_*.  Contiguous layout and the shapes
 * TRIDIAG_ALGO_PARTITION covers (else TRIDIAG_ERR_NOT_SUPPORTED); systems that
 * need no pivoting, as for the forward solve. */
/* 1 if TRIDIAG_ALGO_PARTITION's single-CTA kernel (which the adjoint uses)
 * covers (precision, layout, n). */
int tridiag_partition_supported(int precision, int layout, int n_eqt);
int tridiag_partition_adjoint_single(int layout, const float *a, const float *b, const float *c, const float *x,
                                     const float *xbar, float *ga, float *gb, float *gc, float *gd, int n_eqt,
                                     int n_batch, void *stream);
int tridiag_partition_adjoint_double(int layout, const double *a, const double *b, const double *c,
                                     const double *x, const double *xbar, double *ga, double *gb, double *gc,
                                     double *gd, int n_eqt, int n_batch, void *stream);

/* Ragged batches (no counterpart in the reference): n_batch systems of
 * different sizes packed back to back in a, b, c, d (and x): system s is
 * rows [offsets[s], offsets[s+1]) with 1 <= size <= 2^(TRIDIAG_RAGGED_CLASSES-1).
 * A plan, built on the host from the offsets, groups the systems into size
 * classes (class k: 2^(k-1) < n <= 2^k) and picks a kernel variant per class:
 * 0 = thread-per-system sequential partial pivoting (n <= 64), 1/2/3 = the
 * partitioned solve in one CTA with 64/128/256 partitions, 4/5/6 = in a
 * cluster of 2/4/8 CTAs, 9 = thread-per-system sequential partial pivoting
 * with the eliminated rows in a plan workspace (any n; 2 values + 1 bit per
 * row of its classes), 10 = the partitioned solve in chunks of 4224 rows (one
 * CTA each) with the separators' systems solved in between, each chunk's
 * result checked and a failing system re-solved by 9 (the default where no
 * one-CTA or cluster variant serves the class: FP64 beyond 27648 rows, FP32
 * beyond 65536; ~0.15 values of workspace per row besides 9's).  variant_by_class (may
 * be NULL; entries < 0 mean "default") overrides the choice per class -- the
 * autotuner's output; an entry that cannot serve its class's sizes makes the
 * call return TRIDIAG_ERR_NOT_SUPPORTED.
 * tridiag_ragged_solve_* / _adjoint_* issue one launch per non-empty bucket
 * on the stream (capturable in one CUDA graph); offsets is the device copy of
 * the offsets used to build the plan.  info (may be NULL) per system.  A plan
 * is used by one stream at a time (it holds the bucket tickets and kinds). */
#define TRIDIAG_RAGGED_CLASSES 18
typedef struct tridiag_ragged_plan tridiag_ragged_plan;
int tridiag_ragged_plan_create(tridiag_ragged_plan **plan, int precision, const long long *offsets_host, int n_batch,
                               const int *variant_by_class, int n_classes);
/* As tridiag_ragged_plan_create, with no_pivoting_host (may be NULL; one
 * byte per system): systems marked 1 need no pivoting (diagonally dominant,
 * say) and run the unpivoted partition method in buckets of their own:
 * variant 7, one CTA per system (n <= 4096 FP32 / 2048 FP64), and variant 8
 * for longer ones (chunks of that size per CTA and the separators' system in
 * between; n <= 262144 FP32 / 65536 FP64; the plan holds ~14 values of
 * workspace per 32 (FP32) / 16 (FP64) rows); info entries of those systems
 * are set to 0. */
int tridiag_ragged_plan_create_ex(tridiag_ragged_plan **plan, int precision, const long long *offsets_host,
                                  int n_batch, const int *variant_by_class, int n_classes,
                                  const unsigned char *no_pivoting_host);
/* As tridiag_ragged_plan_create, with the library deciding which systems
 * need no pivoting: every tridiag_ragged_solve_* call starts each system of a
 * size the unpivoted method serves (64 < n <= 262144 FP32 / 65536 FP64) as a
 * candidate; the unpivoted kernels check the rows they stage for strict
 * diagonal dominance by rows (|b_i| > |a_i| + |c_i|) and hand a system that
 * fails, before any arithmetic, to the pivoted bucket of its size class (its
 * list grows on the device; resident CTAs drain every bucket through an
 * atomic ticket, so no count returns to the host).  tridiag_ragged_adjoint_*
 * reuses the marks of the plan's last solve (the same coefficients, as the
 * pivot record of tridiag_gtsv_adjoint_*; called before any solve it marks
 * the systems in a pass of its own).  unpivoted_by_class (may be NULL;
 * entries < 0 = default 7): the variant of the marked systems of each class
 * up to 4096 (FP32) / 2048 (FP64) rows -- 7, or a partitioned pivoted variant
 * 1-6; chunk_rows: 128-byte rows per CTA of variant 8 (64, 128 or 256; 0 =
 * 128) -- both the autotuner's choices. */
int tridiag_ragged_plan_create_classify(tridiag_ragged_plan **plan, int precision, const long long *offsets_host,
                                        int n_batch, const int *variant_by_class, const int *unpivoted_by_class,
                                        int n_classes, int chunk_rows);
/* Refined ragged solves (no counterpart in the reference): FP64 systems
 * solved through an FP32 plan (plan32, precision 0) of the same offsets --
 * FP32 copies of the coefficients and the right-hand side, an FP32 solve,
 * then `iters` (0-8) steps of an FP64 residual (one warp per system, the
 * system boundaries respected) and an FP32 correction solve, the FP64
 * iterate updated each step.  tridiag_ragged_refine_double writes x;
 * tridiag_ragged_refine_adjoint_double solves A^T lambda = xbar the same way
 * (FP32 copies of A^T) and
 * writes gd = lambda and the FP64 gradients ga_i = -lambda_i x_{i-1}, gb_i =
 * -lambda_i x_i, gc_i = -lambda_i x_{i+1} from the forward solution x.  a,
 * b, c, d, xbar are read only.  work: tridiag_ragged_refine_workspace_size()
 * bytes (28 per row); offsets: the device copy of the plan's offsets, which
 * must start at 0 (else TRIDIAG_ERR_INVALID_VALUE).  The
 * FP32 solves see the narrowed coefficients: the result reaches FP64
 * accuracy when the FP32 solve converges the iteration (condition number
 * well below 1 / FP32 epsilon).  A classifying plan32 marks the systems by
 * A's rows in the first FP32 solve of tridiag_ragged_refine_double; its other
 * FP32 solves, and those of the adjoint (A strictly diagonally dominant by
 * rows needs no pivoting for A^T either), run on the marks as they stand --
 * an adjoint on a plan with no marks marks by A's rows first. */
size_t tridiag_ragged_refine_workspace_size(long long total_rows);
int tridiag_ragged_refine_double(tridiag_ragged_plan *plan32, const double *a, const double *b, const double *c,
                                 const double *d, double *x, int iters, void *work, size_t work_bytes,
                                 const long long *offsets, void *stream);
int tridiag_ragged_refine_adjoint_double(tridiag_ragged_plan *plan32, const double *a, const double *b,
                                         const double *c, const double *x, const double *xbar, double *ga,
                                         double *gb, double *gc, double *gd, int iters, void *work,
                                         size_t work_bytes, const long long *offsets, void *stream);
/* As the two above, then `pivoted_iters` (0-8) more steps on the systems
 * the plan solves with pivoting only (every system for a plan without marks):
 * the FP64 residual of their rows, an FP32 correction solve of their buckets
 * alone, their rows of x (lambda) updated in place; the systems marked for
 * the unpivoted kernels keep the result of the `iters` steps.  Diagonally
 * dominant systems converge in fewer steps than the ones that need pivoting,
 * so iters = 1, pivoted_iters = 1 costs little more than one step. */
int tridiag_ragged_refine_ex_double(tridiag_ragged_plan *plan32, const double *a, const double *b, const double *c,
                                    const double *d, double *x, int iters, int pivoted_iters, void *work,
                                    size_t work_bytes, const long long *offsets, void *stream);
int tridiag_ragged_refine_adjoint_ex_double(tridiag_ragged_plan *plan32, const double *a, const double *b,
                                            const double *c, const double *x, const double *xbar, double *ga,
                                            double *gb, double *gc, double *gd, int iters, int pivoted_iters,
                                            void *work, size_t work_bytes, const long long *offsets,
                                            void *stream);
/* The marks (1: solved without pivoting) of the plan's last solve, one byte
 * per system, into host memory (synchronous); TRIDIAG_ERR_NOT_SUPPORTED for
 * a plan without marks. */
int tridiag_ragged_plan_kinds(const tridiag_ragged_plan *plan, unsigned char *kinds_host);
void tridiag_ragged_plan_destroy(tridiag_ragged_plan *plan);
/* Buckets of a plan, longest first: 4 ints each (class, variant, systems,
 * largest n); returns the number of buckets. */
int tridiag_ragged_plan_buckets(const tridiag_ragged_plan *plan, int *out, int max_buckets);
/* Largest n a variant serves (0: none). */
int tridiag_ragged_variant_max_n(int precision, int variant);
int tridiag_ragged_solve_single(tridiag_ragged_plan *plan, const float *a, const float *b, const float *c,
                                const float *d, float *x, int *info, const long long *offsets, void *stream);
int tridiag_ragged_solve_double(tridiag_ragged_plan *plan, const double *a, const double *b, const double *c,
                                const double *d, double *x, int *info, const long long *offsets, void *stream);
int tridiag_ragged_adjoint_single(tridiag_ragged_plan *plan, const float *a, const float *b, const float *c,
                                  const float *x, const float *xbar, float *ga, float *gb, float *gc, float *gd,
                                  int *info, const long long *offsets, void *stream);
int tridiag_ragged_adjoint_double(tridiag_ragged_plan *plan, const double *a, const double *b,
                                  const double *c, const double *x, const double *xbar, double *ga, double *gb,
                                  double *gc, double *gd, int *info, const long long *offsets, void *stream);

/* Layout conversion (no counterpart in the reference): copies a, b, c, d of
 * n_batch systems from from_layout to to_layout (TRIDIAG_LAYOUT_*) in one
 * pass over memory, coalesced on both sides (32 x 32 tiles through shared
 * memory).  For the packed layout only the first pointer of the side is used
 * (the others may be NULL).  Source and destination must not overlap.  Lets
 * callers of the reference's layout-0 entry points reach the kernels that
 * prefer another layout (e.g. the interleaved Thomas sweep) and back. */
int tridiag_relayout_single(int from_layout, int to_layout, const float *a, const float *b, const float *c,
                            const float *d, float *a2, float *b2, float *c2, float *d2, int n_eqt, int n_batch,
                            void *stream);
int tridiag_relayout_double(int from_layout, int to_layout, const double *a, const double *b, const double *c,
                            const double *d, double *a2, double *b2, double *c2, double *d2, int n_eqt,
                            int n_batch, void *stream);

/* cuSPARSE-shaped entry points (no counterpart in the reference's own code:
 * the argument lists of cusparse?gtsv2StridedBatch / ?gtsvInterleavedBatch,
 * the library behind the reference's vendor row, Tridiagonal_CUDA/
 * tridiagonal_basic.cu:207-246), served by this library's kernels; no
 * handle.  Query the buffer size first; pBuffer may be NULL when it is 0.
 *   ?gtsv2StridedBatch: dl, d, du read only (dl[0] and du[m-1] ignored), x
 *   holds the right-hand side on entry and the solution on exit, system j at
 *   j*batchStride.  batchStride == m: WM-pGE (on chip for short systems, the
 *   partitioned pivoted solve for longer ones, the Thomas sweep beyond);
 *   batchStride > m: the partitioned solve (65 <= m <= its limits, else
 *   TRIDIAG_ERR_NOT_SUPPORTED).
 *   ?gtsvInterleavedBatch: interleaved layout (row i of system j at
 *   i*batchCount + j); algo 0 or 1 -> partial pivoting (tridiag_gtsv_*),
 *   algo 2 -> Thomas without pivoting, which overwrites du. */
size_t tridiag_gtsv2StridedBatch_bufferSize(int precision, int m, int batchCount, int batchStride);
int tridiag_Sgtsv2StridedBatch(int m, const float *dl, const float *d, const float *du, float *x, int batchCount,
                               int batchStride, void *pBuffer, void *stream);
int tridiag_Dgtsv2StridedBatch(int m, const double *dl, const double *d, const double *du, double *x, int batchCount,
                               int batchStride, void *pBuffer, void *stream);
size_t tridiag_gtsvInterleavedBatch_bufferSize(int precision, int algo, int m, int batchCount);
int tridiag_SgtsvInterleavedBatch(int algo, int m, float *dl, float *d, float *du, float *x, int batchCount,
                                  void *pBuffer, void *stream);
int tridiag_DgtsvInterleavedBatch(int algo, int m, double *dl, double *d, double *du, double *x, int batchCount,
                                  void *pBuffer, void *stream);

/* Periodic (cyclic) systems (no counterpart in the reference): row 0 also
 * couples x_{n-1} with coefficient a_0 and row n-1 couples x_0 with c_{n-1}.
 * Contiguous layout, n >= 3.  Sherman-Morrison over two tridiagonal solves
 * with `algo` (TRIDIAG_ALGO_GTSV / AUTO: partial pivoting; TRIDIAG_ALGO_WM or
 * TRIDIAG_ALGO_THOMAS: without pivoting, for diagonally dominant systems).
 * a, b, c, d read only; x receives the solution (must not alias a, b, c);
 * work: tridiag_periodic_workspace_size() bytes. */
size_t tridiag_periodic_workspace_size(int precision, int algo, int n_eqt, int n_batch);
int tridiag_periodic_single(int algo, const float *a, const float *b, const float *c, const float *d, float *x,
                            void *work, size_t work_bytes, int n_eqt, int n_batch, void *stream);
int tridiag_periodic_double(int algo, const double *a, const double *b, const double *c, const double *d, double *x,
                            void *work, size_t work_bytes, int n_eqt, int n_batch, void *stream);

/* Factor once, solve many right-hand sides (no counterpart in the
 * reference; the algorithm of LAPACK ?gttrf / ?gttrs, one thread per
 * system).  tridiag_factor_* factors the n_batch systems (any layout; a, b,
 * c read only) into `factors` (tridiag_factor_size() bytes of device
 * memory, the caller's); info (may be NULL) per system as tridiag_gtsv_*.
 * tridiag_factored_solve_* then solves A x = r (transpose = 0) or
 * A^T x = r (transpose = 1) for nrhs right-hand sides held in x (block k at
 * k*n*batch elements, contiguous or interleaved layout), in place. */
size_t tridiag_factor_size(int precision, int n_eqt, int n_batch);
int tridiag_factor_single(int layout, const float *a, const float *b, const float *c, void *factors,
                          size_t factor_bytes, int *info, int n_eqt, int n_batch, void *stream);
int tridiag_factor_double(int layout, const double *a, const double *b, const double *c, void *factors,
                          size_t factor_bytes, int *info, int n_eqt, int n_batch, void *stream);
int tridiag_factored_solve_single(int layout, int transpose, const void *factors, size_t factor_bytes, float *x,
                                  int nrhs, int n_eqt, int n_batch, void *stream);
int tridiag_factored_solve_double(int layout, int transpose, const void *factors, size_t factor_bytes, double *x,
                                  int nrhs, int n_eqt, int n_batch, void *stream);

/* Block tridiagonal systems with 2 x 2 blocks (no counterpart in the
 * reference):  A_i x_{i-1} + B_i x_i + C_i x_{i+1} = d_i for block rows
 * i = 0..n_eqt-1 of each of n_batch systems, x_i and d_i in R^2, blocks
 * row-major; A_0 and C_{n-1} are not read.  Layouts:
 *   TRIDIAG_LAYOUT_CONTIGUOUS   block (i, j) at a[(j*n + i)*4 + k],
 *                               right-hand side at d[(j*n + i)*2 + r];
 *   TRIDIAG_LAYOUT_INTERLEAVED  a[(i*4 + k)*n_batch + j], d[(i*2 + r)*n_batch + j].
 * algo TRIDIAG_BLOCK2_PIVOTED: partial pivoting over the scalar band of
 * order 2n (the LAPACK ?gbsv algorithm); a, b, c are overwritten with the
 * factors.  TRIDIAG_BLOCK2_THOMAS: block Thomas without pivoting (block
 * diagonally dominant systems); a and b are kept, c is overwritten.  d
 * receives x.  info (may be NULL) gets per system 0, or the first zero
 * pivot (PIVOTED: scalar column, 1-based) / singular block (THOMAS: block
 * row, 1-based).  One thread per system: batches of 20k systems or more
 * fill the GPU. */
#define TRIDIAG_BLOCK2_PIVOTED 0
#define TRIDIAG_BLOCK2_THOMAS 1
int tridiag_block2_single(int algo, int layout, float *a, float *b, float *c, float *d, int *info, int n_eqt,
                          int n_batch, void *stream);
int tridiag_block2_double(int algo, int layout, double *a, double *b, double *c, double *d, int *info, int n_eqt,
                          int n_batch, void *stream);

/* Diagnostics: how many systems the partitioned partial-pivoting solve (used
 * by tridiag_gtsv_* without a pivot record, tridiag_solve_out_* with
 * TRIDIAG_ALGO_GTSV and the WM entry points on long systems) handed to its
 * sequential fallback on the current device since the last reset -- systems
 * whose partition-local pivoting broke down or failed the solve's
 * growth/residual check.  Synchronous; reset != 0 clears the count; -1 on a
 * CUDA error. */
long long tridiag_partition_fallbacks(int reset);

/* Diagnostics of the same solve, per path taken since the last reset on the
 * current device: counts[0] systems whose separator system, solved by
 * parallel cyclic reduction, missed its residual bound and was solved again
 * with partial pivoting; counts[1] systems whose separator rows missed the
 * residual bound, so that the exact backward error of all rows was measured;
 * counts[2] refinement passes run (FP64 residual as a new right-hand side);
 * counts[3] sequential fallbacks (as tridiag_partition_fallbacks).
 * Synchronous; reset != 0 clears all four.  Returns a TRIDIAG_* status. */
int tridiag_partition_path_counts(long long *counts, int reset);

/* tridiag_gtsv_* without a pivot record on many FP64 systems -- contiguous
 * ones longer than one CTA's shared memory holds (about 5000 rows) and up to
 * 27648, batch-interleaved ones from 1024 rows (batch from 1024, a workspace
 * of tridiag_gtsv_workspace_size()
 * bytes; also TRIDIAG_ALGO_GTSV of tridiag_solve_out_*) cuts each system
 * into partitions of 64-448 rows, one thread each; counts[0] systems it solved and
 * accepted, counts[1] systems that missed its separator-row test and were
 * solved again by the one-CTA partitioned solve, since the last reset on the
 * current device.  Synchronous; reset != 0 clears both. */
int tridiag_partition_ppt_counts(long long *counts, int reset);

/* Size of the static scratch array of tridiag_gtsv_noalloc_* (32 MiB). */
#define TRIDIAG_NOALLOC_SCRATCH_BYTES (32u << 20)

/* Partial-pivoting solve that allocates no device memory (no counterpart in
 * the reference).  For callers that cannot allocate where they solve -- a
 * loop with a hard latency budget, in which cudaMalloc may synchronise the
 * device, or a process whose GPU memory belongs to another allocator or a
 * fixed quota.  Arguments and results as tridiag_gtsv_* (d: right-hand side
 * in, x out; info may be NULL), without pivot record or workspace: the
 * scratch is one static device array of TRIDIAG_NOALLOC_SCRATCH_BYTES that
 * every GPU loading the library holds until exit.  The first call on a
 * device looks up that array's device address; make it before any stream
 * capture.  After cudaDeviceReset the device's next call looks it up again
 * (the array is new with the new context), so that call too belongs before
 * any capture.  Layout 1: a is the packed base, b and c are ignored, d
 * points at the right-hand-side rows (a + 3n in place), as for
 * tridiag_gtsv_*.  All calls share the array, so calls that overlap on the GPU
 * race and must be serialised by the caller.  Returns TRIDIAG_ERR_WORKSPACE,
 * launching nothing, when 2*n*batch*sizeof(T) plus the pivot bits (each
 * rounded up to 256 bytes) exceed the array.  Returns its status directly
 * (tridiag_last_status() is not updated). */
int tridiag_gtsv_noalloc_single(int layout, const float *a, const float *b, const float *c, float *d, int *info,
                                int n_eqt, int n_batch, void *stream);
int tridiag_gtsv_noalloc_double(int layout, const double *a, const double *b, const double *c, double *d,
                                int *info, int n_eqt, int n_batch, void *stream);

#ifdef __cplusplus
}
#endif

#endif
