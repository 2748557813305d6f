// Launchers of the device kernels (host side), one family per .cu file.
// All are asynchronous on the given stream and return the launch status.
#pragma once
#include <cuda_runtime.h>

namespace tdg {

// A size bucket served by resident CTAs: each takes the next list entry
// from *ticket (zeroed before the launch) while it is below *dcount (the
// entries a device pass wrote; NULL: the launch's count), and skips the
// systems s with kinds[s] != want (kinds NULL: none skipped).
struct BucketTicket {
  int* ticket = nullptr;
  const int* dcount = nullptr;
  const unsigned char* kinds = nullptr;
  int want = 0;
  const int* only = nullptr;  // (partitioned variants) serve only the systems s with only[s] != 0
};
// Ragged forward solves by the unpivoted method that check the rows they
// stage: a system with a row that is not strictly diagonally dominant is
// not solved there but handed to the pivoted bucket of its size class --
// kinds[s] = 0, and s appended once (claim[s]) to the class's kind-0 list
// (region reg[2 k], length kcount[2 k] of klists).
struct RaggedCheck {
  unsigned char* kinds = nullptr;
  int* claim = nullptr;
  const int* reg = nullptr;
  int* kcount = nullptr;
  int* klists = nullptr;
};

// seq.cu: one thread per system
template <typename T>
cudaError_t launch_thomas_seq(int layout, T* a, T* b, T* c, T* d, int n, int batch, cudaStream_t s);
template <typename T>
cudaError_t launch_gtsv_seq(int layout, const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv,
                            int* info, int n, int batch, cudaStream_t s);
// The sequential solve (contiguous or interleaved) of the systems with mask[j] != 0 only;
// info[j] = 0 for the others.
template <typename T>
cudaError_t launch_gtsv_seq_masked(int layout, const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv,
                                   int* info, int n, int batch, const int* mask, cudaStream_t s);
template <typename T>
cudaError_t launch_gtsv_adjoint(int layout, const T* a, const T* b, const T* c, const T* x, const unsigned* piv,
                                const T* g, T* ga, T* gb, T* gc, T* gd, T* wz, T* wm, int n, int batch,
                                cudaStream_t s);

// tw.cu: two-ended sweeps over TMA-staged tiles (CONTIG / INTERLEAVED).
// *used is false when the arrays cannot be described by tensor maps (the
// caller then falls back to the seq.cu kernels, or reports an error where
// the choice must match an earlier call -- see tw_eligible).
template <typename T>
cudaError_t launch_thomas_tw(int layout, T* a, T* b, T* c, T* d, int n, int batch, cudaStream_t s, bool* used);
template <typename T>
cudaError_t launch_gtsv_tw(int layout, const T* a, const T* b, const T* c, T* d, T* w1, T* w2, unsigned* piv,
                           int* info, int n, int batch, cudaStream_t s, bool* used);
template <typename T>
cudaError_t launch_gtsv_adjoint_tw(int layout, const T* a, const T* b, const T* c, const T* x, const unsigned* piv,
                                   const T* g, T* ga, T* gb, T* gc, T* gd, T* wz, T* wm, int n, int batch,
                                   cudaStream_t s, bool* used);

// Whether the two-ended kernels apply, decided on the shape alone (the row
// stride of a tensor map must be a multiple of 16 bytes).  The pivot record
// format of the pivoted solve depends on this choice, so the forward solve
// and its adjoint always agree.
inline bool tw_eligible(int layout, int n, int batch, int elem) {
  if (layout == 2) return ((size_t)batch * elem) % 16 == 0;
  if (layout == 0) return ((size_t)n * elem) % 16 == 0;
  return false;
}

// The library's device error word on the current device (allocated on first
// use, 4 bytes per device), and a synchronous read (optionally clearing it).
int* error_word();
// Ticket counters for persistent kernels that hand out work dynamically: a
// (next, done) pair of ints, zero, one of RING_TICKET_SLOTS per device taken
// in turn per launch; the launch's last CTA sets it to zero again.  (Two
// launches share a pair only when RING_TICKET_SLOTS launches are in flight.)
constexpr unsigned RING_TICKET_SLOTS = 256;
int* ring_tickets();
cudaError_t read_device_error(int* code, bool reset);

// wm.cu: WM-pGE, one warp per system (CONTIG / PACKED, n <= 1024 FP32,
// 512 FP64).  x may alias d.  *used is false when the shape is not covered.
template <typename T>
cudaError_t launch_wm_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                           cudaStream_t st, bool* used);

// wmc.cu: partition method without pivoting, one CTA per system
// (CONTIG / PACKED; n = R * 128 / sizeof(T) with 8 <= R <= 256).  x may alias
// d (PACKED: must).  *used is false when the shape is not covered.
template <typename T>
bool wmc_eligible(int layout, int n);
// any n up to 256 128-byte rows (element-wise staging), CONTIG / PACKED
template <typename T>
bool wmc_gen_eligible(int layout, int n);
// ragged: mode 0 solve (a, b, c, d -> o0 = x), mode 1 adjoint (a, b, c,
// d = xbar, xf = x -> o0..o3 = ga, gb, gc, gd) of systems list[0..count),
// each at most Rmax 128-byte rows
constexpr int WMC_GEN_MAX_ROWS = 256;  // 128-byte rows per system of the general staging
// partitions (128-byte rows) per CTA of the chunked kernels: ~68 KB of
// shared memory, three CTAs per SM, so one CTA's loads overlap another's
// arithmetic
constexpr int WML_CHUNK_R = 128;
// Long unpivoted systems of a ragged plan: L systems (l_sys), their
// partitions' offsets roff (L+1, P in total, largest Pmax) and C chunks
// (cl_li, cl_ch) of 256 128-byte rows.
struct WmlRagged {
  int L = 0, C = 0, Pmax = 0;
  int R = WML_CHUNK_R;  // 128-byte rows per chunk CTA (64, 128 or 256)
  long long P = 0;
  const int* l_sys = nullptr;
  const long long* roff = nullptr;
  const int* cl_li = nullptr;
  const int* cl_ch = nullptr;
};
template <typename T>
size_t wml_ragged_workspace_elems(long long total_partitions);
// kinds (may be NULL): the long systems s with kinds[s] != 1 are skipped
// (a pivoted bucket serves them); chk (forward solves, may be NULL): the
// chunks check the rows they stage (RaggedCheck).
template <typename T>
cudaError_t launch_wml_ragged(int mode, const T* a, const T* b, const T* c, const T* d, const T* xf, T* o0, T* o1,
                              T* o2, T* o3, const long long* offsets, const WmlRagged& lr, T* work, int* info,
                              cudaStream_t s, const unsigned char* kinds = nullptr,
                              const RaggedCheck* chk = nullptr);
// tk (may be NULL): skip systems by kind; with a ticket, resident CTAs drain
// the bucket.  kind_map: the kinds index of launch system j (NULL: j).
// chk: as for launch_wml_ragged (mode 0).
template <typename T>
cudaError_t launch_wmc_ragged(int mode, const T* a, const T* b, const T* c, const T* d, const T* xf, T* o0, T* o1,
                              T* o2, T* o3, const long long* offsets, const int* list, int count, int Rmax, int* info,
                              cudaStream_t s, const BucketTicket* tk = nullptr, const int* kind_map = nullptr,
                              const RaggedCheck* chk = nullptr);
template <typename T>
cudaError_t launch_wmc(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                       cudaStream_t s, bool* used);
// wmc.cu: the same method for long systems (CONTIG, n a multiple of
// 128 / sizeof(T) beyond one CTA's reach): chunks per CTA, the separators'
// system by the single-CTA kernel, chunks again; `work` of
// wml_workspace_bytes().  *used is false when not covered.
template <typename T>
bool wml_eligible(int layout, int n);
template <typename T>
size_t wml_workspace_bytes(int n, int batch);
template <typename T>
cudaError_t launch_wml(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch, void* work,
                       size_t work_bytes, cudaStream_t s, bool* used);

// wmc.cu: adjoint of the unpivoted partition solve (CONTIG): A^T lambda =
// xbar and the gradients ga, gb, gc, gd = lambda.
template <typename T>
cudaError_t launch_wmc_adjoint(const T* a, const T* b, const T* c, const T* x, const T* xbar, T* ga, T* gb, T* gc,
                               T* gd, int n, int batch, cudaStream_t s, bool* used);

// wm.cu: PCR-pThomas on the persistent TMA-fed chunk kernel (CONTIG,
// n = 512 FP32 / 256 FP64); *used is false for other shapes.
template <typename T>
cudaError_t launch_pcr_tma(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                           cudaStream_t st, bool* used);

// wm.cu: CR-PCR hybrid on the same chunk layout (cyclic reduction in
// registers down to one row per lane, warp PCR on those rows).
template <typename T>
cudaError_t launch_crpcr_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                              cudaStream_t st, bool* used);

// pcr.cu: PCR-pThomas, one warp per system (CONTIG / PACKED, n <= 1024
// FP32, 512 FP64).  x may alias d.
template <typename T>
cudaError_t launch_pcr_warp(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch,
                            cudaStream_t st, bool* used);

// pge.cu: partitioned partial-pivoting solve (WM-pGE), one CTA per system
// staged in shared memory (CONTIG / PACKED; n up to ~5K FP64, ~8K FP32).
// Writes no pivot record.  x may alias d; info (may be null) per system.
template <typename T>
bool pge_eligible(int layout, int n);
template <typename T>
cudaError_t launch_pge(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                       cudaStream_t s, bool* used);

// The partitioned solve on contiguous systems `stride` elements apart
// (stride >= n; system j at j*stride).
template <typename T>
cudaError_t launch_pge_strided(const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                               size_t stride, cudaStream_t s, bool* used);
// Adjoint with the partitioned solve: lambda = A^{-T} xbar (written to gd)
// and ga = -lambda x_{i-1}, gb = -lambda x_i, gc = -lambda x_{i+1}, xf being
// the forward solution.  No pivot record needed.
template <typename T>
cudaError_t launch_pge_adjoint(int layout, const T* a, const T* b, const T* c, const T* xf, const T* xbar, T* ga,
                               T* gb, T* gc, T* gd, int* info, int n, int batch, cudaStream_t s, bool* used);
// Variants of the partitioned solve (1-3: one CTA with 64/128/256
// partitions, 4-6: a cluster of 2/4/8 CTAs), their largest n, the default
// variant for n (0: none) -- used by the ragged planner.
inline int pge_variant_partitions(int v) {
  return v == 1 ? 64 : v == 2 ? 128 : v == 3 || v == 4 ? 256 : v == 5 ? 512 : v == 6 ? 1024 : 0;
}
template <typename T>
int pge_default_variant(int n);
template <typename T>
int pge_variant_max_n(int v);
template <typename T>
int pge_variant_mmax(int v);
// One size bucket of a ragged batch: `count` systems list[0..count) of the
// packed arrays (system s = rows [offsets[s], offsets[s+1])), variant v, shared
// memory for m_max rows per partition; mode 0 solves, mode 1 is the adjoint
// (d = xbar, x = lambda, gradients to ga/gb/gc, xf = forward solution).
// With tk (ticket set): resident CTAs (clusters) drain the bucket.
template <typename T>
cudaError_t launch_pge_ragged(int variant, int mode, const T* a, const T* b, const T* c, const T* d, T* x,
                              const T* xf, T* ga, T* gb, T* gc, int* info, const long long* offsets, const int* list,
                              int count, int m_max, cudaStream_t s, const BucketTicket* tk = nullptr);

// periodic.cu: Sherman-Morrison pieces of the periodic solve (contiguous).
template <typename T>
cudaError_t launch_periodic_prep(const T* a, const T* b, const T* c, T* bp, T* u, int n, int batch, cudaStream_t s);
template <typename T>
cudaError_t launch_periodic_combine(const T* a, const T* b, const T* y, const T* z, T* x, int n, int batch,
                                    cudaStream_t s);

// layout.cu: a, b, c, d from one layout to another in one pass (packed:
// only src[0] / dst[0] is used).
template <typename T>
cudaError_t launch_relayout(int from, int to, const T* const src[4], T* const dst[4], int n, int batch,
                            cudaStream_t s);

// Number of systems the partitioned solve handed to its sequential fallback
// (synchronous read; optionally reset).
// Long systems (uniform contiguous batch, n beyond one chunk of 128 x 33
// rows): the partitioned pivoted solve in chunks, in place on d.  w1, w2:
// n batch elements each, piv: the pivot words of tridiag_gtsv's workspace,
// flag: batch ints.  *used = false when n is not covered.
template <typename T>
bool pge_long_eligible(int n);
// Ragged long systems in chunks of pge_long_chunk_rows() rows (see pge.cu):
// the largest n the separators' systems allow, and the passes of one size
// bucket (chunk entries cl_sys / cl_ch over the bucket's class; separator
// rows of system s at sep_off[s]; flag[s] set where a chunk fails).
int pge_long_chunk_rows();
int pge_long_retry_rows();
template <typename T>
int pge_long_ragged_max_n();
template <typename T>
cudaError_t launch_pge_long_ragged(const T* a, const T* b, const T* c, const T* d, T* x, const long long* offsets,
                                   const int* cl_sys, const int* cl_ch, int C, const long long* sep_off,
                                   size_t sep_total, T* sep, T* xsep, T* carry, int* flag, int sep_variant,
                                   int sep_m_max, const int* list, int count, const BucketTicket* tk,
                                   cudaStream_t s, int chunk_rows);
template <typename T>
cudaError_t launch_pge_long(const T* a, const T* b, const T* c, T* d, int* info, int n, int batch, T* w1, T* w2,
                            unsigned* piv, int* flag, cudaStream_t s, bool* used);
// The systems list[0 .. *dcount) (at most batch) of a uniform contiguous
// batch by the partitioned solve, drained through `ticket` (zero first).
template <typename T>
cudaError_t launch_pge_list(const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                            const int* list, const int* dcount, int* ticket, cudaStream_t s);

// ppt.cu: the partitioned pivoted solve with a thread per (system,
// partition) for contiguous batches of many systems (x may alias d); systems
// that miss its acceptance test are solved again by launch_pge_list.
// *used = false when (n, batch) is not covered or the workspace is short.
bool ppt_eligible(int layout, int n, int batch);
template <typename T>
size_t ppt_workspace_bytes(int n, int batch);
template <typename T>
cudaError_t launch_ppt(int layout, const T* a, const T* b, const T* c, const T* d, T* x, int* info, int n, int batch,
                       void* work, size_t work_bytes, cudaStream_t s, bool* used);
// out[0]: systems it accepted, out[1]: systems it listed (synchronous).
cudaError_t ppt_counts(unsigned long long* out, bool reset);

cudaError_t pge_fallback_count(unsigned long long* out, bool reset);
cudaError_t pge_path_counts(unsigned long long* out, bool reset);  // out[4]

// refine.cu: pieces of the mixed-precision refined solve (FP64 in/out).
cudaError_t launch_narrow4(const double* a, const double* b, const double* c, const double* d, float* a32,
                           float* b32, float* c32, float* d32, size_t count, cudaStream_t s);
// x_new = x_old + dx, r = d - A x_new (FP64, stored as FP32); x_old may be null (zero).
cudaError_t launch_residual(int layout, const double* a, const double* b, const double* c, const double* d,
                            const double* xold, const float* dx, double* xnew, float* r32, int n, int batch,
                            cudaStream_t s);
cudaError_t launch_update(const double* xold, const float* dx, double* xout, size_t count, cudaStream_t s);
// Ragged batches (system s = rows [offsets[s], offsets[s+1]) of `rows`
// packed rows): one warp per RAGGED_ROW_CHUNK rows of the packed arrays,
// chunk_sys[k] = the system holding row k * RAGGED_ROW_CHUNK (built with the
// plan).  FP32 copies of A (trans: of A^T) and of rhs; x_new = x_old + dx and
// r = rhs - A x_new (trans: A^T) in FP64, r stored as FP32; the adjoint's
// gradients from lambda and x.
constexpr int RAGGED_ROW_CHUNK = 2048;
struct RaggedRows {
  const long long* offsets;
  int batch;
  const int* chunk_sys;
  long long rows;
};
cudaError_t launch_ragged_narrow(bool trans, const double* a, const double* b, const double* c, const double* rhs,
                                 float* a32, float* b32, float* c32, float* r32, const RaggedRows& rr,
                                 cudaStream_t s);
cudaError_t launch_ragged_residual(bool trans, const double* a, const double* b, const double* c, const double* rhs,
                                   const double* xold, const float* dx, double* xnew, float* r32,
                                   const RaggedRows& rr, cudaStream_t s);
cudaError_t launch_ragged_gradient(const double* lam, const double* x, double* ga, double* gb, double* gc,
                                   const RaggedRows& rr, cudaStream_t s);
// restricted to the systems with kinds[s] == 0 (all when kinds is NULL), x in place
cudaError_t launch_ragged_residual_sel(bool trans, const double* a, const double* b, const double* c,
                                       const double* rhs, const double* x, float* r32, const unsigned char* kinds,
                                       const RaggedRows& rr, cudaStream_t s);
cudaError_t launch_ragged_update_sel(double* x, const float* dx, const unsigned char* kinds, const RaggedRows& rr,
                                     cudaStream_t s);
cudaError_t launch_convert_probe(const double* in, float* out, double* back, size_t count, cudaStream_t s);

// ipt.cu: Thomas for batch-interleaved systems, P partitions per system
// (top-down first, bottom-up last, spikes in between), the separators by one
// thread per system, then the back substitution; out of place.  `work` of
// ipt_workspace_bytes(); *used is false where fewer than three partitions
// would fill the GPU (the two-ended sweep is as good there) or the workspace
// is short.
template <typename T>
size_t ipt_workspace_bytes(int n, int batch);
template <typename T>
cudaError_t launch_ipt(const T* a, const T* b, const T* c, const T* d, T* x, int n, int batch, void* work,
                       size_t work_bytes, cudaStream_t s, bool* used);

// pivot record: one 32-bit word per 32 rows per system
inline size_t pivot_words(int n, int batch) { return (size_t)((n + 31) / 32) * (size_t)batch; }

}  // namespace tdg
