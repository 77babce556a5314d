/*
 * starpu_gb300_kernels.h -- C-ABI of the GB300 (sm_103a) kernel layer.
 *
 * This is the thin layer that the StarPU codelets' cuda_funcs call in place of
 * the vendor libraries.  Plain pointers and sizes only; every matrix is
 * column-major (StarPU matrix interface: nx rows contiguous, ld >= nx).
 * `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * Every entry point only enqueues work on that stream and returns; none
 * synchronises, none allocates device memory.
 *
 * Return codes: 0 = enqueued, GB300_EINVAL = bad argument (nothing enqueued),
 * GB300_ENOTSUP = unsupported option, GB300_ECUDA = a launch failed (the CUDA
 * error string is available from starpu_gb300_last_error()).
 * Numeric failure (a non-positive pivot) is not a return code: it is written
 * to the device status word *d_info (LAPACK convention: 0 = success, k > 0 =
 * the leading minor of order k is not positive definite) without trapping.
 */
#ifndef STARPU_GB300_KERNELS_H
#define STARPU_GB300_KERNELS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB300_OK 0
#define GB300_EINVAL (-22)
#define GB300_ENOTSUP (-95)
#define GB300_ENOMEM (-12)
#define GB300_ECUDA (-1000)
#define GB300_ETIMEDOUT (-110)
#define GB300_EDOM (-33)

/* Message of the last CUDA error seen by this library in the calling thread. */
const char *starpu_gb300_last_error(void);

/* ---------------- tile codelet bodies (one tile, FP32 / FP64) ------------- */

/* In-place lower Cholesky of the n x n tile A.
 * Replaces cusolverDnSpotrf(handle, LOWER, n, A, lda, work, lwork, devInfo)
 * of examples/cholesky/cholesky_kernels.c:354 (and the MAGMA / host-loop
 * fallbacks at :369 and :391-416).  No workspace is needed. d_info may be NULL. */
int starpu_gb300_spotrf_tile(void *stream, int n, float *A, int lda, int *d_info);
int starpu_gb300_dpotrf_tile(void *stream, int n, double *A, int lda, int *d_info);
/* Same, accumulating into a status word that is not reset: the first failing
 * tile's info (relative to the tile) is kept across many tiles of one run. */
int starpu_gb300_spotrf_tile_status(void *stream, int n, float *A, int lda, int *d_status);
int starpu_gb300_dpotrf_tile_status(void *stream, int n, double *A, int lda, int *d_status);

/* B[m x n] <- alpha * B * L^{-T}, L n x n lower non-unit (alpha must be 1).
 * Replaces cublasStrsm(RIGHT, LOWER, TRANS, NON_UNIT, m, n, &1, L, ldl, B, ldb)
 * of examples/cholesky/cholesky_kernels.c:258. */
int starpu_gb300_strsm_rltn_tile(void *stream, int m, int n, float alpha, const float *L, int ldl, float *B, int ldb);
int starpu_gb300_dtrsm_rltn_tile(void *stream, int m, int n, double alpha, const double *L, int ldl, double *B, int ldb);

/* C[n x n] (lower) <- alpha * A * A^T + beta * C, A n x k.
 * Replaces cublasSsyrk(LOWER, N, n, k, &-1, A, lda, &1, C, ldc) of
 * examples/cholesky/cholesky_kernels.c:177. */
int starpu_gb300_ssyrk_ln_tile(void *stream, int n, int k, float alpha, const float *A, int lda, float beta, float *C, int ldc);
int starpu_gb300_dsyrk_ln_tile(void *stream, int n, int k, double alpha, const double *A, int lda, double beta, double *C, int ldc);

/* C[m x n] <- alpha * A * B^T + beta * C, A m x k, B n x k.
 * Replaces cublasSgemm(N, T, m, n, k, &-1, A, lda, B, ldb, &1, C, ldc) of
 * examples/cholesky/cholesky_kernels.c:98. */
int starpu_gb300_sgemm_nt_tile(void *stream, int m, int n, int k, float alpha, const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc);
int starpu_gb300_dgemm_nt_tile(void *stream, int m, int n, int k, double alpha, const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);

/* ---------------- LU tile codelet bodies (examples/lu, FP32 / FP64) -------
 * The reference LU keeps the pivot in L: A = L U with L lower non-unit and U
 * unit upper (examples/lu/xlu_kernels.c:369-380). */

/* In-place LU of the n x n tile A, no pivoting.  Replaces the GETRF codelet
 * (cusolverDnSgetrf, or the host loop of cublasSscal / cublasSger with one
 * synchronisation per column, examples/lu/xlu_kernels.c:385-433).  A zero
 * pivot writes info = k + 1 to *d_info (may be NULL) without trapping. */
int starpu_gb300_sgetrf_tile(void *stream, int n, float *A, int lda, int *d_info);
int starpu_gb300_dgetrf_tile(void *stream, int n, double *A, int lda, int *d_info);

/* The GETRF_PIVOT codelet (xlu_kernels.c:491-657): as above, except that a
 * step whose pivot has magnitude below `threshold` takes the largest entry of
 * its row (first on ties) and swaps those two whole columns.  d_ipiv (device,
 * n ints) receives, per step, the column swapped in (the step itself when it
 * pivoted in place) or -1 when the step did not pivot.  `work` (device,
 * >= _workspace(n) bytes) holds a copy of the tile: the blocked factorisation
 * runs first and, if a step needed a pivot, the tile is restored and factored
 * again with pivoting. */
size_t starpu_gb300_sgetrf_pivot_tile_workspace(int n);
size_t starpu_gb300_dgetrf_pivot_tile_workspace(int n);
int starpu_gb300_sgetrf_pivot_tile(void *stream, int n, float *A, int lda, float threshold, int *d_ipiv, void *work,
                                   size_t lwork, int *d_info);
int starpu_gb300_dgetrf_pivot_tile(void *stream, int n, double *A, int lda, double threshold, int *d_ipiv, void *work,
                                   size_t lwork, int *d_info);

/* B[m x n] <- L^{-1} B, L m x m lower non-unit.  Replaces cublasStrsm(LEFT,
 * LOWER, N, NON_UNIT) of the TRSM_LL codelet, xlu_kernels.c:192-199. */
int starpu_gb300_strsm_llnn_tile(void *stream, int m, int n, const float *L, int ldl, float *B, int ldb);
int starpu_gb300_dtrsm_llnn_tile(void *stream, int m, int n, const double *L, int ldl, double *B, int ldb);

/* B[m x n] <- B U^{-1}, U n x n unit upper.  Replaces cublasStrsm(RIGHT,
 * UPPER, N, UNIT) of the TRSM_RU codelet, xlu_kernels.c:281-289. */
int starpu_gb300_strsm_runu_tile(void *stream, int m, int n, const float *U, int ldu, float *B, int ldb);
int starpu_gb300_dtrsm_runu_tile(void *stream, int m, int n, const double *U, int ldu, double *B, int ldb);

/* C[m x n] <- alpha * A * B + beta * C, A m x k, B k x n.  Replaces
 * cublasSgemm(N, N) of the LU GEMM codelet, xlu_kernels.c:74-78. */
int starpu_gb300_sgemm_nn_tile(void *stream, int m, int n, int k, float alpha, const float *A, int lda, const float *B,
                               int ldb, float beta, float *C, int ldc);
int starpu_gb300_dgemm_nn_tile(void *stream, int m, int n, int k, double alpha, const double *A, int lda,
                               const double *B, int ldb, double beta, double *C, int ldc);

/* Swap columns pairs[2s] and pairs[2s+1] of the m x n tile A, for s = 0 ..
 * npairs-1 in that order (pairs is a HOST array; an index outside [0, n) is
 * GB300_EINVAL).  Replaces the cublasSswap loop of the PIVOT codelet,
 * xlu_kernels.c:696-708. */
int starpu_gb300_sswap_columns_tile(void *stream, int m, int n, float *A, int lda, const int *pairs, int npairs);
int starpu_gb300_dswap_columns_tile(void *stream, int m, int n, double *A, int lda, const int *pairs, int npairs);

/* ---------------- whole matrix, plain precision --------------------------- */

/* Tiled right-looking Cholesky of the whole n x n matrix with tile nb (0 =
 * 512): the DAG of examples/cholesky/cholesky_implicit.c:244-318 (POTRF k,
 * TRSM m>k, SYRK/GEMM) with the tasks of one step fused into whole-panel
 * launches.  Only the lower triangle is read and written. */
int starpu_gb300_spotrf(void *stream, int n, float *A, int lda, int nb, int *d_info);
int starpu_gb300_dpotrf(void *stream, int n, double *A, int lda, int nb, int *d_info);

/* Solve A X = B with the lower factor L from *potrf (LAPACK xPOTRS, uplo=L,
 * min-dgels/base/SRC/dpotrs.c), B n x nrhs overwritten by X. */
int starpu_gb300_spotrs(void *stream, int n, int nrhs, const float *L, int ldl, float *B, int ldb);
int starpu_gb300_dpotrs(void *stream, int n, int nrhs, const double *L, int ldl, double *B, int ldb);

/* Same solve as starpu_gb300_spotrs, as two single-launch sweeps (one per
 * triangle and group of 16 right-hand sides) over 64-row blocks whose
 * diagonal blocks are inverted first.  `work` (device, >= _workspace(n)
 * bytes) holds the inverted blocks and the sweeps' completion flags; d_err
 * is set non-zero if an internal wait timed out (the result is then invalid).
 * Same LAPACK xPOTRS contract (min-dgels/base/SRC/dpotrs.c, uplo = L). */
size_t starpu_gb300_spotrs_sweep_workspace(int n);
int starpu_gb300_spotrs_sweep(void *stream, int n, int nrhs, const float *L, int ldl, float *B, int ldb, void *work,
                              size_t lwork, int *d_err);

/* Same LAPACK xPOTRS contract (min-dgels/base/SRC/dpotrs.c, uplo = L) when
 * the factorisation kept the inverses of its nb x nb diagonal tiles: two
 * single-launch sweeps per group of 16 right-hand sides over 32-row slabs,
 * n / nb dependent steps each.  Tile T's inverse (lower triangular, zero
 * above the diagonal) is at Dinv + T * ldd * ldd with leading dimension
 * ldd >= nb; nb a multiple of 32, at most 1024.  `work` (device, >=
 * _workspace(n, nb) bytes) holds the sweeps' scratch and counters; d_err is
 * set non-zero if an internal wait timed out (the result is then invalid). */
size_t starpu_gb300_spotrs_inv_tiles_workspace(int n, int nb);
int starpu_gb300_spotrs_inv_tiles(void *stream, int n, int nrhs, int nb, const float *L, int ldl, const float *Dinv,
                                  int ldd, float *B, int ldb, void *work, size_t lwork, int *d_err);

/* Allocation-free variant of starpu_gb300_spotrs_sweep.  It has no
 * counterpart in the reference.  For callers that must not allocate device
 * memory -- a codelet body running inside a runtime that owns all device
 * buffers, a serving or real-time loop -- it takes no workspace: its scratch
 * is one static device array sized for n <= STARPU_GB300_NOALLOC_MAX_N (about
 * 4 MiB, held by every GPU that loads the library until the process exits).
 * Larger n is rejected with GB300_EINVAL.  It calls no allocator.  The first
 * call on a device (with it current) looks the array's address up once; make
 * it before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race and must be serialised by the caller.  d_err, when given, is
 * used as starpu_gb300_spotrs_sweep uses it (set non-zero on a timeout, never
 * cleared by the call: zero it before the first call).  d_err may be NULL:
 * the call then waits for its stream and returns GB300_ETIMEDOUT if an
 * internal wait timed out (B is then invalid). */
#define STARPU_GB300_NOALLOC_MAX_N 16384
int starpu_gb300_spotrs_noalloc(void *stream, int n, int nrhs, const float *L, int ldl, float *B, int ldb,
                                int *d_err);

/* Limit of every bounded wait of the sweeps (starpu_gb300_spotrs_sweep,
 * _noalloc, _inv_tiles and the mixed solve's correction solves) on a flag
 * that another CTA of the same launch publishes; a wait that runs out sets
 * the call's error word and the launch still ends.  Default 2 s; 0 restores
 * it.  Returns the previous limit.  The tensor-core kernels' pipeline waits
 * keep their own fixed limit.  No counterpart in the reference (its CUDA
 * path has no device-side waits). */
unsigned long long starpu_gb300_set_wait_budget_ns(unsigned long long ns);

/* Host-only self-check of the per-device bookkeeping of kernel attributes
 * (dynamic shared memory limits are set once per function and device).
 * Needs no GPU; returns 0 on success, else the number of the failing step. */
int starpu_gb300_selftest_attr_book(void);

/* Host-only self-check of the tile sweeps' task order (starpu_gb300_spotrs_inv_tiles
 * and the mixed solve's correction solves) for ntiles tile rows of spt slabs:
 * every ticket maps to one task and every dependency has a smaller ticket.
 * Needs no GPU; returns 0 on success. */
int starpu_gb300_selftest_sweep_tickets(int ntiles, int spt);

/* ---------------- tensor-core trailing update (tcgen05, sm_103a) ---------- */

/* P (m x k FP32, column-major, ldp) -> hi = bf16(P), lo = bf16(P - hi), both
 * stored K-major (row i = P[i, 0..k), row stride ldk elements, ldk % 8 == 0,
 * 16-byte aligned).  lo may be NULL.  Columns k..ldk-1 are written as 0. */
int starpu_gb300_split_bf16(void *stream, int m, int k, const float *P, int ldp, void *hi, void *lo, int ldk);

/* C[m x n] (FP32, column-major) -= A B^T on the tensor cores, A = m x k and
 * B = n x k BF16 K-major (the layout starpu_gb300_split_bf16 writes).
 * nterms = 1: A_hi B_hi^T.  nterms = 3: A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T
 * (split-BF16, ~2^-16 relative).  lower = 1 (requires m == n): only elements
 * with row >= col are written (the SYRK form).  This is the fused GEMM/SYRK
 * trailing update that replaces cublasSgemm(N,T) / cublasSsyrk(L,N) of
 * examples/cholesky/cholesky_kernels.c:98,177 for every tile of one step.
 * d_err: device status word, set non-zero if an internal wait timed out. */
int starpu_gb300_tc_update(void *stream, int m, int n, int k, const void *a_hi, const void *a_lo, int lda,
                           const void *b_hi, const void *b_lo, int ldb, int nterms, int lower, float *C, int ldc,
                           int *d_err);

/* The FP32 tile update on the tensor cores, for the codelets of the tiled
 * Cholesky: C[m x n] -= A B^T (A m x k, B n x k, FP32, column-major).  Each
 * operand row is scaled by a power of two and split as h + l in FP16 (about
 * 22 significant bits) in `work`; the three products h h + h l + l h
 * accumulate in FP32 on the tensor cores.  lower = 1 (m == n) writes only
 * row >= col: the SYRK form, and B == A (same pointer and ld) splits once.
 * Replaces cublasSgemm(N, T, -1, +1) of examples/cholesky/cholesky_kernels.c:98
 * and cublasSsyrk(L, N, -1, +1) of :177 for FP32 tiles.  `work`: device,
 * >= starpu_gb300_tile_tc_workspace(max(m, n, k)) bytes.  d_err: device status
 * word, set non-zero if an internal wait timed out.  _prepare sets the
 * kernel's shared-memory limit on the current device (call it once before a
 * stream capture that records these updates). */
size_t starpu_gb300_tile_tc_workspace(int nmax);
int starpu_gb300_tile_tc_prepare(void);
int starpu_gb300_sgemm_nt_tile_tc(void *stream, int m, int n, int k, const float *A, int lda, const float *B,
                                  int ldb, float *C, int ldc, int lower, void *work, size_t lwork, int *d_err);

/* Bytes of split-panel workspace starpu_gb300_spotrf_tc needs. */
size_t starpu_gb300_spotrf_tc_workspace(int n, int nb);

/* Tiled Cholesky of an FP32 matrix (tile nb): FP32 POTRF of the diagonal
 * tile (CUDA cores), its explicit inverse, the panel TRSM as one split
 * tensor-core product P * L_kk^-T, and the trailing update on the tensor
 * cores with the panel split per row to FP16 h + l scaled by a power of two
 * (nterms 3, ~22 bits; nterms 1: plain BF16 operands). */
int starpu_gb300_spotrf_tc(void *stream, int n, float *A, int lda, int nb, int nterms, void *work, size_t lwork,
                           int *d_info, int *d_err);

/* ---------------- device memory helpers for hosts without a CUDA binding -- */

void *starpu_gb300_device_malloc(size_t bytes);
int starpu_gb300_device_free(void *p);
void *starpu_gb300_host_malloc_pinned(size_t bytes);
int starpu_gb300_host_free_pinned(void *p);
int starpu_gb300_memcpy_h2d(void *stream, void *dst, const void *src, size_t bytes);
int starpu_gb300_memcpy_d2h(void *stream, void *dst, const void *src, size_t bytes);
int starpu_gb300_memset(void *stream, void *dst, int value, size_t bytes);
int starpu_gb300_stream_sync(void *stream);
void *starpu_gb300_stream_create(void);
int starpu_gb300_stream_destroy(void *stream);
int starpu_gb300_device_count(void);

/* CUDA events (timing on a stream from hosts without a CUDA binding). */
void *starpu_gb300_event_create(void);
int starpu_gb300_event_record(void *event, void *stream);
double starpu_gb300_event_elapsed_ms(void *start, void *end); /* waits for `end` */
int starpu_gb300_event_destroy(void *event);

/* ---------------- measurement --------------------------------------------
 * Number of kernels this library has launched since it was loaded. */
unsigned long long starpu_gb300_launch_count(void);

/* Per-kernel-class profiling, the counterpart of StarPU's per-task profiling
 * information (STARPU_PROFILING, src/profiling/profiling.c): when enabled,
 * each launch of a profiled class is bracketed by CUDA events on its own
 * stream and its algorithmic flops / bytes are recorded.  Classes:
 * 0 = tensor-core trailing update, 1 = panel (POTRF + TRSM + split),
 * 2 = refinement residual, 3 = triangular solves, 4 = batched solves,
 * 5 = host<->device transfers of the solver context (bytes = bytes moved).
 * _get resolves pending events. */
void starpu_gb300_profiling_enable(int on);
void starpu_gb300_profiling_reset(void);
int starpu_gb300_profiling_get(int kind, unsigned long long *launches, double *total_ms, double *flops, double *bytes);
/* The time-weighted mean fraction of the SMs a class's launches were limited
 * to (1 unless a launch shared the GPU by design: the trailing updates that
 * run beside the next panel leave that panel's SMs free). */
int starpu_gb300_profiling_sm_share(int kind, double *share);
/* Per-launch start and end times (ms, relative to the first profiled launch
 * after a reset; events on each launch's own stream, so overlapping launches
 * show as overlapping spans), the counterpart of the start / end times of
 * StarPU's per-task profiling information.  Fills up to `max` entries in
 * profiling order and returns how many are recorded (at most 65536). */
int starpu_gb300_profiling_timeline(int max, int *kinds, double *start_ms, double *end_ms);

#ifdef __cplusplus
}
#endif

#endif /* STARPU_GB300_KERNELS_H */
