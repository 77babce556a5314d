/*
 * starpu_gb300_solver.h -- SPD solve entry points of the GB300 kernel layer.
 *
 * The reference has no solve, no mixed precision, no batching and no serving
 * (its Cholesky is FP32 factorisation only: examples/cholesky/cholesky_kernels.c:53-55);
 * these entry points extend the factorisation of starpu_gb300_kernels.h to
 * A X = B for SPD A with LAPACK dposv / dsposv semantics.  Same conventions
 * as starpu_gb300_kernels.h: column-major, void* stream, no synchronisation,
 * no device allocation (work buffers are passed in).
 */
#ifndef STARPU_GB300_SOLVER_H
#define STARPU_GB300_SOLVER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- synthetic inputs (benchmarks and tests) ----------------
 * Row i of B ~ N(0,1) from PCG64 stream i+1 of `seed` (Box-Muller pairs);
 * right-hand-side column j ~ U[-1,1] from PCG64 stream 2^40+j.
 * gen_spd_gram: A = B B^T / n + alpha I (full symmetric), `work` n*n doubles. */
int starpu_gb300_gen_normal(void *stream, int rows, int cols, uint64_t seed, double *B, int ldb);
int starpu_gb300_gen_uniform_rhs(void *stream, int n, int nrhs, uint64_t seed, double *B, int ldb);
int starpu_gb300_gen_spd_gram(void *stream, int n, uint64_t seed, double alpha, double *A, int lda, double *work);
/* A_ii += delta (re-targets the conditioning of B B^T / n + alpha I). */
int starpu_gb300_shift_diagonal(void *stream, int n, double *A, int lda, double delta);
/* cudaSetDevice for hosts without a CUDA binding (one process per GPU). */
int starpu_gb300_set_device(int device);
int starpu_gb300_memcpy_d2d(void *stream, void *dst, const void *src, size_t bytes);

/* ---------------- mixed precision + FP64 iterative refinement ------------ */

/* Outcome of one starpu_gb300_dsposv call. */
typedef struct starpu_gb300_ir_info {
    int status;            /* 0 converged; GB300_EDOM factor failed; GB300_ETIMEDOUT not converged */
    int iterations;        /* refinement corrections applied (each: one solve with the factor) */
    int factor_terms;      /* products per trailing-update term (1: BF16; 3: split operands) */
    int potrf_info;        /* LAPACK-style info of the last factorisation (mixed, or FP64 after a fallback) */
    double backward_error; /* max over RHS of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) */
    double anorm;          /* ||A||_inf */
    int method;            /* refinement at the end: 0 classic corrections, 1 preconditioned conjugate gradients */
    int fallback;          /* LAPACK dsposv ITER < 0: 0 none; 1 the mixed factorisation failed (ITER -3);
                              2 its refinement did not converge (ITER -31); then the FP64 factorisation on the
                              GPU solved the system and status/backward_error describe that solve */
} starpu_gb300_ir_info;

/* Refinement policy of starpu_gb300_dsposv (process-wide; returns the
 * previous value, a negative argument only queries):
 *   mode 0 classic corrections only, 1 preconditioned conjugate gradients
 *   from the first correction, 2 (default; STARPU_GB300_REFINE=ir|pcg sets
 *   0|1) classic corrections, switching to conjugate gradients when one
 *   leaves more than 5 % of the backward error;
 *   on 1 (default; STARPU_GB300_FP64_FALLBACK=0 sets 0) LAPACK's FP64
 *   fallback after a failed factorisation or a refinement that stalls. */
int starpu_gb300_dsposv_set_refinement(int mode);
int starpu_gb300_dsposv_set_fp64_fallback(int on);

/* Bytes of device workspace starpu_gb300_dsposv needs (tile nb, 0 = 1024). */
size_t starpu_gb300_dsposv_workspace(int n, int nrhs, int nb);

/* Solve A X = B (A SPD, FP64; only the lower triangle of A is read, LAPACK
 * dsposv with uplo = 'L') with an FP32-storage tiled Cholesky whose panel
 * TRSM and trailing updates run on the tensor cores (row-scaled FP16 split
 * operands, nterms = 3, or plain BF16, nterms = 1), then iterative
 * refinement: r = b - A x to ~2^-55 of ||A|| ||x|| (exact digit products on
 * the tensor cores, FP64 sums), correction solved with the low-precision
 * factor, x += d in FP64, until every column's normwise backward error <= tol
 * or max_iter corrections were applied.  When a correction contracts the
 * error slowly (kappa(A) near 1e6 and above) the refinement continues as
 * preconditioned conjugate gradients with the same factor.  As LAPACK
 * dsposv, a failed low-precision factorisation or a refinement that does
 * not converge falls back to the FP64 factorisation and solve on the GPU
 * (info->fallback; STARPU_GB300_FP64_FALLBACK=0 disables it).  X is output
 * only.  Synchronises the stream once per refinement step to read the error.
 * Returns 0, GB300_EDOM (not positive definite) or GB300_ETIMEDOUT (no
 * convergence, or a bounded wait ran out); *info (may be NULL) gets the
 * details. */
int starpu_gb300_dsposv(void *stream, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                        int ldx, int nb, int nterms, double tol, int max_iter, void *work, size_t lwork,
                        starpu_gb300_ir_info *info);

/* Persistent solver context: owns a stream and device buffers for systems up
 * to n_max x n_max with up to nrhs_max right-hand sides, so that repeated
 * solves allocate nothing.  _dsposv_host takes HOST buffers (pinned for full
 * copy bandwidth), copies the lower triangle of A (the only part the solve
 * reads) and B in, solves as starpu_gb300_dsposv, copies X out and
 * synchronises. */
typedef struct starpu_gb300_solver starpu_gb300_solver;
starpu_gb300_solver *starpu_gb300_solver_create(int n_max, int nrhs_max, int nb, int nterms);
int starpu_gb300_solver_destroy(starpu_gb300_solver *solver);
void *starpu_gb300_solver_stream(starpu_gb300_solver *solver);
/* Pinned-input path of _dsposv_host: 1 gathers A superblock by superblock
 * while the factorisation starts on the first columns (bit-identical
 * result, more device memory: every step's split panel is kept), 0 gathers
 * the whole matrix first; -1 (the default) follows
 * STARPU_GB300_HOST_OVERLAP=1 (otherwise off).  Returns the previous
 * setting. */
int starpu_gb300_solver_host_overlap(starpu_gb300_solver *solver, int on);
int starpu_gb300_solver_dsposv_host(starpu_gb300_solver *solver, int n, int nrhs, const double *A, int lda,
                                    const double *B, int ldb, double *X, int ldx, double tol, int max_iter,
                                    starpu_gb300_ir_info *info);

/* Normwise backward error of X for A X = B, per column, computed on the
 * device in FP64 (||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf));
 * synchronises and writes nrhs values to berr_host. */
size_t starpu_gb300_backward_error_workspace(int n, int nrhs);
int starpu_gb300_backward_error(void *stream, int n, int nrhs, const double *A, int lda, const double *X, int ldx,
                                const double *B, int ldb, void *work, size_t lwork, double *berr_host);

/* ---------------- batched: many independent systems, one persistent launch
 * System i: order n[i] (1..1024), A_i FP64 column-major (ld n[i]) at
 * A + a_off[i], B_i and X_i (n[i] x nrhs, ld n[i]) at B / X + b_off[i]
 * (offsets in elements; n, a_off, b_off are HOST arrays).  Each system is
 * factored in FP32 (blocked, block size from the tuning table) and refined in
 * FP64 until its backward error <= tol or max_iter corrections.  nrhs <= 8.
 * Synchronous: on return status[i] (host, may be NULL) holds the number of
 * corrections (>= 0), -k if the FP32 factor met a non-positive pivot k, or
 * -1000 if it did not converge; berr[i] (host, may be NULL) the final error. */
size_t starpu_gb300_dposv_batched_workspace(int nsys, const int *n, int nrhs);
int starpu_gb300_dposv_batched(void *stream, int nsys, const int *n, const double *A, const long long *a_off,
                               const double *B, const long long *b_off, double *X, int nrhs, double tol,
                               int max_iter, void *work, size_t lwork, int *status, double *berr);

/* Autotuner of the batched solve: times every candidate block size (16, 32,
 * 64) on a batch of each size bucket (n <= 32, 64, ..., 1024), keeps the
 * fastest and stores the table next to the history perfmodels
 * (<perfmodel dir>/codelets/45/gb300_chol_tuning.<hostname>); later calls in
 * any process load it.  systems_per_bucket / reps <= 0 pick defaults. */
int starpu_gb300_batched_autotune(int systems_per_bucket, int reps);
/* Current block size per bucket (6 buckets); returns the bucket count. */
int starpu_gb300_batched_get_tuning(signed char *nb_per_bucket, int nbuckets);

/* Autotunes the schedule of the mixed solve's tensor-core factorisation for
 * tile nb (64..1024) at order n (>= 3 nb) on the current device: times the
 * diagonal-tile kernel on a quarter of the SMs, the trailing update on the
 * whole GPU and the panel solve on the quarter, then whole factorisations of
 * an n x n matrix with the lookahead split of the per-step model on those
 * times, and with a quarter, a third, half of the SMs and no lookahead; the
 * fastest choice and the measured times are stored in the same table
 * (gb300_chol_tuning.<host>, beside the perfmodels) and every later
 * factorisation with tile nb uses them (GB300_LOOKAHEAD_SMS still overrides).
 * Allocates its own buffers.  StarPU's counterpart is the calibration of the
 * history perfmodels (src/core/perfmodel/perfmodel.c:663-713). */
int starpu_gb300_dense_autotune(int n, int nb, int reps);
/* The stored schedule for tile nb: lookahead SMs (-1: the per-step model),
 * diagonal-tile time, update rate, panel-solve rate relative to it, and the
 * tuning factorisation's time.  Returns 1 when a tuning exists, else 0. */
int starpu_gb300_dense_get_tuning(int nb, int *lookahead_sms, double *t_diag_us, double *update_tflops,
                                  double *panel_rate, double *step_ms);

/* ---------------- serving: a request loop with continuous batching --------
 * A server owns `executors` worker threads, each with its own CUDA stream and
 * buffers for systems up to max_n x max_n with max_nrhs right-hand sides.
 * Submitted requests wait in an admission queue; whenever an executor is free
 * it takes either every queued request with n <= 1024 (up to 512) as one
 * batched persistent launch, or the oldest larger request, so requests that
 * arrive while others run are admitted as executors and memory free up and
 * their work overlaps on the device.  Factors of requests with a non-zero
 * matrix_id stay on the device (FP64 A + FP32 factor, LRU) for later
 * requests with the same id (repeat right-hand sides: no refactorisation).
 * Device memory (executor buffers + cached factors) stays within
 * hbm_budget_bytes; a request that cannot be cached is still served.
 * mode 0: mixed precision + refinement (the path above); mode 1: the plain
 * baseline -- every request alone, FP64 dposv, one at a time; mode 2: every
 * request alone as one mixed solve (factor + refinement, no batched launch,
 * no factor cache), which isolates what batching and overlap add. 
 * A, B may be host or device pointers; X is written where it points. */
typedef struct starpu_gb300_request {
    int n, nrhs;
    const double *A;        /* n x n, ld n (read only when the factor is not cached) */
    const double *B;        /* n x nrhs, ld n */
    double *X;              /* n x nrhs, ld n (output) */
    uint64_t matrix_id;     /* 0: do not cache the factor */
    double tol;             /* backward error target (<= 0: 1e-12) */
    int max_iter;           /* refinement steps allowed (<= 0: 30) */
    /* filled by the server */
    int status;             /* 0 ok, GB300_EDOM, GB300_ETIMEDOUT, GB300_EINVAL, ... */
    int iterations;
    int cache_hit;          /* 1 when a cached factor was reused */
    int batched;            /* 1 when served inside a batched launch */
    double backward_error;
    double submit_us, start_us, end_us;  /* starpu_timing_now() clock */
    int done;
    int reserved;
} starpu_gb300_request;

typedef struct starpu_gb300_server starpu_gb300_server;
starpu_gb300_server *starpu_gb300_server_create(size_t hbm_budget_bytes, int executors, int max_n, int max_nrhs,
                                                int mode);
/* Queue a request (the struct must stay valid until it is done).  0 or GB300_EINVAL. */
int starpu_gb300_server_submit(starpu_gb300_server *server, starpu_gb300_request *req);
/* Block until req is done; returns req->status (GB300_EINVAL for a NULL server
 * or a request that was not queued). */
int starpu_gb300_server_wait(starpu_gb300_server *server, starpu_gb300_request *req);
/* Block until every submitted request is done. */
int starpu_gb300_server_drain(starpu_gb300_server *server);
/* Counters: served, batched launches, cache hits, evictions, bytes in use (may be NULL). */
int starpu_gb300_server_stats(starpu_gb300_server *server, unsigned long long *served, unsigned long long *batches,
                              unsigned long long *cache_hits, unsigned long long *evictions, size_t *bytes_in_use);
int starpu_gb300_server_destroy(starpu_gb300_server *server);

/* R = B - A X for symmetric A (n x n, only the lower triangle is read), X, B,
 * R n x nrhs, all FP64, to ~2^-56 of ||A||_inf ||X||_inf: the refinement
 * residual of starpu_gb300_dsposv.  The products run on the tensor cores as
 * exact integer products of 7-bit slices of A and X (fixed point with a power-
 * of-two scale per matrix and per column).  Deterministic.  `work` (device,
 * >= _workspace bytes); d_err is set non-zero if an internal wait timed out. */
size_t starpu_gb300_dsyresidual_workspace(int n, int nrhs);
int starpu_gb300_dsyresidual(void *stream, int n, int nrhs, const double *A, int lda, const double *X, int ldx,
                             const double *B, int ldb, double *R, int ldr, void *work, size_t lwork, int *d_err);

/* Plain FP64 solve: dpotrf (tile nb) + dpotrs, A and B overwritten (LAPACK dposv). */
int starpu_gb300_dposv(void *stream, int n, int nrhs, double *A, int lda, double *B, int ldb, int nb, int *d_info);

#ifdef __cplusplus
}
#endif

#endif /* STARPU_GB300_SOLVER_H */
