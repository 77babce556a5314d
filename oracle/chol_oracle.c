/*
 * ORACLE -- test infrastructure only.  CPU restatement of the reference's
 * tiled Cholesky path, used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py as the checker.  Never linked into, called by
 * or shipped with the product library.
 *
 * Everything is plain C (no BLAS) so that it builds anywhere with gcc, and
 * each routine cites the reference code it restates:
 *   - input matrix of the reference driver: examples/cholesky/cholesky_implicit.c:477-484
 *   - tile loop (POTRF k, TRSM m>k, SYRK n>k, GEMM m>n>k): cholesky_implicit.c:244-318
 *   - tile partitioning (block filters, ragged remainder first):
 *       src/datawizard/interfaces/matrix_filters.c:22-104, src/datawizard/filters.c:1655-1679
 *   - per-tile arithmetic of the CPU codelets: cholesky_kernels.c:75 (SGEMM N,T),
 *       :169 (SSYRK L,N), :254 (STRSM R,L,T,N), :329-342 (unblocked POTRF loop)
 *   - reconstruction check: cholesky_implicit.c:530-585 (relative error <= 1e-4)
 *   - FLOP model: examples/cholesky/cholesky.h:95-119
 *   - POTRS (two triangular sweeps): min-dgels/base/SRC/dpotrs.c
 * The FP64 / solve / refinement routines have no reference implementation;
 * they restate LAPACK semantics (dpotrf/dpotrs) in FP64 and are pinned
 * against the CLAPACK sources shipped in min-dgels (built into oracle/_ref).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define IDX(i, j, ld) ((size_t)(i) + (size_t)(j) * (size_t)(ld))

/* ---------------------------------------------------------------- inputs */

/* A_mn = 1/(1+m+n) + size*delta_mn in FP32 (cholesky_implicit.c:481). */
void oracle_hilbert_f32(int n, float *A, int lda)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
            A[IDX(i, j, lda)] = (1.0f / (1.0f + i + j)) + ((i == j) ? 1.0f * n : 0.0f);
}

/* PCG64, XSL-RR 128/64 output (O'Neill 2014): state advances by a 128-bit
 * LCG, output = rotr64(hi ^ lo, hi >> 58).  Stream s uses increment 2s+1. */
typedef struct { unsigned __int128 state, inc; } pcg64_t;

static const unsigned __int128 PCG_MULT =
    ((unsigned __int128)0x2360ED051FC65DA4ULL << 64) | (unsigned __int128)0x4385DF649FCCF645ULL;

static inline uint64_t pcg64_next(pcg64_t *r)
{
    r->state = r->state * PCG_MULT + r->inc;
    uint64_t hi = (uint64_t)(r->state >> 64), lo = (uint64_t)r->state;
    uint64_t x = hi ^ lo;
    unsigned rot = (unsigned)(hi >> 58);
    return (x >> rot) | (x << ((64 - rot) & 63));
}

static inline void pcg64_seed(pcg64_t *r, uint64_t seed, uint64_t stream)
{
    r->inc = ((unsigned __int128)stream << 1) | 1u;
    r->state = 0;
    pcg64_next(r);
    r->state += ((unsigned __int128)seed << 64) | (unsigned __int128)(seed ^ 0x9E3779B97F4A7C15ULL);
    pcg64_next(r);
}

/* uniform in (0, 1]: 53 random bits */
static inline double u01_open0(uint64_t x) { return ((double)(x >> 11) + 1.0) * (1.0 / 9007199254740992.0); }
/* uniform in [0, 1) */
static inline double u01(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

/* Row i of the N(0,1) matrix B comes from PCG64 stream (i + 1) of `seed`:
 * pairs of draws (u1, u2) give, by Box-Muller, z0 = r cos(2 pi u2) for an
 * even column and z1 = r sin(2 pi u2) for the next odd column. */
/* Rows row0 .. row0 + rows - 1 of the matrix below, stored from B (row row0
 * at B[0]): independent row streams, so callers may fill row ranges in
 * parallel. */
void oracle_normal_rows(int row0, int rows, int cols, uint64_t seed, double *B, int ldb)
{
    const double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < rows; i++) {
        pcg64_t r;
        pcg64_seed(&r, seed, (uint64_t)(row0 + i) + 1);
        for (int j = 0; j < cols; j += 2) {
            double u1 = u01_open0(pcg64_next(&r));
            double u2 = u01(pcg64_next(&r));
            double rad = sqrt(-2.0 * log(u1));
            double th = two_pi * u2;
            B[IDX(i, j, ldb)] = rad * cos(th);
            if (j + 1 < cols) B[IDX(i, j + 1, ldb)] = rad * sin(th);
        }
    }
}

void oracle_normal_matrix(int rows, int cols, uint64_t seed, double *B, int ldb)
{
    const double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < rows; i++) {
        pcg64_t r;
        pcg64_seed(&r, seed, (uint64_t)i + 1);
        for (int j = 0; j < cols; j += 2) {
            double u1 = u01_open0(pcg64_next(&r));
            double u2 = u01(pcg64_next(&r));
            double rad = sqrt(-2.0 * log(u1));
            double th = two_pi * u2;
            B[IDX(i, j, ldb)] = rad * cos(th);
            if (j + 1 < cols) B[IDX(i, j + 1, ldb)] = rad * sin(th);
        }
    }
}

/* Right-hand sides iid U[-1,1]: column j from PCG64 stream (2^40 + j). */
void oracle_uniform_rhs(int n, int nrhs, uint64_t seed, double *B, int ldb)
{
    for (int j = 0; j < nrhs; j++) {
        pcg64_t r;
        pcg64_seed(&r, seed, ((uint64_t)1 << 40) + (uint64_t)j);
        for (int i = 0; i < n; i++) B[IDX(i, j, ldb)] = 2.0 * u01(pcg64_next(&r)) - 1.0;
    }
}

/* A = B B^T / n + alpha I with B n x n iid N(0,1) (both triangles written).
 * Each entry is one dot product accumulated in increasing index order. */
void oracle_spd_gram(int n, uint64_t seed, double alpha, double *A, int lda)
{
    double *B = (double *)malloc((size_t)n * n * sizeof(double));
    double *Bt = (double *)malloc((size_t)n * n * sizeof(double));
    oracle_normal_matrix(n, n, seed, B, n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) Bt[IDX(j, i, n)] = B[IDX(i, j, n)]; /* row i of B contiguous */
    const double inv_n = 1.0 / (double)n;
    for (int j = 0; j < n; j++) {
        const double *bj = Bt + (size_t)j * n;
        for (int i = j; i < n; i++) {
            const double *bi = Bt + (size_t)i * n;
            double s = 0.0;
            for (int p = 0; p < n; p++) s = fma(bi[p], bj[p], s);
            double v = s * inv_n + ((i == j) ? alpha : 0.0);
            A[IDX(i, j, lda)] = v;
            A[IDX(j, i, lda)] = v;
        }
    }
    free(B);
    free(Bt);
}

/* --------------------------------------------------------- tile kernels */

/* size/offset of chunk `id` of `n` split in `parts` (remainder goes to the
 * first chunks): src/datawizard/filters.c:1655-1679 */
void oracle_chunk(int n, int parts, int id, int *size, int *offset)
{
    int base = n / parts, rem = n % parts;
    *size = base + (id < rem ? 1 : 0);
    *offset = id * base + (id < rem ? id : rem);
}

#define DEFINE_TILE_KERNELS(T, SFX, SQRT)                                                          \
    /* unblocked lower POTRF: cholesky_kernels.c:329-342 (sqrt, SSCAL by 1/lambda, SSYR L) */        \
    static int potrf_tile_##SFX(int n, T *A, int lda)                                               \
    {                                                                                              \
        for (int z = 0; z < n; z++) {                                                              \
            T d = A[IDX(z, z, lda)];                                                               \
            if (!(d > (T)0)) return z + 1;                                                         \
            T lambda = SQRT(d);                                                                    \
            A[IDX(z, z, lda)] = lambda;                                                            \
            T inv = (T)1 / lambda;                                                                 \
            for (int i = z + 1; i < n; i++) A[IDX(i, z, lda)] *= inv;                              \
            for (int c = z + 1; c < n; c++) {                                                      \
                T t = -A[IDX(c, z, lda)];                                                          \
                for (int i = c; i < n; i++) A[IDX(i, c, lda)] += A[IDX(i, z, lda)] * t;            \
            }                                                                                      \
        }                                                                                          \
        return 0;                                                                                  \
    }                                                                                              \
    /* B[m x n] <- B L^{-T}: STRSM(R,L,T,N), reference-BLAS column order (cholesky_kernels.c:254) */ \
    static void trsm_tile_##SFX(int m, int n, const T *L, int ldl, T *B, int ldb)                   \
    {                                                                                              \
        for (int k = 0; k < n; k++) {                                                              \
            T inv = (T)1 / L[IDX(k, k, ldl)];                                                      \
            for (int i = 0; i < m; i++) B[IDX(i, k, ldb)] *= inv;                                  \
            for (int j = k + 1; j < n; j++) {                                                      \
                T t = L[IDX(j, k, ldl)];                                                           \
                if (t != (T)0)                                                                     \
                    for (int i = 0; i < m; i++) B[IDX(i, j, ldb)] -= t * B[IDX(i, k, ldb)];        \
            }                                                                                      \
        }                                                                                          \
    }                                                                                              \
    /* C[n x n] (lower) -= A A^T: SSYRK(L,N,-1,+1) (cholesky_kernels.c:169) */                     \
    static void syrk_tile_##SFX(int n, int k, const T *A, int lda, T *C, int ldc)                  \
    {                                                                                              \
        for (int j = 0; j < n; j++)                                                                \
            for (int p = 0; p < k; p++) {                                                          \
                T t = -A[IDX(j, p, lda)];                                                          \
                for (int i = j; i < n; i++) C[IDX(i, j, ldc)] += t * A[IDX(i, p, lda)];            \
            }                                                                                      \
    }                                                                                              \
    /* C[m x n] -= A B^T: SGEMM(N,T,-1,+1) (cholesky_kernels.c:75) */                              \
    static void gemm_tile_##SFX(int m, int n, int k, const T *A, int lda, const T *B, int ldb, T *C, int ldc) \
    {                                                                                              \
        for (int j = 0; j < n; j++)                                                                \
            for (int p = 0; p < k; p++) {                                                          \
                T t = -B[IDX(j, p, ldb)];                                                          \
                for (int i = 0; i < m; i++) C[IDX(i, j, ldc)] += t * A[IDX(i, p, lda)];            \
            }                                                                                      \
    }                                                                                              \
    /* Tiled right-looking Cholesky in the task order of cholesky_implicit.c:244-318, */           \
    /* nblocks x nblocks tiles cut like starpu_matrix_filter_block / _vertical_block.  */           \
    /* Returns 0 or the LAPACK-style info of the first failing pivot. */                           \
    int oracle_potrf_tiled_##SFX(int n, T *A, int lda, int nblocks)                                 \
    {                                                                                              \
        int sz[1024], off[1024];                                                                   \
        if (nblocks < 1) nblocks = 1;                                                              \
        if (nblocks > 1024 || nblocks > n) return -1;                                             \
        for (int b = 0; b < nblocks; b++) oracle_chunk(n, nblocks, b, &sz[b], &off[b]);            \
        for (int k = 0; k < nblocks; k++) {                                                        \
            T *Akk = A + IDX(off[k], off[k], lda);                                                 \
            int info = potrf_tile_##SFX(sz[k], Akk, lda);                                          \
            if (info) return off[k] + info;                                                        \
            for (int m = k + 1; m < nblocks; m++)                                                  \
                trsm_tile_##SFX(sz[m], sz[k], Akk, lda, A + IDX(off[m], off[k], lda), lda);        \
            for (int nn = k + 1; nn < nblocks; nn++) {                                             \
                syrk_tile_##SFX(sz[nn], sz[k], A + IDX(off[nn], off[k], lda), lda,                 \
                                A + IDX(off[nn], off[nn], lda), lda);                              \
                for (int m = nn + 1; m < nblocks; m++)                                             \
                    gemm_tile_##SFX(sz[m], sz[nn], sz[k], A + IDX(off[m], off[k], lda), lda,       \
                                    A + IDX(off[nn], off[k], lda), lda, A + IDX(off[m], off[nn], lda), lda); \
            }                                                                                      \
        }                                                                                          \
        return 0;                                                                                  \
    }                                                                                              \
    /* POTRS: L y = b then L^T x = y (min-dgels/base/SRC/dpotrs.c, uplo = L) */                     \
    void oracle_potrs_##SFX(int n, int nrhs, const T *L, int ldl, T *B, int ldb)                   \
    {                                                                                              \
        for (int c = 0; c < nrhs; c++) {                                                           \
            T *b = B + (size_t)c * ldb;                                                            \
            for (int j = 0; j < n; j++) {                                                          \
                b[j] /= L[IDX(j, j, ldl)];                                                         \
                T t = b[j];                                                                        \
                for (int i = j + 1; i < n; i++) b[i] -= t * L[IDX(i, j, ldl)];                     \
            }                                                                                      \
            for (int j = n - 1; j >= 0; j--) {                                                     \
                T s = b[j];                                                                        \
                for (int i = j + 1; i < n; i++) s -= L[IDX(i, j, ldl)] * b[i];                     \
                b[j] = s / L[IDX(j, j, ldl)];                                                      \
            }                                                                                      \
        }                                                                                          \
    }

DEFINE_TILE_KERNELS(float, f32, sqrtf)
DEFINE_TILE_KERNELS(double, f64, sqrt)

/* ---------------------------------------------------------------- checks */

/* The reference's -check (cholesky_implicit.c:530-585): zero the strict
 * upper part, T = L L^T, every lower element of T must match the known input
 * 1/(1+m+n) + size*delta within relative error `tol` (1e-4 there).  Returns
 * the number of violations; *max_err gets the largest relative error. */
int oracle_check_hilbert_f32(int n, const float *L, int ldl, float tol, double *max_err)
{
    int bad = 0;
    double worst = 0.0;
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++) {
            float s = 0.0f;
            for (int p = 0; p <= j; p++) s += L[IDX(i, p, ldl)] * L[IDX(j, p, ldl)];
            float orig = (1.0f / (1.0f + i + j)) + ((i == j) ? 1.0f * n : 0.0f);
            float err = fabsf(s - orig) / orig;
            if (err > worst) worst = err;
            if (err > tol) bad++;
        }
    if (max_err) *max_err = worst;
    return bad;
}

/* ||A - L L^T||_F / ||A||_F over the full symmetric matrix (lower of A read),
 * accumulated in double; L may be float (is_f32) or double. */
double oracle_llt_residual(int n, const double *A, int lda, const void *L, int ldl, int is_f32)
{
    const float *Lf = (const float *)L;
    const double *Ld = (const double *)L;
#define LV(i, j) (is_f32 ? (double)Lf[IDX(i, j, ldl)] : Ld[IDX(i, j, ldl)])
    double num = 0.0, den = 0.0;
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++) {
            double s = 0.0;
            for (int p = 0; p <= j; p++) s += LV(i, p) * LV(j, p);
            double a = A[IDX(i, j, lda)];
            double w = (i == j) ? 1.0 : 2.0;
            num += w * (a - s) * (a - s);
            den += w * a * a;
        }
#undef LV
    return sqrt(num) / sqrt(den);
}

/* Normwise backward error per right-hand side:
 * ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), A full symmetric.
 * Writes one value per column into berr and returns the max. */
double oracle_backward_error(int n, int nrhs, const double *A, int lda, const double *X, int ldx, const double *B,
                             int ldb, double *berr)
{
    double anorm = 0.0;
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int j = 0; j < n; j++) s += fabs(A[IDX(i, j, lda)]);
        if (s > anorm) anorm = s;
    }
    double worst = 0.0;
    double *r = (double *)malloc((size_t)n * sizeof(double));
    for (int c = 0; c < nrhs; c++) {
        const double *x = X + (size_t)c * ldx, *b = B + (size_t)c * ldb;
        for (int i = 0; i < n; i++) r[i] = b[i];
        for (int j = 0; j < n; j++) {
            double t = x[j];
            for (int i = 0; i < n; i++) r[i] -= A[IDX(i, j, lda)] * t;
        }
        double rn = 0, xn = 0, bn = 0;
        for (int i = 0; i < n; i++) {
            if (fabs(r[i]) > rn) rn = fabs(r[i]);
            if (fabs(x[i]) > xn) xn = fabs(x[i]);
            if (fabs(b[i]) > bn) bn = fabs(b[i]);
        }
        double e = rn / (anorm * xn + bn);
        if (berr) berr[c] = e;
        if (e > worst) worst = e;
    }
    free(r);
    return worst;
}

/* FLOPS_SPOTRF(n) of examples/cholesky/cholesky.h:95-98 (magma flop model). */
double oracle_flops_potrf(double n)
{
    double fmuls = n * (((1. / 6.) * n + 0.5) * n + (1. / 3.));
    double fadds = n * (((1. / 6.) * n) * n - (1. / 6.));
    return fmuls + fadds;
}

/* ------------------------------------------------- mixed precision + IR */

/* Restatement of the mixed-precision solve: factor an FP32 copy of A with the
 * tiled algorithm, solve in FP32, then iterate r = b - A x (FP64),
 * d = (L L^T)^{-1} r (FP32), x += d (FP64) until the normwise backward error
 * is <= tol or max_iter corrections were applied (LAPACK dsposv semantics).
 * Returns the number of corrections, -1 if it did not converge, or -(1000+info)
 * if the FP32 factorisation failed. */
int oracle_dsposv_ir(int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X, int ldx,
                     int nblocks, double tol, int max_iter, double *final_berr)
{
    float *L = (float *)malloc((size_t)n * n * sizeof(float));
    float *w = (float *)malloc((size_t)n * nrhs * sizeof(float));
    double *R = (double *)malloc((size_t)n * nrhs * sizeof(double));
    double *berr = (double *)malloc((size_t)nrhs * sizeof(double));
    int ret = -1;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) L[IDX(i, j, n)] = (float)A[IDX(i, j, lda)];
    int info = oracle_potrf_tiled_f32(n, L, n, nblocks);
    if (info) { ret = -(1000 + info); goto out; }
    for (int c = 0; c < nrhs; c++)
        for (int i = 0; i < n; i++) w[IDX(i, c, n)] = (float)B[IDX(i, c, ldb)];
    oracle_potrs_f32(n, nrhs, L, n, w, n);
    for (int c = 0; c < nrhs; c++)
        for (int i = 0; i < n; i++) X[IDX(i, c, ldx)] = (double)w[IDX(i, c, n)];
    for (int it = 0; it <= max_iter; it++) {
        double e = oracle_backward_error(n, nrhs, A, lda, X, ldx, B, ldb, berr);
        if (final_berr) *final_berr = e;
        if (e <= tol) { ret = it; goto out; }
        if (it == max_iter) break;
        for (int c = 0; c < nrhs; c++) {
            for (int i = 0; i < n; i++) R[IDX(i, c, n)] = B[IDX(i, c, ldb)];
            for (int j = 0; j < n; j++) {
                double t = X[IDX(j, c, ldx)];
                for (int i = 0; i < n; i++) R[IDX(i, c, n)] -= A[IDX(i, j, lda)] * t;
            }
            for (int i = 0; i < n; i++) w[IDX(i, c, n)] = (float)R[IDX(i, c, n)];
        }
        oracle_potrs_f32(n, nrhs, L, n, w, n);
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) X[IDX(i, c, ldx)] += (double)w[IDX(i, c, n)];
    }
out:
    free(L);
    free(w);
    free(R);
    free(berr);
    return ret;
}
