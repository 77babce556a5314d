// C-ABI over the SIMT dense kernels: tile codelet bodies (POTRF/TRSM/SYRK/GEMM
// on one tile, FP32 and FP64) and the whole-matrix tiled factorisation and
// triangular solves composed from them.  Every entry point only enqueues work
// on the caller's stream and returns; nothing here synchronises or allocates.
#include "kernels/simt_blas.cuh"
#include "kernels/trsv_sweep.cuh"
#include "gb300_internal.h"
#include "starpu_gb300_kernels.h"

#include <algorithm>
#include <type_traits>

namespace gb300 {

static inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

template <typename T, bool TA, bool TB, int BM, int BN, int BK, int TM, int TN>
static void gemm_launch(cudaStream_t s, bool lower, int m, int n, int k, T alpha, const T *A, long lda, const T *B,
                        long ldb, T beta, T *C, long ldc)
{
    constexpr int NT = (BM / TM) * (BN / TN);
    // the lower-triangular form is only ever used as C -= A A^T (N,T)
    if constexpr (!TA && TB && BM == BN) {
        if (lower) {
            long tb = cdiv(m, BM);
            gb300_count_launch(), gemm_simt_kernel<T, TA, TB, BM, BN, BK, TM, TN, true>
                <<<dim3((unsigned)(tb * (tb + 1) / 2)), NT, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
            return;
        }
    }
    {
        gb300_count_launch(), gemm_simt_kernel<T, TA, TB, BM, BN, BK, TM, TN, false>
            <<<dim3(cdiv(m, BM), cdiv(n, BN)), NT, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    }
}

template <typename T> struct simt_cfg;
// FP32: 128x128 block tiles, 8x8 per thread; narrow variant for few columns (RHS blocks).
template <> struct simt_cfg<float> {
    template <bool TA, bool TB>
    static void run(cudaStream_t s, bool lower, int m, int n, int k, float al, const float *A, long lda,
                    const float *B, long ldb, float be, float *C, long ldc)
    {
        if (!lower && n <= 32)
            gemm_launch<float, TA, TB, 128, 32, 8, 8, 2>(s, lower, m, n, k, al, A, lda, B, ldb, be, C, ldc);
        else
            gemm_launch<float, TA, TB, 128, 128, 8, 8, 8>(s, lower, m, n, k, al, A, lda, B, ldb, be, C, ldc);
    }
};
// FP64: 64x64 block tiles, 4x4 per thread.
template <> struct simt_cfg<double> {
    template <bool TA, bool TB>
    static void run(cudaStream_t s, bool lower, int m, int n, int k, double al, const double *A, long lda,
                    const double *B, long ldb, double be, double *C, long ldc)
    {
        if (!lower && n <= 16)
            gemm_launch<double, TA, TB, 64, 16, 8, 4, 2>(s, lower, m, n, k, al, A, lda, B, ldb, be, C, ldc);
        else
            gemm_launch<double, TA, TB, 64, 64, 8, 4, 4>(s, lower, m, n, k, al, A, lda, B, ldb, be, C, ldc);
    }
};

template <typename T>
void gemm(cudaStream_t s, bool ta, bool tb, bool lower, int m, int n, int k, T alpha, const T *A, long lda,
          const T *B, long ldb, T beta, T *C, long ldc)
{
    if (m <= 0 || n <= 0) return;
    if (!ta && !tb) simt_cfg<T>::template run<false, false>(s, lower, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (!ta && tb) simt_cfg<T>::template run<false, true>(s, lower, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (ta && !tb) simt_cfg<T>::template run<true, false>(s, lower, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else simt_cfg<T>::template run<true, true>(s, lower, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// `batch` independent products C_z = alpha * A_z B_z + beta * C_z (no
// transposes), A_z = A + z * astride and likewise for B and C: one launch.
template <typename T>
void gemm_batched_nn(cudaStream_t s, int m, int n, int k, T alpha, const T *A, long lda, long astride, const T *B,
                     long ldb, long bstride, T beta, T *C, long ldc, long cstride, int batch)
{
    if (m <= 0 || n <= 0 || batch <= 0) return;
    if constexpr (std::is_same<T, float>::value)
        gb300_count_launch(), gemm_simt_kernel<T, false, false, 128, 128, 8, 8, 8, false>
            <<<dim3(cdiv(m, 128), cdiv(n, 128), batch), 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, -1,
                                                                    cstride, astride, bstride);
    else
        gb300_count_launch(), gemm_simt_kernel<T, false, false, 64, 64, 8, 4, 4, false>
            <<<dim3(cdiv(m, 64), cdiv(n, 64), batch), 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, -1,
                                                                  cstride, astride, bstride);
}

// Linv (n x n, ld ldi, strictly upper part zeroed) = inverse of the lower
// triangle of L: the 64 x 64 diagonal blocks by forward substitution, then
// doubling -- neighbouring inverted blocks of order h combine as
//   [L11 0; L21 L22]^-1 = [I11 0; -I22 (L21 I11)  I22],
// every pair of one level in one batched launch per product.  scratch holds
// >= n * n / 4 elements.
template <typename T>
void trtri_lower(cudaStream_t s, int n, const T *L, long ldl, T *Linv, long ldi, T *scratch)
{
    if (n <= 0) return;
    cudaMemset2DAsync(Linv, ldi * sizeof(T), 0, n * sizeof(T), n, s);
    gb300_count_launch(), invert_diag_blocks_kernel<T, 64>
        <<<cdiv(n, 64), 64, 0, s>>>(n, L, ldl, Linv, ldi, 64 * (ldi + 1), true);
    for (int h = 64; h < n; h *= 2) {
        const int full = n / (2 * h);  // pairs whose halves both have order h
        const long sl = 2L * h * (ldl + 1), si = 2L * h * (ldi + 1);
        if (full > 0) {
            gemm_batched_nn<T>(s, h, h, h, T(1), L + h, ldl, sl, Linv, ldi, si, T(0), scratch, h, (long)h * h, full);
            gemm_batched_nn<T>(s, h, h, h, T(-1), Linv + h + (long)h * ldi, ldi, si, scratch, h, (long)h * h, T(0),
                               Linv + h, ldi, si, full);
        }
        const int o = full * 2 * h, r = n - o - h;  // a last pair whose second half has order r < h
        if (r > 0) {
            gemm<T>(s, false, false, false, r, h, h, T(1), L + (o + h) + (long)o * ldl, ldl, Linv + o + (long)o * ldi,
                    ldi, T(0), scratch, r);
            gemm<T>(s, false, false, false, r, h, r, T(-1), Linv + (o + h) + (long)(o + h) * ldi, ldi, scratch, r, T(0),
                    Linv + (o + h) + (long)o * ldi, ldi);
        }
    }
}

// B[m x nc] <- B * L^{-T}, blocked by SMALL_W columns: small triangular solve
// of one column block, then a GEMM update of the remaining columns.
template <typename T>
void trsm_rltn(cudaStream_t s, int m, int nc, const T *L, long ldl, T *B, long ldb)
{
    if (m <= 0 || nc <= 0) return;
    constexpr int SMALL_W = small_w<T>::value;
    for (int j0 = 0; j0 < nc; j0 += SMALL_W) {
        const int w = std::min(SMALL_W, nc - j0);
        const T *Ljj = L + j0 + (long)j0 * ldl;
        T *Bj = B + (long)j0 * ldb;
        if (w == SMALL_W)
            gb300_count_launch(), trsm_rltn_small_kernel<T, SMALL_W, true><<<cdiv(m, 128), 128, 0, s>>>(m, w, Ljj, ldl, Bj, ldb);
        else
            gb300_count_launch(), trsm_rltn_small_kernel<T, SMALL_W, false><<<cdiv(m, 128), 128, 0, s>>>(m, w, Ljj, ldl, Bj, ldb);
        const int rest = nc - j0 - w;
        if (rest > 0)
            gemm<T>(s, false, true, false, m, rest, w, T(-1), Bj, ldb, L + (j0 + w) + (long)j0 * ldl, ldl, T(1),
                    B + (long)(j0 + w) * ldb, ldb);
    }
}

// Right-looking tiled Cholesky with tile nb: POTRF(k), TRSM of the whole
// column panel below it, then the lower-triangular trailing update.  This is
// the loop of examples/cholesky/cholesky_implicit.c:244-318 with the tasks of
// one step k fused into whole-panel launches.  Diagonal blocks larger than
// SMALL_W are themselves factored by the same algorithm with tile SMALL_W.
template <typename T>
void potrf_tiled(cudaStream_t s, int n, T *A, long lda, int nb, int *info, int info_base)
{
    constexpr int SMALL_W = small_w<T>::value;
    if (nb <= 0) nb = n;
    for (int k0 = 0; k0 < n; k0 += nb) {
        const int kb = std::min(nb, n - k0);
        T *Akk = A + k0 + (long)k0 * lda;
        if (kb <= SMALL_W)
            gb300_count_launch(), potf2_small_kernel<T, SMALL_W><<<1, 256, 0, s>>>(kb, Akk, lda, info, info_base + k0);
        else
            potrf_tiled<T>(s, kb, Akk, lda, SMALL_W, info, info_base + k0);
        const int m = n - k0 - kb;
        if (m > 0) {
            T *P = A + (k0 + kb) + (long)k0 * lda;
            trsm_rltn<T>(s, m, kb, Akk, lda, P, lda);
            gemm<T>(s, false, true, true, m, m, kb, T(-1), P, lda, P, lda, T(1), A + (k0 + kb) + (long)(k0 + kb) * lda,
                    lda);
        }
    }
}

// POTRS with a lower factor: L y = b (forward), then L^T x = y (backward),
// blocked by SMALL_W rows; min-dgels/base/SRC/dpotrs.c does the same two
// sweeps through dtrsm.
// Block width of the POTRS sweeps: 128 rows (FP32) / 64 rows (FP64) per
// diagonal solve, so a sweep over n rows costs n / W diagonal solves and
// n / W GEMM updates.
template <typename T> struct potrs_w { static constexpr int value = 128; };
template <> struct potrs_w<double> { static constexpr int value = 64; };

template <typename T, bool TRANS>
static void trsv_block(cudaStream_t s, int w, int nrhs, const T *L, long ldl, T *B, long ldb)
{
    constexpr int W = potrs_w<T>::value;
    constexpr size_t smem = (size_t)(W * (W + 1) + W * 16) * sizeof(T);
    if (gb300_func_dyn_smem((const void *)trsv_block_kernel<T, W, TRANS>, (int)smem)) return;
    gb300_count_launch(), trsv_block_kernel<T, W, TRANS><<<cdiv(nrhs, 16), 128, smem, s>>>(w, nrhs, L, ldl, B, ldb);
}

template <typename T>
void potrs_blocked(cudaStream_t s, int n, int nrhs, const T *L, long ldl, T *B, long ldb)
{
    if (n <= 0 || nrhs <= 0) return;
    constexpr int W = potrs_w<T>::value;
    for (int j0 = 0; j0 < n; j0 += W) {
        const int w = std::min(W, n - j0);
        trsv_block<T, false>(s, w, nrhs, L + j0 + (long)j0 * ldl, ldl, B + j0, ldb);
        const int rest = n - j0 - w;
        if (rest > 0)
            gemm<T>(s, false, false, false, rest, nrhs, w, T(-1), L + (j0 + w) + (long)j0 * ldl, ldl, B + j0, ldb,
                    T(1), B + j0 + w, ldb);
    }
    const int last = ((n - 1) / W) * W;
    for (int j0 = last; j0 >= 0; j0 -= W) {
        const int w = std::min(W, n - j0);
        trsv_block<T, true>(s, w, nrhs, L + j0 + (long)j0 * ldl, ldl, B + j0, ldb);
        if (j0 > 0)
            gemm<T>(s, true, false, false, j0, nrhs, w, T(-1), L + j0, ldl, B + j0, ldb, T(1), B, ldb);
    }
}

// ---- single-launch POTRS sweeps with inverted 64 x 64 diagonal blocks ------

template <typename T>
size_t potrs_sweep_workspace(int n)
{
    const size_t nblk = ((size_t)n + 63) / 64;
    return ((nblk * 64 * 64 * sizeof(T) + 255) & ~(size_t)255) + (((nblk + 2) * sizeof(int) + 255) & ~(size_t)255);
}

// Invert every diagonal 64 x 64 block of L (once per factorisation).
template <typename T>
void potrs_sweep_prepare(cudaStream_t s, int n, const T *L, long ldl, void *ws)
{
    if (n <= 0) return;
    const unsigned nblk = cdiv(n, 64);
    gb300_count_launch(), invert_diag_blocks_kernel<T, 64><<<nblk, 64, 0, s>>>(n, L, ldl, (T *)ws, 64, 64 * 64, false);
}

// L y = b then L^T x = y, one launch per sweep and group of 16 columns (FP32).
template <typename T>
void potrs_sweep(cudaStream_t s, int n, int nrhs, const T *L, long ldl, void *ws, T *B, long ldb, int *err)
{
    if (n <= 0 || nrhs <= 0) return;
    const int nblk = (int)cdiv(n, 64);
    const T *Linv = (const T *)ws;
    int *flags = (int *)((char *)ws + (((size_t)nblk * 64 * 64 * sizeof(T) + 255) & ~(size_t)255));
    unsigned *ticket = (unsigned *)(flags + nblk);
    const unsigned long long budget = gb300_wait_budget_ns();
    static_assert(std::is_same<T, float>::value, "the single-launch sweeps are FP32");
    if (gb300_func_dyn_smem((const void *)trsv_sweep_kernel<false>, SWEEP_SMEM) ||
        gb300_func_dyn_smem((const void *)trsv_sweep_kernel<true>, SWEEP_SMEM))
        return;
    for (int c0 = 0; c0 < nrhs; c0 += 16) {
        const int nr = std::min(16, nrhs - c0);
        cudaMemsetAsync(flags, 0, (nblk + 1) * sizeof(int), s);
        gb300_count_launch(), trsv_sweep_kernel<false>
            <<<nblk, 256, SWEEP_SMEM, s>>>(n, nr, L, ldl, Linv, B + (long)c0 * ldb, ldb, ticket, flags, err, budget);
        cudaMemsetAsync(flags, 0, (nblk + 1) * sizeof(int), s);
        gb300_count_launch(), trsv_sweep_kernel<true>
            <<<nblk, 256, SWEEP_SMEM, s>>>(n, nr, L, ldl, Linv, B + (long)c0 * ldb, ldb, ticket, flags, err, budget);
    }
}

template size_t potrs_sweep_workspace<float>(int);
template size_t potrs_sweep_workspace<double>(int);
template void potrs_sweep_prepare<float>(cudaStream_t, int, const float *, long, void *);
template void potrs_sweep_prepare<double>(cudaStream_t, int, const double *, long, void *);
template void potrs_sweep<float>(cudaStream_t, int, int, const float *, long, void *, float *, long, int *);

template void gemm<float>(cudaStream_t, bool, bool, bool, int, int, int, float, const float *, long, const float *,
                          long, float, float *, long);
template void gemm<double>(cudaStream_t, bool, bool, bool, int, int, int, double, const double *, long,
                           const double *, long, double, double *, long);
template void trsm_rltn<float>(cudaStream_t, int, int, const float *, long, float *, long);
template void trsm_rltn<double>(cudaStream_t, int, int, const double *, long, double *, long);
template void potrf_tiled<float>(cudaStream_t, int, float *, long, int, int *, int);
template void trtri_lower<float>(cudaStream_t, int, const float *, long, float *, long, float *);
template void potrf_tiled<double>(cudaStream_t, int, double *, long, int, int *, int);
template void potrs_blocked<float>(cudaStream_t, int, int, const float *, long, float *, long);
template void potrs_blocked<double>(cudaStream_t, int, int, const double *, long, double *, long);

} // namespace gb300

using namespace gb300;

#define GB300_STREAM(s) ((cudaStream_t)(s))

extern "C" {

// ---- tile codelet bodies -------------------------------------------------

int starpu_gb300_spotrf_tile(void *stream, int n, float *A, int lda, int *d_info)
{
    if (n < 0 || lda < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), GB300_STREAM(stream));
    if (n) potrf_tiled<float>(GB300_STREAM(stream), n, A, lda, small_w<float>::value, d_info, 0);
    return gb300_last_launch_status();
}

int starpu_gb300_dpotrf_tile(void *stream, int n, double *A, int lda, int *d_info)
{
    if (n < 0 || lda < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), GB300_STREAM(stream));
    if (n) potrf_tiled<double>(GB300_STREAM(stream), n, A, lda, small_w<double>::value, d_info, 0);
    return gb300_last_launch_status();
}

int starpu_gb300_spotrf_tile_status(void *stream, int n, float *A, int lda, int *d_status)
{
    if (n < 0 || lda < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (n) potrf_tiled<float>(GB300_STREAM(stream), n, A, lda, small_w<float>::value, d_status, 0);
    return gb300_last_launch_status();
}

int starpu_gb300_dpotrf_tile_status(void *stream, int n, double *A, int lda, int *d_status)
{
    if (n < 0 || lda < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (n) potrf_tiled<double>(GB300_STREAM(stream), n, A, lda, small_w<double>::value, d_status, 0);
    return gb300_last_launch_status();
}

int starpu_gb300_strsm_rltn_tile(void *stream, int m, int n, float alpha, const float *L, int ldl, float *B, int ldb)
{
    if (m < 0 || n < 0 || ldl < (n > 1 ? n : 1) || ldb < (m > 1 ? m : 1)) return GB300_EINVAL;
    if (alpha != 1.0f) return GB300_ENOTSUP;
    trsm_rltn<float>(GB300_STREAM(stream), m, n, L, ldl, B, ldb);
    return gb300_last_launch_status();
}

int starpu_gb300_dtrsm_rltn_tile(void *stream, int m, int n, double alpha, const double *L, int ldl, double *B, int ldb)
{
    if (m < 0 || n < 0 || ldl < (n > 1 ? n : 1) || ldb < (m > 1 ? m : 1)) return GB300_EINVAL;
    if (alpha != 1.0) return GB300_ENOTSUP;
    trsm_rltn<double>(GB300_STREAM(stream), m, n, L, ldl, B, ldb);
    return gb300_last_launch_status();
}

int starpu_gb300_ssyrk_ln_tile(void *stream, int n, int k, float alpha, const float *A, int lda, float beta, float *C,
                               int ldc)
{
    if (n < 0 || k < 0 || lda < (n > 1 ? n : 1) || ldc < (n > 1 ? n : 1)) return GB300_EINVAL;
    gemm<float>(GB300_STREAM(stream), false, true, true, n, n, k, alpha, A, lda, A, lda, beta, C, ldc);
    return gb300_last_launch_status();
}

int starpu_gb300_dsyrk_ln_tile(void *stream, int n, int k, double alpha, const double *A, int lda, double beta,
                               double *C, int ldc)
{
    if (n < 0 || k < 0 || lda < (n > 1 ? n : 1) || ldc < (n > 1 ? n : 1)) return GB300_EINVAL;
    gemm<double>(GB300_STREAM(stream), false, true, true, n, n, k, alpha, A, lda, A, lda, beta, C, ldc);
    return gb300_last_launch_status();
}

int starpu_gb300_sgemm_nt_tile(void *stream, int m, int n, int k, float alpha, const float *A, int lda, const float *B,
                               int ldb, float beta, float *C, int ldc)
{
    if (m < 0 || n < 0 || k < 0 || lda < (m > 1 ? m : 1) || ldb < (n > 1 ? n : 1) || ldc < (m > 1 ? m : 1))
        return GB300_EINVAL;
    gemm<float>(GB300_STREAM(stream), false, true, false, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return gb300_last_launch_status();
}

int starpu_gb300_dgemm_nt_tile(void *stream, int m, int n, int k, double alpha, const double *A, int lda,
                               const double *B, int ldb, double beta, double *C, int ldc)
{
    if (m < 0 || n < 0 || k < 0 || lda < (m > 1 ? m : 1) || ldb < (n > 1 ? n : 1) || ldc < (m > 1 ? m : 1))
        return GB300_EINVAL;
    gemm<double>(GB300_STREAM(stream), false, true, false, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return gb300_last_launch_status();
}

// ---- whole-matrix plain-precision factorisation and solve -----------------

int starpu_gb300_spotrf(void *stream, int n, float *A, int lda, int nb, int *d_info)
{
    if (n < 0 || lda < (n > 1 ? n : 1) || nb < 0) return GB300_EINVAL;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), GB300_STREAM(stream));
    if (n) potrf_tiled<float>(GB300_STREAM(stream), n, A, lda, nb ? nb : 512, d_info, 0);
    return gb300_last_launch_status();
}

int starpu_gb300_dpotrf(void *stream, int n, double *A, int lda, int nb, int *d_info)
{
    if (n < 0 || lda < (n > 1 ? n : 1) || nb < 0) return GB300_EINVAL;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), GB300_STREAM(stream));
    if (n) potrf_tiled<double>(GB300_STREAM(stream), n, A, lda, nb ? nb : 512, d_info, 0);
    return gb300_last_launch_status();
}

int starpu_gb300_spotrs(void *stream, int n, int nrhs, const float *L, int ldl, float *B, int ldb)
{
    if (n < 0 || nrhs < 0 || ldl < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1)) return GB300_EINVAL;
    potrs_blocked<float>(GB300_STREAM(stream), n, nrhs, L, ldl, B, ldb);
    return gb300_last_launch_status();
}

int starpu_gb300_dpotrs(void *stream, int n, int nrhs, const double *L, int ldl, double *B, int ldb)
{
    if (n < 0 || nrhs < 0 || ldl < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1)) return GB300_EINVAL;
    potrs_blocked<double>(GB300_STREAM(stream), n, nrhs, L, ldl, B, ldb);
    return gb300_last_launch_status();
}

size_t starpu_gb300_spotrs_sweep_workspace(int n)
{
    if (n <= 0) return 0;
    return potrs_sweep_workspace<float>(n) + 256;
}

int starpu_gb300_spotrs_sweep(void *stream, int n, int nrhs, const float *L, int ldl, float *B, int ldb, void *work,
                              size_t lwork, int *d_err)
{
    if (n < 0 || nrhs < 0 || ldl < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (!n || !nrhs) return GB300_OK;
    if (!work || lwork < starpu_gb300_spotrs_sweep_workspace(n) || !d_err) return GB300_EINVAL;
    cudaStream_t s = GB300_STREAM(stream);
    potrs_sweep_prepare<float>(s, n, L, ldl, work);
    potrs_sweep<float>(s, n, nrhs, L, ldl, work, B, ldb, d_err);
    return gb300_last_launch_status();
}

} // extern "C"
