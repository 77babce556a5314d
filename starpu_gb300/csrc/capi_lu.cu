// C-ABI of the tiled LU codelet bodies (examples/lu), FP32 and FP64: the
// factor form of the reference codelets, A = L U with L lower non-unit and U
// unit upper, and their threshold column pivoting.  Every entry point only
// enqueues work on the caller's stream; none synchronises or allocates.
#include <algorithm>
#include <string.h>

#include "gb300_internal.h"
#include "kernels/lu_blas.cuh"
#include "kernels/simt_blas.cuh"
#include "starpu_gb300_kernels.h"

namespace gb300 {

static inline unsigned lu_cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

// B[m x n] <- L^{-1} B, L m x m lower non-unit, blocked by SMALL_W rows:
// diagonal-block solve (one thread per column of B), then the GEMM update of
// the rows below.
template <typename T>
static void trsm_llnn(cudaStream_t s, int m, int n, const T *L, long ldl, T *B, long ldb)
{
    constexpr int W = small_w<T>::value;
    for (int r0 = 0; r0 < m; r0 += W) {
        const int w = std::min(W, m - r0);
        gb300_count_launch(), trsm_left_small_kernel<T, W, false>
            <<<lu_cdiv(n, 64), 64, 0, s>>>(w, n, L + r0 + (long)r0 * ldl, ldl, B + r0, ldb);
        const int rest = m - r0 - w;
        if (rest > 0)
            gemm<T>(s, false, false, false, rest, n, w, T(-1), L + (r0 + w) + (long)r0 * ldl, ldl, B + r0, ldb, T(1),
                    B + r0 + w, ldb);
    }
}

// B[m x n] <- B U^{-1}, U n x n unit upper, blocked by SMALL_W columns.
template <typename T>
static void trsm_runu(cudaStream_t s, int m, int n, const T *U, long ldu, T *B, long ldb)
{
    constexpr int W = small_w<T>::value;
    for (int c0 = 0; c0 < n; c0 += W) {
        const int w = std::min(W, n - c0);
        if (w == W)
            gb300_count_launch(), trsm_runu_small_kernel<T, W, true>
                <<<lu_cdiv(m, 128), 128, 0, s>>>(m, w, U + c0 + (long)c0 * ldu, ldu, B + (long)c0 * ldb, ldb);
        else
            gb300_count_launch(), trsm_runu_small_kernel<T, W, false>
                <<<lu_cdiv(m, 128), 128, 0, s>>>(m, w, U + c0 + (long)c0 * ldu, ldu, B + (long)c0 * ldb, ldb);
        const int rest = n - c0 - w;
        if (rest > 0)
            gemm<T>(s, false, false, false, m, rest, w, T(-1), B + (long)c0 * ldb, ldb, U + c0 + (long)(c0 + w) * ldu,
                    ldu, T(1), B + (long)(c0 + w) * ldb, ldb);
    }
}

// Blocked right-looking LU of one n x n tile (A = L U, L non-unit, U unit):
// per SMALL_W block, the register-resident leaf, U12 = L11^-1 A12,
// L21 = A21 U11^-1, A22 -= L21 U12.  thr > 0 records the first step whose
// pivot falls below thr into *d_first (the diagonal block of a step is fully
// updated when its leaf runs, so the test sees the same values as the
// unblocked loop up to rounding).
template <typename T>
static void getrf_blocked(cudaStream_t s, int n, T *A, long lda, T thr, int *d_first, int *info)
{
    constexpr int W = small_w<T>::value;
    for (int k0 = 0; k0 < n; k0 += W) {
        const int kb = std::min(W, n - k0);
        T *Akk = A + k0 + (long)k0 * lda;
        gb300_count_launch(), getf2_small_kernel<T, W><<<1, 256, 0, s>>>(kb, Akk, lda, thr, d_first, info, k0);
        const int rest = n - k0 - kb;
        if (rest <= 0) break;
        T *A12 = A + k0 + (long)(k0 + kb) * lda, *A21 = A + (k0 + kb) + (long)k0 * lda;
        trsm_llnn<T>(s, kb, rest, Akk, lda, A12, lda);
        trsm_runu<T>(s, rest, kb, Akk, lda, A21, lda);
        gemm<T>(s, false, false, false, rest, rest, kb, T(-1), A21, lda, A12, lda, T(1),
                A + (k0 + kb) + (long)(k0 + kb) * lda, lda);
    }
}

template <typename T>
static int getrf_tile(void *stream, int n, T *A, int lda, int *d_info)
{
    if (n < 0 || lda < (n > 1 ? n : 1)) return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), s);
    if (n) getrf_blocked<T>(s, n, A, lda, T(0), nullptr, d_info);
    return gb300_last_launch_status();
}

// Workspace of the pivoting GETRF: a copy of the tile (n * n elements, ld n)
// and the step at which pivoting began.
template <typename T> static size_t getrf_pivot_ws(int n)
{
    return ((size_t)n * n * sizeof(T) + 255) / 256 * 256 + 256;
}

template <typename T>
static int getrf_pivot_tile(void *stream, int n, T *A, int lda, T threshold, int *d_ipiv, void *work, size_t lwork,
                            int *d_info)
{
    if (n < 0 || lda < (n > 1 ? n : 1) || !(threshold >= T(0))) return GB300_EINVAL;
    if (n && (!d_ipiv || !work || lwork < getrf_pivot_ws<T>(n))) return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), s);
    if (!n) return GB300_OK;
    T *copy = (T *)work;
    int *d_first = (int *)((char *)work + ((size_t)n * n * sizeof(T) + 255) / 256 * 256);
    // no step pivoted yet: ipiv all -1, d_first = n
    cudaMemsetAsync(d_ipiv, 0xff, sizeof(int) * n, s);
    gb300_count_launch(), lu_set_int_kernel<<<1, 1, 0, s>>>(d_first, n);
    cudaMemcpy2DAsync(copy, sizeof(T) * n, A, sizeof(T) * lda, sizeof(T) * n, n, cudaMemcpyDeviceToDevice, s);
    // optimistic: the blocked factorisation, recording the first small pivot
    getrf_blocked<T>(s, n, A, lda, threshold, threshold > T(0) ? d_first : nullptr, d_info);
    if (threshold > T(0)) {
        // if a step needed a pivot: restore the tile and factor it again with pivoting
        gb300_count_launch(), restore_if_flagged_kernel<T>
            <<<lu_cdiv((long)n * n, 256), 256, 0, s>>>(n, copy, A, lda, d_first, d_info);
        gb300_count_launch(), getrf_pivot_unblocked_kernel<T>
            <<<1, 1024, 0, s>>>(n, A, lda, threshold, d_first, d_ipiv, d_info);
    }
    return gb300_last_launch_status();
}

template <typename T>
static int swap_columns(void *stream, int m, int n, T *A, int lda, const int *pairs, int npairs)
{
    if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || npairs < 0 || (npairs && !pairs)) return GB300_EINVAL;
    for (int k = 0; k < 2 * npairs; ++k)
        if (pairs[k] < 0 || pairs[k] >= n) return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (!m || !npairs) return GB300_OK;
    LuSwapList list;
    for (int s0 = 0; s0 < npairs; s0 += LU_SWAP_MAX) {
        list.count = std::min(LU_SWAP_MAX, npairs - s0);
        for (int k = 0; k < list.count; ++k) list.pairs[k] = make_int2(pairs[2 * (s0 + k)], pairs[2 * (s0 + k) + 1]);
        gb300_count_launch(), swap_columns_kernel<T><<<lu_cdiv(m, 256), 256, 0, s>>>(m, A, lda, list);
    }
    return gb300_last_launch_status();
}

template <typename T>
static int trsm_llnn_tile(void *stream, int m, int n, const T *L, int ldl, T *B, int ldb)
{
    if (m < 0 || n < 0 || ldl < (m > 1 ? m : 1) || ldb < (m > 1 ? m : 1)) return GB300_EINVAL;
    if (m && n) trsm_llnn<T>((cudaStream_t)stream, m, n, L, ldl, B, ldb);
    return gb300_last_launch_status();
}

template <typename T>
static int trsm_runu_tile(void *stream, int m, int n, const T *U, int ldu, T *B, int ldb)
{
    if (m < 0 || n < 0 || ldu < (n > 1 ? n : 1) || ldb < (m > 1 ? m : 1)) return GB300_EINVAL;
    if (m && n) trsm_runu<T>((cudaStream_t)stream, m, n, U, ldu, B, ldb);
    return gb300_last_launch_status();
}

template <typename T>
static int gemm_nn_tile(void *stream, int m, int n, int k, T alpha, const T *A, int lda, const T *B, int ldb, T beta,
                        T *C, int ldc)
{
    if (m < 0 || n < 0 || k < 0 || lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1))
        return GB300_EINVAL;
    gemm<T>((cudaStream_t)stream, false, false, false, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    return gb300_last_launch_status();
}

} // namespace gb300

using namespace gb300;

extern "C" {

int starpu_gb300_sgetrf_tile(void *stream, int n, float *A, int lda, int *d_info)
{
    return getrf_tile<float>(stream, n, A, lda, d_info);
}
int starpu_gb300_dgetrf_tile(void *stream, int n, double *A, int lda, int *d_info)
{
    return getrf_tile<double>(stream, n, A, lda, d_info);
}

size_t starpu_gb300_sgetrf_pivot_tile_workspace(int n) { return n > 0 ? getrf_pivot_ws<float>(n) : 0; }
size_t starpu_gb300_dgetrf_pivot_tile_workspace(int n) { return n > 0 ? getrf_pivot_ws<double>(n) : 0; }

int starpu_gb300_sgetrf_pivot_tile(void *stream, int n, float *A, int lda, float threshold, int *d_ipiv, void *work,
                                   size_t lwork, int *d_info)
{
    return getrf_pivot_tile<float>(stream, n, A, lda, threshold, d_ipiv, work, lwork, d_info);
}
int starpu_gb300_dgetrf_pivot_tile(void *stream, int n, double *A, int lda, double threshold, int *d_ipiv, void *work,
                                   size_t lwork, int *d_info)
{
    return getrf_pivot_tile<double>(stream, n, A, lda, threshold, d_ipiv, work, lwork, d_info);
}

int starpu_gb300_strsm_llnn_tile(void *stream, int m, int n, const float *L, int ldl, float *B, int ldb)
{
    return trsm_llnn_tile<float>(stream, m, n, L, ldl, B, ldb);
}
int starpu_gb300_dtrsm_llnn_tile(void *stream, int m, int n, const double *L, int ldl, double *B, int ldb)
{
    return trsm_llnn_tile<double>(stream, m, n, L, ldl, B, ldb);
}

int starpu_gb300_strsm_runu_tile(void *stream, int m, int n, const float *U, int ldu, float *B, int ldb)
{
    return trsm_runu_tile<float>(stream, m, n, U, ldu, B, ldb);
}
int starpu_gb300_dtrsm_runu_tile(void *stream, int m, int n, const double *U, int ldu, double *B, int ldb)
{
    return trsm_runu_tile<double>(stream, m, n, U, ldu, B, ldb);
}

int starpu_gb300_sgemm_nn_tile(void *stream, int m, int n, int k, float alpha, const float *A, int lda, const float *B,
                               int ldb, float beta, float *C, int ldc)
{
    return gemm_nn_tile<float>(stream, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
int starpu_gb300_dgemm_nn_tile(void *stream, int m, int n, int k, double alpha, const double *A, int lda,
                               const double *B, int ldb, double beta, double *C, int ldc)
{
    return gemm_nn_tile<double>(stream, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

int starpu_gb300_sswap_columns_tile(void *stream, int m, int n, float *A, int lda, const int *pairs, int npairs)
{
    return swap_columns<float>(stream, m, n, A, lda, pairs, npairs);
}
int starpu_gb300_dswap_columns_tile(void *stream, int m, int n, double *A, int lda, const int *pairs, int npairs)
{
    return swap_columns<double>(stream, m, n, A, lda, pairs, npairs);
}

} // extern "C"
