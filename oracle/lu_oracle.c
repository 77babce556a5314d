/*
 * ORACLE (test infrastructure only; never linked into the product): plain-C
 * restatement of the CPU branches of the LU codelets of examples/lu, in FP32
 * and FP64, used by tests/ to check the GPU tile kernels.  The reference's
 * own CPU codelets, compiled from its tree (oracle/Makefile target
 * `ref-lu`), pin it through the golden vectors tests/golden/lu_golden.npz.
 *
 * Factor form (examples/lu/xlu_kernels.c:369-380): A = L U with L lower
 * non-unit (the pivot stays in L) and U unit upper (the pivot row is scaled by
 * 1/pivot, the scale computed in double and rounded to the element type).
 * Threshold pivoting (xlu_kernels.c:516-545): when |a_zz| < thr, the largest
 * |a_zj| (j >= z, first on ties) is found and columns z and j are swapped
 * over all rows; ipiv[z] records j, -1 when step z did not pivot.
 *
 * iamax_shift: the reference CPU branch uses STARPU_ISAMAX as a 0-based
 * index (xlu_kernels.c:524-534), but with a Fortran-interface BLAS
 * (examples/common/blas.c:376-381, the OpenBLAS build) that routine returns
 * the 1-based index, so that build swaps in the column after the largest
 * entry; its CUDA branch subtracts 1 (xlu_kernels.c:566).  iamax_shift = 0 is
 * the CUDA branch (the intended choice), 1 reproduces the CPU branch of the
 * Fortran-BLAS build (used only to pin this restatement to its outputs).
 */
#include <math.h>
#include <stddef.h>

#define LU_DEFINE(T, P)                                                                                               \
    /* returns 0, or k + 1 for the first zero pivot */                                                              \
    int oracle_##P##lu_getrf(int n, T *A, int lda, T thr, int *ipiv, int iamax_shift)                                 \
    {                                                                                                               \
        int info = 0;                                                                                               \
        for (int z = 0; z < n; ++z) {                                                                               \
            T pivot = A[z + (size_t)z * lda];                                                                       \
            if (ipiv) ipiv[z] = -1;                                                                                 \
            if (thr > 0 && fabs((double)pivot) < (double)thr) {                                                    \
                int best = z;                                                                                       \
                double bv = fabs((double)A[z + (size_t)z * lda]);                                                  \
                for (int j = z + 1; j < n; ++j) {                                                                   \
                    const double v = fabs((double)A[z + (size_t)j * lda]);                                         \
                    if (v > bv) bv = v, best = j;                                                                   \
                }                                                                                                   \
                best += iamax_shift;                                                                                \
                if (best >= n) best = n - 1;                                                                        \
                if (ipiv) ipiv[z] = best;                                                                           \
                if (best != z)                                                                                      \
                    for (int i = 0; i < n; ++i) {                                                                   \
                        T t = A[i + (size_t)z * lda];                                                               \
                        A[i + (size_t)z * lda] = A[i + (size_t)best * lda];                                         \
                        A[i + (size_t)best * lda] = t;                                                              \
                    }                                                                                               \
                pivot = A[z + (size_t)z * lda];                                                                     \
            }                                                                                                       \
            if (pivot == 0 && !info) info = z + 1;                                                                  \
            const T inv = (T)(1.0 / (double)pivot);                                                                 \
            for (int j = z + 1; j < n; ++j) A[z + (size_t)j * lda] *= inv;                                          \
            for (int j = z + 1; j < n; ++j) {                                                                       \
                const T u = A[z + (size_t)j * lda];                                                                 \
                for (int i = z + 1; i < n; ++i) A[i + (size_t)j * lda] -= A[i + (size_t)z * lda] * u;               \
            }                                                                                                       \
        }                                                                                                           \
        return info;                                                                                                \
    }                                                                                                               \
    /* B <- L^-1 B, L m x m lower non-unit (xlu_kernels.c:192, STRSM L,L,N,N) */                                    \
    void oracle_##P##lu_trsm_ll(int m, int n, const T *L, int ldl, T *B, int ldb)                                    \
    {                                                                                                               \
        for (int c = 0; c < n; ++c) {                                                                               \
            T *b = B + (size_t)c * ldb;                                                                             \
            for (int k = 0; k < m; ++k) {                                                                           \
                b[k] /= L[k + (size_t)k * ldl];                                                                     \
                for (int i = k + 1; i < m; ++i) b[i] -= b[k] * L[i + (size_t)k * ldl];                              \
            }                                                                                                       \
        }                                                                                                           \
    }                                                                                                               \
    /* B <- B U^-1, U n x n unit upper (xlu_kernels.c:281, STRSM R,U,N,U) */                                        \
    void oracle_##P##lu_trsm_ru(int m, int n, const T *U, int ldu, T *B, int ldb)                                    \
    {                                                                                                               \
        for (int j = 0; j < n; ++j)                                                                                 \
            for (int k = 0; k < j; ++k) {                                                                           \
                const T u = U[k + (size_t)j * ldu];                                                                 \
                for (int i = 0; i < m; ++i) B[i + (size_t)j * ldb] -= u * B[i + (size_t)k * ldb];                   \
            }                                                                                                       \
    }                                                                                                               \
    /* C <- C - A B (xlu_kernels.c:66, GEMM N,N alpha = -1, beta = 1) */                                            \
    void oracle_##P##lu_gemm(int m, int n, int k, const T *A, int lda, const T *B, int ldb, T *C, int ldc)          \
    {                                                                                                               \
        for (int j = 0; j < n; ++j)                                                                                 \
            for (int p = 0; p < k; ++p) {                                                                           \
                const T b = B[p + (size_t)j * ldb];                                                                 \
                for (int i = 0; i < m; ++i) C[i + (size_t)j * ldc] -= A[i + (size_t)p * lda] * b;                   \
            }                                                                                                       \
    }                                                                                                               \
    /* the PIVOT codelet (xlu_kernels.c:686-693): for r = 0 .. n-1 in order,   \
       swap columns r and ipiv[r] when they differ (ipiv tile-local) */                                             \
    void oracle_##P##lu_pivot(int n, T *A, int lda, const int *ipiv)                                                 \
    {                                                                                                               \
        for (int r = 0; r < n; ++r) {                                                                               \
            const int p = ipiv[r];                                                                                  \
            if (p != r)                                                                                             \
                for (int i = 0; i < n; ++i) {                                                                       \
                    T t = A[i + (size_t)r * lda];                                                                   \
                    A[i + (size_t)r * lda] = A[i + (size_t)p * lda];                                                \
                    A[i + (size_t)p * lda] = t;                                                                     \
                }                                                                                                   \
        }                                                                                                           \
    }

LU_DEFINE(float, s)
LU_DEFINE(double, d)
