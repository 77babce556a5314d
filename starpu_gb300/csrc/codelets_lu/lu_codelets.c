/*
 * The six LU codelets of examples/lu for the GB300 CUDA worker -- the drop-in
 * replacement of examples/lu/xlu_kernels.c's CUDA branches (codelet names and
 * buffer modes of xlu_kernels.c:149-163, 239-253, 328-342, 460-485, 643-657,
 * 747-762), so the unchanged lu_example.c and xlu*.c link against them.  One
 * library serves the float and the double drivers: the element size of the
 * registered matrix selects the FP32 or FP64 kernels.  Each body calls the
 * C-ABI kernel that replaces the reference's vendor calls, on the worker's
 * stream:
 *   GETRF        cusolverDnSgetrf / cublasSscal + cublasSger per column  -> starpu_gb300_?getrf_tile
 *   GETRF_PIVOT  per-column host loop with cublasIsamax / Sswap          -> starpu_gb300_?getrf_pivot_tile
 *   TRSM_LL      cublasStrsm(L, L, N, N)                                 -> starpu_gb300_?trsm_llnn_tile
 *   TRSM_RU      cublasStrsm(R, U, N, U)                                 -> starpu_gb300_?trsm_runu_tile
 *   GEMM         cublasSgemm(N, N)                                       -> starpu_gb300_?gemm_nn_tile
 *   PIVOT        cublasSswap per swapped column                          -> starpu_gb300_?swap_columns_tile
 * All but GETRF_PIVOT are STARPU_CUDA_ASYNC.  GETRF_PIVOT writes the host
 * pivot array of its codelet argument (xlu.h struct piv_s), so it waits for
 * its stream, like the reference's.  The reference asserts on a zero pivot
 * from the host after one synchronisation per column; here nothing waits, so
 * a zero pivot shows as non-finite entries of the factor (the driver's check
 * then fails).
 */
#include <starpu.h>
#include <string.h>

#include "starpu_gb300_kernels.h"

/* the codelet argument of the pivoting codelets (examples/lu/xlu.h) */
struct piv_s {
    unsigned *piv;
    unsigned first;
    unsigned last;
};

starpu_data_handle_t scratch = NULL;
starpu_data_handle_t devInfo = NULL;

/* the reference's pivot thresholds (lu-float.h:45, lu-double.h:45) */
#define THRESHOLD_F32 10e-5
#define THRESHOLD_F64 10e-10

void lu_kernel_fini(void);
static int *d_ipiv = NULL;     /* pivot record of one GETRF_PIVOT tile */
static void *d_work = NULL;    /* copy of one tile for the pivoting fallback */
static size_t work_bytes = 0;
static int ipiv_cap = 0;

#define CHECK_LAUNCH(rc)                                                                                          \
    do {                                                                                                          \
        int _rc = (rc);                                                                                           \
        if (_rc != 0) STARPU_ABORT_MSG("GB300 kernel launch failed (%d): %s", _rc, starpu_gb300_last_error());   \
    } while (0)

#define IS_F64(d) (STARPU_MATRIX_GET_ELEMSIZE(d) == sizeof(double))

static void lu_gb300_getrf(void *descr[], void *arg)
{
    (void)arg;
    void *a = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    const int n = (int)STARPU_MATRIX_GET_NX(descr[0]), ld = (int)STARPU_MATRIX_GET_LD(descr[0]);
    void *s = starpu_cuda_get_local_stream();
    if (IS_F64(descr[0]))
        CHECK_LAUNCH(starpu_gb300_dgetrf_tile(s, n, a, ld, NULL));
    else
        CHECK_LAUNCH(starpu_gb300_sgetrf_tile(s, n, a, ld, NULL));
}

static void lu_gb300_getrf_pivot(void *descr[], void *arg)
{
    struct piv_s *piv = arg;
    void *a = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    const int n = (int)STARPU_MATRIX_GET_NX(descr[0]), ld = (int)STARPU_MATRIX_GET_LD(descr[0]);
    const int f64 = IS_F64(descr[0]);
    void *s = starpu_cuda_get_local_stream();
    const size_t need = f64 ? starpu_gb300_dgetrf_pivot_tile_workspace(n) : starpu_gb300_sgetrf_pivot_tile_workspace(n);
    if (!d_work || need > work_bytes || n > ipiv_cap) {
        /* xlu_implicit_pivot.c calls no lu_kernel_init (only xlu.c and
         * xlu_implicit.c do), so the first pivoting tile sizes the workspace.
         * This codelet synchronises its stream anyway (it fills the host pivot
         * record), so no earlier use of the buffers is still in flight. */
        lu_kernel_fini();
        work_bytes = starpu_gb300_dgetrf_pivot_tile_workspace(n);
        ipiv_cap = n;
        d_work = starpu_gb300_device_malloc(work_bytes);
        d_ipiv = starpu_gb300_device_malloc(sizeof(int) * (size_t)n);
        STARPU_ASSERT_MSG(d_work && d_ipiv, "cannot allocate the LU pivoting workspace for tiles of order %d", n);
    }
    if (f64)
        CHECK_LAUNCH(starpu_gb300_dgetrf_pivot_tile(s, n, a, ld, THRESHOLD_F64, d_ipiv, d_work, work_bytes, NULL));
    else
        CHECK_LAUNCH(starpu_gb300_sgetrf_pivot_tile(s, n, a, ld, (float)THRESHOLD_F32, d_ipiv, d_work, work_bytes,
                                                     NULL));
    int *h = malloc(sizeof(int) * (size_t)n);
    STARPU_ASSERT(h);
    CHECK_LAUNCH(starpu_gb300_memcpy_d2h(s, h, d_ipiv, sizeof(int) * (size_t)n));
    CHECK_LAUNCH(starpu_gb300_stream_sync(s));
    /* the reference records a step only when it pivoted */
    for (int z = 0; z < n; ++z)
        if (h[z] >= 0) piv->piv[z + piv->first] = (unsigned)h[z] + piv->first;
    free(h);
}

static void lu_gb300_pivot(void *descr[], void *arg)
{
    struct piv_s *piv = arg;
    void *a = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    const int m = (int)STARPU_MATRIX_GET_NX(descr[0]), n = (int)STARPU_MATRIX_GET_NY(descr[0]);
    const int ld = (int)STARPU_MATRIX_GET_LD(descr[0]);
    int *pairs = malloc(sizeof(int) * 2 * (size_t)m);
    STARPU_ASSERT(pairs);
    int np = 0;
    for (int r = 0; r < m; ++r) {
        const int rp = (int)(piv->piv[r + piv->first] - piv->first);
        if (rp != r) {
            pairs[2 * np] = r;
            pairs[2 * np + 1] = rp;
            ++np;
        }
    }
    void *s = starpu_cuda_get_local_stream();
    if (np) {
        if (IS_F64(descr[0]))
            CHECK_LAUNCH(starpu_gb300_dswap_columns_tile(s, m, n, a, ld, pairs, np));
        else
            CHECK_LAUNCH(starpu_gb300_sswap_columns_tile(s, m, n, a, ld, pairs, np));
    }
    free(pairs);
}

/* sub12 <- L11^-1 sub12 (descr[0] = the diagonal tile, descr[1] = sub12) */
static void lu_gb300_trsm_ll(void *descr[], void *arg)
{
    (void)arg;
    void *l = (void *)STARPU_MATRIX_GET_PTR(descr[0]), *b = (void *)STARPU_MATRIX_GET_PTR(descr[1]);
    const int ldl = (int)STARPU_MATRIX_GET_LD(descr[0]), ldb = (int)STARPU_MATRIX_GET_LD(descr[1]);
    const int m = (int)STARPU_MATRIX_GET_NX(descr[1]), n = (int)STARPU_MATRIX_GET_NY(descr[1]);
    void *s = starpu_cuda_get_local_stream();
    if (IS_F64(descr[1]))
        CHECK_LAUNCH(starpu_gb300_dtrsm_llnn_tile(s, m, n, l, ldl, b, ldb));
    else
        CHECK_LAUNCH(starpu_gb300_strsm_llnn_tile(s, m, n, l, ldl, b, ldb));
}

/* sub21 <- sub21 U11^-1 (descr[0] = the diagonal tile, descr[1] = sub21) */
static void lu_gb300_trsm_ru(void *descr[], void *arg)
{
    (void)arg;
    void *u = (void *)STARPU_MATRIX_GET_PTR(descr[0]), *b = (void *)STARPU_MATRIX_GET_PTR(descr[1]);
    const int ldu = (int)STARPU_MATRIX_GET_LD(descr[0]), ldb = (int)STARPU_MATRIX_GET_LD(descr[1]);
    const int m = (int)STARPU_MATRIX_GET_NX(descr[1]), n = (int)STARPU_MATRIX_GET_NY(descr[1]);
    void *s = starpu_cuda_get_local_stream();
    if (IS_F64(descr[1]))
        CHECK_LAUNCH(starpu_gb300_dtrsm_runu_tile(s, m, n, u, ldu, b, ldb));
    else
        CHECK_LAUNCH(starpu_gb300_strsm_runu_tile(s, m, n, u, ldu, b, ldb));
}

/* center -= descr[0] * descr[1] */
static void lu_gb300_gemm(void *descr[], void *arg)
{
    (void)arg;
    void *a = (void *)STARPU_MATRIX_GET_PTR(descr[0]), *b = (void *)STARPU_MATRIX_GET_PTR(descr[1]);
    void *c = (void *)STARPU_MATRIX_GET_PTR(descr[2]);
    const int m = (int)STARPU_MATRIX_GET_NX(descr[2]), n = (int)STARPU_MATRIX_GET_NY(descr[2]);
    const int k = (int)STARPU_MATRIX_GET_NY(descr[0]);
    const int lda = (int)STARPU_MATRIX_GET_LD(descr[0]), ldb = (int)STARPU_MATRIX_GET_LD(descr[1]);
    const int ldc = (int)STARPU_MATRIX_GET_LD(descr[2]);
    void *s = starpu_cuda_get_local_stream();
    if (IS_F64(descr[2]))
        CHECK_LAUNCH(starpu_gb300_dgemm_nn_tile(s, m, n, k, -1.0, a, lda, b, ldb, 1.0, c, ldc));
    else
        CHECK_LAUNCH(starpu_gb300_sgemm_nn_tile(s, m, n, k, -1.0f, a, lda, b, ldb, 1.0f, c, ldc));
}

static struct starpu_perfmodel model_getrf = {.type = STARPU_HISTORY_BASED, .symbol = "lu_gb300_model_getrf"};
static struct starpu_perfmodel model_getrf_pivot = {.type = STARPU_HISTORY_BASED,
                                                    .symbol = "lu_gb300_model_getrf_pivot"};
static struct starpu_perfmodel model_trsm_ll = {.type = STARPU_HISTORY_BASED, .symbol = "lu_gb300_model_trsm_ll"};
static struct starpu_perfmodel model_trsm_ru = {.type = STARPU_HISTORY_BASED, .symbol = "lu_gb300_model_trsm_ru"};
static struct starpu_perfmodel model_gemm = {.type = STARPU_HISTORY_BASED, .symbol = "lu_gb300_model_gemm"};
static struct starpu_perfmodel model_pivot = {.type = STARPU_HISTORY_BASED, .symbol = "lu_gb300_model_pivot"};

struct starpu_codelet cl_getrf = {
    .where = STARPU_CUDA,
    .cuda_funcs = {lu_gb300_getrf},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 1,
    .modes = {STARPU_RW},
    .model = &model_getrf,
    .name = "lu_gb300_getrf",
};
struct starpu_codelet cl_getrf_pivot = {
    .where = STARPU_CUDA,
    .cuda_funcs = {lu_gb300_getrf_pivot},
    .nbuffers = 1,
    .modes = {STARPU_RW},
    .model = &model_getrf_pivot,
    .name = "lu_gb300_getrf_pivot",
};
struct starpu_codelet cl_trsm_ll = {
    .where = STARPU_CUDA,
    .cuda_funcs = {lu_gb300_trsm_ll},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 2,
    .modes = {STARPU_R, STARPU_RW},
    .model = &model_trsm_ll,
    .name = "lu_gb300_trsm_ll",
};
struct starpu_codelet cl_trsm_ru = {
    .where = STARPU_CUDA,
    .cuda_funcs = {lu_gb300_trsm_ru},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 2,
    .modes = {STARPU_R, STARPU_RW},
    .model = &model_trsm_ru,
    .name = "lu_gb300_trsm_ru",
};
struct starpu_codelet cl_gemm = {
    .where = STARPU_CUDA,
    .cuda_funcs = {lu_gb300_gemm},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 3,
    .modes = {STARPU_R, STARPU_R, STARPU_RW},
    .model = &model_gemm,
    .name = "lu_gb300_gemm",
};
struct starpu_codelet cl_pivot = {
    .where = STARPU_CUDA,
    .cuda_funcs = {lu_gb300_pivot},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 1,
    .modes = {STARPU_RW},
    .model = &model_pivot,
    .name = "lu_gb300_pivot",
};

/* nb: the tile order the driver will use (xlu*.c call it with size / nblocks) */
void lu_kernel_init(int nb)
{
    if (!starpu_cuda_worker_get_count() || nb <= 0) return;
    work_bytes = starpu_gb300_dgetrf_pivot_tile_workspace(nb);
    ipiv_cap = nb;
    d_work = starpu_gb300_device_malloc(work_bytes);
    d_ipiv = starpu_gb300_device_malloc(sizeof(int) * (size_t)nb);
    STARPU_ASSERT_MSG(d_work && d_ipiv, "cannot allocate the LU codelet workspace");
}

void lu_kernel_fini(void)
{
    if (d_work) starpu_gb300_device_free(d_work);
    if (d_ipiv) starpu_gb300_device_free(d_ipiv);
    d_work = NULL;
    d_ipiv = NULL;
    work_bytes = 0;
    ipiv_cap = 0;
}
