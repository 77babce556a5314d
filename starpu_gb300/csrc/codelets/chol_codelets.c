/*
 * The four tile codelets of the tiled Cholesky for the GB300 CUDA worker --
 * the drop-in replacement of examples/cholesky/cholesky_kernels.c's CUDA
 * branches.  Same codelet names, buffer counts, access modes and history
 * perfmodel symbols (chol_model_potrf/trsm/syrk/gemm, :504-634), so the
 * unchanged cholesky_implicit.c links against them; each body calls the C-ABI
 * kernel that replaces the reference's vendor call on the worker's stream:
 *   GEMM  cublasSgemm(N,T)      :98  -> starpu_gb300_sgemm_nt_tile
 *   SYRK  cublasSsyrk(L,N)      :177 -> starpu_gb300_ssyrk_ln_tile
 *   TRSM  cublasStrsm(R,L,T,N)  :258 -> starpu_gb300_strsm_rltn_tile
 *   POTRF cusolverDnSpotrf(L)   :354 -> starpu_gb300_spotrf_tile
 * FP32 GEMM and SYRK tiles of order 1024 and more (STARPU_GB300_CHOL_TC_MIN)
 * run on the tensor cores (starpu_gb300_sgemm_nt_tile_tc: row-scaled FP16
 * splits, ~22 significant bits, FP32 accumulation); smaller tiles, FP64
 * tiles, and every tile when STARPU_GB300_CHOL_TC=0, on the CUDA-core
 * kernels.  (Measured at 16384^2 in 512-tiles: the tensor-core tiles take
 * 496 ms task by task against 701 ms, but 199 ms as one CUDA graph against
 * 147 ms -- eight concurrent 512-tile updates of 8 CTAs each leave the GPU
 * less busy than the CUDA-core tiles, which pack more CTAs per SM.)  The splits need a
 * workspace per concurrently running stream: cholesky_kernel_init allocates
 * 16 of them, for tiles up to the order it is given (plus a ragged margin);
 * a stream that finds none free, and a driver that calls no init, gets the
 * CUDA-core kernels.
 * All four are STARPU_CUDA_ASYNC (they only enqueue), which lets the runtime
 * record a whole factorisation as one CUDA graph.  The element size of the
 * registered matrix selects FP32 or FP64 kernels.  There are no cpu_funcs:
 * this library has no CPU fallback (a run with no CUDA worker gets -ENODEV
 * from starpu_task_insert, which the driver reports as "skipped").
 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include <starpu.h>

#include "starpu_gb300_chol.h"
#include "starpu_gb300_kernels.h"

starpu_data_handle_t scratch = NULL;
starpu_data_handle_t devInfo = NULL;

/* device status word of the POTRF tiles (LAPACK info of the first failing
 * pivot), readable with starpu_gb300_chol_status() */
static int *d_status = NULL;

/* tensor-core tile workspaces, one per stream the tasks run on */
#define TC_SLOTS 16
#define TC_MIN_TILE 256       /* smallest tile order the tensor-core path takes at all */
static int tc_min = 1024;      /* STARPU_GB300_CHOL_TC_MIN */
static struct {
    void *stream;
    void *work;
} tc_slot[TC_SLOTS];
static size_t tc_bytes = 0;
static int tc_max = 0;       /* largest tile order the workspaces hold */
static int *d_tcerr = NULL;  /* status word of the tensor-core updates (wait timeouts) */
static pthread_mutex_t tc_mu = PTHREAD_MUTEX_INITIALIZER;

/* the workspace of `stream` (assigned on first use), or NULL */
static void *tc_work_for(void *stream, int m, int n, int k)
{
    if (!tc_max || m < tc_min || n < tc_min || k < tc_min || m > tc_max || n > tc_max || k > tc_max) return NULL;
    void *w = NULL;
    pthread_mutex_lock(&tc_mu);
    for (int i = 0; i < TC_SLOTS && !w; ++i) {
        if (tc_slot[i].work && tc_slot[i].stream == stream) w = tc_slot[i].work;
        else if (tc_slot[i].work && !tc_slot[i].stream) {
            tc_slot[i].stream = stream;
            w = tc_slot[i].work;
        }
    }
    pthread_mutex_unlock(&tc_mu);
    return w;
}

#define CHECK_LAUNCH(rc)                                                                                \
    do {                                                                                                \
        int _rc = (rc);                                                                                 \
        if (_rc != 0) STARPU_ABORT_MSG("GB300 kernel launch failed (%d): %s", _rc, starpu_gb300_last_error()); \
    } while (0)

static void chol_gb300_codelet_update_gemm(void *descr[], void *arg)
{
    (void)arg;
    void *left = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    void *right = (void *)STARPU_MATRIX_GET_PTR(descr[1]);
    void *center = (void *)STARPU_MATRIX_GET_PTR(descr[2]);
    int dx = (int)STARPU_MATRIX_GET_NY(descr[2]);
    int dy = (int)STARPU_MATRIX_GET_NX(descr[2]);
    int dz = (int)STARPU_MATRIX_GET_NY(descr[0]);
    int ld21 = (int)STARPU_MATRIX_GET_LD(descr[0]), ld12 = (int)STARPU_MATRIX_GET_LD(descr[1]);
    int ld22 = (int)STARPU_MATRIX_GET_LD(descr[2]);
    void *s = starpu_cuda_get_local_stream();
    void *w = STARPU_MATRIX_GET_ELEMSIZE(descr[2]) == sizeof(float) ? tc_work_for(s, dy, dx, dz) : NULL;
    if (w)
        CHECK_LAUNCH(starpu_gb300_sgemm_nt_tile_tc(s, dy, dx, dz, left, ld21, right, ld12, center, ld22, 0, w, tc_bytes,
                                                   d_tcerr));
    else if (STARPU_MATRIX_GET_ELEMSIZE(descr[2]) == sizeof(double))
        CHECK_LAUNCH(starpu_gb300_dgemm_nt_tile(s, dy, dx, dz, -1.0, left, ld21, right, ld12, 1.0, center, ld22));
    else
        CHECK_LAUNCH(starpu_gb300_sgemm_nt_tile(s, dy, dx, dz, -1.0f, left, ld21, right, ld12, 1.0f, center, ld22));
}

static void chol_gb300_codelet_update_syrk(void *descr[], void *arg)
{
    (void)arg;
    void *left = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    void *center = (void *)STARPU_MATRIX_GET_PTR(descr[1]);
    int dx = (int)STARPU_MATRIX_GET_NY(descr[1]);
    int dz = (int)STARPU_MATRIX_GET_NY(descr[0]);
    int ld21 = (int)STARPU_MATRIX_GET_LD(descr[0]), ld22 = (int)STARPU_MATRIX_GET_LD(descr[1]);
    void *s = starpu_cuda_get_local_stream();
    void *w = STARPU_MATRIX_GET_ELEMSIZE(descr[1]) == sizeof(float) ? tc_work_for(s, dx, dx, dz) : NULL;
    if (w)
        CHECK_LAUNCH(starpu_gb300_sgemm_nt_tile_tc(s, dx, dx, dz, left, ld21, left, ld21, center, ld22, 1, w, tc_bytes,
                                                   d_tcerr));
    else if (STARPU_MATRIX_GET_ELEMSIZE(descr[1]) == sizeof(double))
        CHECK_LAUNCH(starpu_gb300_dsyrk_ln_tile(s, dx, dz, -1.0, left, ld21, 1.0, center, ld22));
    else
        CHECK_LAUNCH(starpu_gb300_ssyrk_ln_tile(s, dx, dz, -1.0f, left, ld21, 1.0f, center, ld22));
}

static void chol_gb300_codelet_update_trsm(void *descr[], void *arg)
{
    (void)arg;
    void *sub11 = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    void *sub21 = (void *)STARPU_MATRIX_GET_PTR(descr[1]);
    int ld11 = (int)STARPU_MATRIX_GET_LD(descr[0]), ld21 = (int)STARPU_MATRIX_GET_LD(descr[1]);
    int nx21 = (int)STARPU_MATRIX_GET_NY(descr[1]);
    int ny21 = (int)STARPU_MATRIX_GET_NX(descr[1]);
    void *s = starpu_cuda_get_local_stream();
    /* reference: strsm(R, L, T, N, m = rows of A21 (nx), n = cols (ny)) with the
     * StarPU naming nx21 = NY, ny21 = NX; the operation is A21 <- A21 L11^-T */
    if (STARPU_MATRIX_GET_ELEMSIZE(descr[1]) == sizeof(double))
        CHECK_LAUNCH(starpu_gb300_dtrsm_rltn_tile(s, ny21, nx21, 1.0, sub11, ld11, sub21, ld21));
    else
        CHECK_LAUNCH(starpu_gb300_strsm_rltn_tile(s, ny21, nx21, 1.0f, sub11, ld11, sub21, ld21));
}

static void chol_gb300_codelet_update_potrf(void *descr[], void *arg)
{
    (void)arg;
    void *sub11 = (void *)STARPU_MATRIX_GET_PTR(descr[0]);
    int nx = (int)STARPU_MATRIX_GET_NY(descr[0]);
    int ld = (int)STARPU_MATRIX_GET_LD(descr[0]);
    void *s = starpu_cuda_get_local_stream();
    /* the status word is not reset per tile: the first failing pivot is kept */
    if (STARPU_MATRIX_GET_ELEMSIZE(descr[0]) == sizeof(double))
        CHECK_LAUNCH(starpu_gb300_dpotrf_tile_status(s, nx, sub11, ld, d_status));
    else
        CHECK_LAUNCH(starpu_gb300_spotrf_tile_status(s, nx, sub11, ld, d_status));
}

struct starpu_perfmodel chol_model_potrf = {.type = STARPU_HISTORY_BASED, .symbol = "chol_model_potrf"};
struct starpu_perfmodel chol_model_trsm = {.type = STARPU_HISTORY_BASED, .symbol = "chol_model_trsm"};
struct starpu_perfmodel chol_model_syrk = {.type = STARPU_HISTORY_BASED, .symbol = "chol_model_syrk"};
struct starpu_perfmodel chol_model_gemm = {.type = STARPU_HISTORY_BASED, .symbol = "chol_model_gemm"};

struct starpu_codelet cl_potrf = {
    .type = STARPU_SEQ,
    .cuda_funcs = {chol_gb300_codelet_update_potrf},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 1,
    .modes = {STARPU_RW},
    .model = &chol_model_potrf,
    .name = "cl_POTRF",
    .color = 0xffff00,
};

struct starpu_codelet cl_trsm = {
    .type = STARPU_SEQ,
    .cuda_funcs = {chol_gb300_codelet_update_trsm},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 2,
    .modes = {STARPU_R, STARPU_RW},
    .model = &chol_model_trsm,
    .name = "cl_TRSM",
    .color = 0x8080ff,
};

struct starpu_codelet cl_syrk = {
    .type = STARPU_SEQ,
    .max_parallelism = INT_MAX,
    .cuda_funcs = {chol_gb300_codelet_update_syrk},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 2,
    .modes = {STARPU_R, STARPU_RW},
    .model = &chol_model_syrk,
    .name = "cl_SYRK",
    .color = 0x00ff00,
};

struct starpu_codelet cl_gemm = {
    .type = STARPU_SEQ,
    .max_parallelism = INT_MAX,
    .cuda_funcs = {chol_gb300_codelet_update_gemm},
    .cuda_flags = {STARPU_CUDA_ASYNC},
    .nbuffers = 3,
    .modes = {STARPU_R, STARPU_R, STARPU_RW},
    .model = &chol_model_gemm,
    .name = "cl_GEMM",
    .color = 0x00c000,
};

/* the GPU-only variants of the reference are the same codelets here */
struct starpu_codelet cl_potrf_gpu, cl_trsm_gpu, cl_syrk_gpu, cl_gemm_gpu;

void cholesky_kernel_init(int nb)
{
    cl_potrf_gpu = cl_potrf;
    cl_trsm_gpu = cl_trsm;
    cl_syrk_gpu = cl_syrk;
    cl_gemm_gpu = cl_gemm;
    if (starpu_cuda_worker_get_count() && !d_status) {
        d_status = (int *)starpu_gb300_device_malloc(sizeof(int));
        if (d_status) starpu_gb300_memset(NULL, d_status, 0, sizeof(int));
        starpu_gb300_stream_sync(NULL);
    }
    const char *e = getenv("STARPU_GB300_CHOL_TC"), *emin = getenv("STARPU_GB300_CHOL_TC_MIN");
    if (emin && atoi(emin) > 0) tc_min = atoi(emin) < TC_MIN_TILE ? TC_MIN_TILE : atoi(emin);
    if (starpu_cuda_worker_get_count() && !tc_max && nb + 1 >= tc_min && !(e && !strcmp(e, "0"))) {
        /* the filters give the first tiles one more row or column */
        const int nmax = nb + 1;
        tc_bytes = starpu_gb300_tile_tc_workspace(nmax);
        d_tcerr = (int *)starpu_gb300_device_malloc(sizeof(int));
        int ok = d_tcerr != NULL && starpu_gb300_tile_tc_prepare() == 0;
        if (ok) starpu_gb300_memset(NULL, d_tcerr, 0, sizeof(int));
        for (int i = 0; i < TC_SLOTS && ok; ++i) {
            tc_slot[i].stream = NULL;
            tc_slot[i].work = starpu_gb300_device_malloc(tc_bytes);
            ok = tc_slot[i].work != NULL;
        }
        starpu_gb300_stream_sync(NULL);
        if (ok) tc_max = nmax;
        else cholesky_kernel_fini();
    }
}

void cholesky_kernel_fini(void)
{
    starpu_task_wait_for_all();
    pthread_mutex_lock(&tc_mu);
    for (int i = 0; i < TC_SLOTS; ++i) {
        if (tc_slot[i].work) starpu_gb300_device_free(tc_slot[i].work);
        tc_slot[i].work = NULL;
        tc_slot[i].stream = NULL;
    }
    if (d_tcerr) starpu_gb300_device_free(d_tcerr);
    d_tcerr = NULL;
    tc_max = 0;
    tc_bytes = 0;
    pthread_mutex_unlock(&tc_mu);
}

/* LAPACK-style info of the first non-positive pivot met by the POTRF tiles
 * since the last reset (0 = every tile factored). */
int starpu_gb300_chol_status(int reset)
{
    int h = 0;
    if (!d_status) return 0;
    starpu_task_wait_for_all();
    starpu_gb300_memcpy_d2h(NULL, &h, d_status, sizeof h);
    starpu_gb300_stream_sync(NULL);
    if (reset) {
        starpu_gb300_memset(NULL, d_status, 0, sizeof(int));
        starpu_gb300_stream_sync(NULL);
    }
    return h;
}
