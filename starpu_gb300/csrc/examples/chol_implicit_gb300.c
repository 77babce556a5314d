/*
 * chol_implicit_gb300 -- tiled Cholesky through the StarPU API on the GB300
 * runtime, with implicit data dependencies: the right-looking task loop of
 * examples/cholesky/cholesky_implicit.c:244-318 (POTRF k; TRSM m>k; SYRK n>k;
 * GEMM m>n>k) over the tiles made by starpu_matrix_filter_block +
 * starpu_matrix_filter_vertical_block, written for this project so the GPU
 * path can run where the reference sources are not available.
 *
 *   chol_implicit_gb300 [-size N] [-nblocks NB] [-double] [-niter K] [-check] [-no-prio] [-break P]
 *
 * -break P makes the input indefinite (A_PP = -1): the run must end with
 * status 2 and report the failing leading minor instead of faulting.
 *
 * Input: A_mn = 1/(1+m+n) + N delta_mn (the reference driver's input).
 * Output on stdout, like the reference: "# size\tms\tGFlops" then one line.
 * -check: per-element relative error of L L^T against A must be <= 1e-4
 * (FP32) / 1e-12 (FP64); exit status 1 otherwise.  Exit 77 if no worker can
 * run the codelets (no GPU).
 */
#include <math.h>
#include <starpu.h>

#include "starpu_gb300_chol.h"

extern struct starpu_codelet cl_potrf, cl_trsm, cl_syrk, cl_gemm;
void cholesky_kernel_init(int nb);
void cholesky_kernel_fini(void);

static double flops_potrf(double n)
{
    /* FLOPS_SPOTRF of examples/cholesky/cholesky.h:95-98 */
    double fmuls = n * (((1. / 6.) * n + 0.5) * n + (1. / 3.));
    double fadds = n * (((1. / 6.) * n) * n - (1. / 6.));
    return fmuls + fadds;
}

static int run(void *mat, unsigned n, unsigned nblocks, size_t es, int noprio, double *ms)
{
    starpu_data_handle_t A;
    starpu_matrix_data_register(&A, STARPU_MAIN_RAM, (uintptr_t)mat, n, n, n, es);
    struct starpu_data_filter rows = {.filter_func = starpu_matrix_filter_block, .nchildren = nblocks};
    struct starpu_data_filter cols = {.filter_func = starpu_matrix_filter_vertical_block, .nchildren = nblocks};
    starpu_data_map_filters(A, 2, &rows, &cols);
    cholesky_kernel_init((int)(n / nblocks));
    double t0 = starpu_timing_now();
    int ret = 0;
    for (unsigned k = 0; k < nblocks && !ret; ++k) {
        starpu_data_handle_t akk = starpu_data_get_sub_data(A, 2, k, k);
        ret = starpu_task_insert(&cl_potrf, STARPU_PRIORITY, noprio ? 0 : (int)(2 * nblocks - 2 * k), STARPU_RW, akk,
                                 STARPU_NAME, "POTRF", 0);
        for (unsigned m = k + 1; m < nblocks && !ret; ++m)
            ret = starpu_task_insert(&cl_trsm, STARPU_PRIORITY, noprio ? 0 : (int)(2 * nblocks - 2 * k - m), STARPU_R,
                                     akk, STARPU_RW, starpu_data_get_sub_data(A, 2, m, k), STARPU_NAME, "TRSM", 0);
        for (unsigned j = k + 1; j < nblocks && !ret; ++j) {
            starpu_data_handle_t ajk = starpu_data_get_sub_data(A, 2, j, k);
            ret = starpu_task_insert(&cl_syrk, STARPU_PRIORITY, noprio ? 0 : (int)(2 * nblocks - 2 * k - j), STARPU_R,
                                     ajk, STARPU_RW, starpu_data_get_sub_data(A, 2, j, j), STARPU_NAME, "SYRK", 0);
            for (unsigned m = j + 1; m < nblocks && !ret; ++m)
                ret = starpu_task_insert(&cl_gemm, STARPU_PRIORITY,
                                         noprio ? 0 : (int)(2 * nblocks - 2 * k - m - j), STARPU_R,
                                         starpu_data_get_sub_data(A, 2, m, k), STARPU_R, ajk, STARPU_RW,
                                         starpu_data_get_sub_data(A, 2, m, j), STARPU_NAME, "GEMM", 0);
        }
    }
    starpu_task_wait_for_all();
    *ms = (starpu_timing_now() - t0) / 1e3;
    cholesky_kernel_fini();
    starpu_data_unpartition(A, STARPU_MAIN_RAM);
    starpu_data_unregister(A);
    return ret;
}

int main(int argc, char **argv)
{
    unsigned n = 2048, nblocks = 8;
    int dbl = 0, check = 0, niter = 1, noprio = 0, brk = -1;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "-size") && i + 1 < argc) n = (unsigned)atoi(argv[++i]);
        else if (!strcmp(argv[i], "-nblocks") && i + 1 < argc) nblocks = (unsigned)atoi(argv[++i]);
        else if (!strcmp(argv[i], "-niter") && i + 1 < argc) niter = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-double")) dbl = 1;
        else if (!strcmp(argv[i], "-check")) check = 1;
        else if (!strcmp(argv[i], "-no-prio")) noprio = 1;
        else if (!strcmp(argv[i], "-break") && i + 1 < argc) brk = atoi(argv[++i]);
        else {
            fprintf(stderr, "usage: %s [-size N] [-nblocks NB] [-double] [-niter K] [-check] [-no-prio]\n", argv[0]);
            return 0;
        }
    }
    int ret = starpu_init(NULL);
    if (ret == -ENODEV) return 77;
    STARPU_CHECK_RETURN_VALUE(ret, "starpu_init");
    starpu_cublas_init();
    const size_t es = dbl ? sizeof(double) : sizeof(float);
    void *mat = NULL;
    starpu_malloc_flags(&mat, (size_t)n * n * es, STARPU_MALLOC_PINNED);
    int status = 0;
    double best = 1e300;
    for (int it = 0; it < niter && !status; ++it) {
        for (size_t j = 0; j < n; ++j)
            for (size_t i = 0; i < n; ++i) {
                double v = 1.0 / (1.0 + (double)i + (double)j) + (i == j ? (double)n : 0.0);
                if (dbl) ((double *)mat)[i + j * n] = v;
                else ((float *)mat)[i + j * n] = (float)(1.0f / (1.0f + i + j)) + (i == j ? 1.0f * n : 0.0f);
            }
        if (brk >= 0 && (unsigned)brk < n) { /* make the input indefinite at pivot brk */
            if (dbl) ((double *)mat)[brk + (size_t)brk * n] = -1.0;
            else ((float *)mat)[brk + (size_t)brk * n] = -1.0f;
        }
        double ms = 0;
        ret = run(mat, n, nblocks, es, noprio, &ms);
        if (ret == -ENODEV) {
            starpu_free_flags(mat, (size_t)n * n * es, STARPU_MALLOC_PINNED);
            starpu_shutdown();
            return 77;
        }
        STARPU_CHECK_RETURN_VALUE(ret, "starpu_task_insert");
        if (ms < best) best = ms;
        int info = starpu_gb300_chol_status(1);
        if (info) {
            fprintf(stderr, "factorisation failed: leading minor %d is not positive definite\n", info);
            status = 2;
        }
    }
    printf("# size\tms\tGFlops\n%u\t%.0f\t%.1f\n", n, best, flops_potrf(n) / (best * 1e-3) / 1e9);
    struct starpu_gb300_runtime_stats st;
    starpu_gb300_runtime_get_stats(&st);
    fprintf(stderr, "# tasks cpu=%lu cuda=%lu graph=%lu graphs=%lu build_ms=%.2f exec_ms=%.2f h2d=%lu d2h=%lu\n",
            st.tasks_cpu, st.tasks_cuda, st.tasks_graph, st.graphs_launched, st.graph_build_us / 1e3,
            st.graph_exec_us / 1e3, st.h2d_bytes, st.d2h_bytes);
    if (check && !status) {
        double tol = dbl ? 1e-12 : 1e-4, worst = 0;
        for (size_t j = 0; j < n; ++j)
            for (size_t i = j; i < n; ++i) {
                double s = 0;
                for (size_t p = 0; p <= j; ++p) {
                    double a = dbl ? ((double *)mat)[i + p * n] : ((float *)mat)[i + p * n];
                    double b = dbl ? ((double *)mat)[j + p * n] : ((float *)mat)[j + p * n];
                    s += a * b;
                }
                double orig = 1.0 / (1.0 + (double)i + (double)j) + (i == j ? (double)n : 0.0);
                double e = fabs(s - orig) / orig;
                if (e > worst) worst = e;
            }
        fprintf(stderr, "check: max relative error %.3e (tolerance %.0e)\n", worst, tol);
        if (worst > tol) status = 1;
    }
    starpu_free_flags(mat, (size_t)n * n * es, STARPU_MALLOC_PINNED);
    starpu_cublas_shutdown();
    starpu_shutdown();
    return status;
}
