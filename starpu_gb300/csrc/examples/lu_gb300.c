/*
 * Tiled LU through the StarPU-API runtime with the GB300 LU codelets
 * (libstarpu_gb300_lu.so): the DAG of examples/lu/xlu_implicit.c:146-185 and,
 * with -piv, of xlu_implicit_pivot.c:165-210 (GETRF_PIVOT of the diagonal
 * tile, the column swaps of the other tiles of its block column, the two
 * TRSMs and the GEMM updates), implicit data dependencies, the reference's
 * bottom-level priorities.  One deliberate difference: each PIVOT task also
 * reads the diagonal tile, so it runs after the GETRF_PIVOT that writes its
 * pivot record (the reference's tasks have no dependency on it).
 *
 *   lu_gb300 [-size n] [-nblocks b] [-double] [-piv] [-check] [-seed s] [-niter k] [-small-pivots]
 *
 * Input as the reference driver (lu_example.c:221-233): a_ij uniform [0, 1),
 * a_ii = (a_ii + 1) * n.  -small-pivots zeroes row i up to and including the
 * diagonal for i = 5, 102, 199, ... (i mod 97 = 5): every term of that step's
 * eliminated pivot is then a product with an exact zero, so the pivot is
 * exactly 0 in either precision and the step must pivot (a zero diagonal
 * entry alone leaves a pivot near -0.8 / n, above both thresholds).  -check: || A P v - L (U v) || / (||A|| ||v|| n) for
 * random v (P the recorded column swaps), must be <= 1e-4 (the reference's
 * PIVOT_THRESHHOLD bound on ||PA - LU|| / (||A|| n)).  Prints "n ms GFlop/s"
 * (flops 2 n^3 / 3).  Exit 77 without a CUDA worker, 1 on a failed check.
 */
#include <math.h>
#include <starpu.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern struct starpu_codelet cl_getrf, cl_getrf_pivot, cl_trsm_ll, cl_trsm_ru, cl_gemm, cl_pivot;
void lu_kernel_init(int nb);
void lu_kernel_fini(void);

struct piv_s {
    unsigned *piv;
    unsigned first;
    unsigned last;
};

static unsigned n = 2048, nblocks = 8, check = 0, pivot = 0, is_double = 0, small_pivots = 0, niter = 1;
static long seed = 1;

static starpu_data_handle_t tile(starpu_data_handle_t A, unsigned row, unsigned col)
{
    /* first filter: column blocks, second: row blocks (xlu_implicit.c:250-262) */
    return starpu_data_get_sub_data(A, 2, col, row);
}

static void submit(struct starpu_codelet *cl, int prio, void *arg, int nh, starpu_data_handle_t h0,
                   starpu_data_handle_t h1, starpu_data_handle_t h2)
{
    struct starpu_task *t = starpu_task_create();
    t->cl = cl;
    t->cl_arg = arg;
    t->priority = prio;
    starpu_data_handle_t hs[3] = {h0, h1, h2};
    for (int i = 0; i < nh; ++i) t->handles[i] = hs[i];
    int ret = starpu_task_submit(t);
    if (ret == -ENODEV) {
        fprintf(stderr, "no worker can run the GB300 LU codelets\n");
        exit(77);
    }
    STARPU_CHECK_RETURN_VALUE(ret, "starpu_task_submit");
}

/* R access to the diagonal tile orders PIVOT after GETRF_PIVOT */
static struct starpu_codelet cl_pivot_after_getrf;

static double factorise(void *A, unsigned *ipiv)
{
    starpu_data_handle_t dA;
    const size_t es = is_double ? sizeof(double) : sizeof(float);
    starpu_matrix_data_register(&dA, STARPU_MAIN_RAM, (uintptr_t)A, n, n, n, es);
    struct starpu_data_filter fv = {.filter_func = starpu_matrix_filter_vertical_block, .nchildren = nblocks};
    struct starpu_data_filter fb = {.filter_func = starpu_matrix_filter_block, .nchildren = nblocks};
    starpu_data_map_filters(dA, 2, &fv, &fb);
    struct piv_s *pd = calloc(nblocks, sizeof *pd);
    for (unsigned b = 0; b < nblocks; ++b) {
        pd[b].piv = ipiv;
        pd[b].first = b * (n / nblocks);
        pd[b].last = (b + 1) * (n / nblocks);
    }
    const double t0 = starpu_timing_now();
    const int B = (int)nblocks;
    for (unsigned k = 0; k < nblocks; ++k) {
        starpu_data_handle_t dkk = tile(dA, k, k);
        if (pivot) {
            submit(&cl_getrf_pivot, 3 * B - 3 * (int)k, &pd[k], 1, dkk, NULL, NULL);
            for (unsigned i = 0; i < nblocks; ++i)
                if (i != k) submit(&cl_pivot_after_getrf, 3 * B - (2 * (int)k + (int)i), &pd[k], 2, tile(dA, i, k), dkk, NULL);
        } else {
            submit(&cl_getrf, 3 * B - 3 * (int)k, NULL, 1, dkk, NULL, NULL);
        }
        for (unsigned i = k + 1; i < nblocks; ++i) {
            submit(&cl_trsm_ll, 3 * B - (2 * (int)k + (int)i), NULL, 2, dkk, tile(dA, k, i), NULL);
            submit(&cl_trsm_ru, 3 * B - (2 * (int)k + (int)i), NULL, 2, dkk, tile(dA, i, k), NULL);
        }
        for (unsigned i = k + 1; i < nblocks; ++i)
            for (unsigned j = k + 1; j < nblocks; ++j)
                submit(&cl_gemm, 3 * B - ((int)k + (int)i + (int)j), NULL, 3, tile(dA, i, k), tile(dA, k, j),
                       tile(dA, i, j));
    }
    starpu_task_wait_for_all();
    const double t1 = starpu_timing_now();
    starpu_data_unpartition(dA, STARPU_MAIN_RAM);
    starpu_data_unregister(dA);
    free(pd);
    return (t1 - t0) / 1000.0;
}

#define ELEM(M, i, j) (is_double ? ((double *)(M))[(size_t)(i) + (size_t)(j) * n] : (double)((float *)(M))[(size_t)(i) + (size_t)(j) * n])

static double check_factor(const void *A0, const void *LU, const unsigned *ipiv)
{
    /* column swaps of the pivot record, in order (lu_example.c, pivot_saved_matrix) */
    unsigned *perm = malloc(sizeof(unsigned) * n);
    for (unsigned c = 0; c < n; ++c) perm[c] = c;
    for (unsigned k = 0; k < n; ++k)
        if (ipiv[k] != k) {
            unsigned t = perm[k];
            perm[k] = perm[ipiv[k]];
            perm[ipiv[k]] = t;
        }
    double *v = malloc(sizeof(double) * n), *u = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n);
    double worst = 0.0, anorm = 0.0;
    for (unsigned j = 0; j < n; ++j)
        for (unsigned i = 0; i < n; ++i) anorm = fmax(anorm, fabs(ELEM(A0, i, j)));
    srand48(seed + 7);
    for (int probe = 0; probe < 3; ++probe) {
        double vn = 0.0;
        for (unsigned i = 0; i < n; ++i) v[i] = drand48() - 0.5, vn = fmax(vn, fabs(v[i]));
        /* r = A P v: column c of A P is column perm[c] of A */
        for (unsigned i = 0; i < n; ++i) r[i] = 0.0;
        for (unsigned c = 0; c < n; ++c)
            for (unsigned i = 0; i < n; ++i) r[i] += ELEM(A0, i, perm[c]) * v[c];
        /* u = U v (unit upper), then r -= L u (lower with diagonal) */
        for (unsigned i = 0; i < n; ++i) u[i] = v[i];
        for (unsigned c = 0; c < n; ++c)
            for (unsigned i = 0; i < c; ++i) u[i] += ELEM(LU, i, c) * v[c];
        for (unsigned c = 0; c < n; ++c)
            for (unsigned i = c; i < n; ++i) r[i] -= ELEM(LU, i, c) * u[c];
        double rn = 0.0;
        for (unsigned i = 0; i < n; ++i) rn = fmax(rn, fabs(r[i]));
        worst = fmax(worst, rn / (anorm * vn * n));
    }
    free(perm);
    free(v);
    free(u);
    free(r);
    return worst;
}

int main(int argc, char **argv)
{
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "-size") && i + 1 < argc) n = (unsigned)atoi(argv[++i]);
        else if (!strcmp(argv[i], "-nblocks") && i + 1 < argc) nblocks = (unsigned)atoi(argv[++i]);
        else if (!strcmp(argv[i], "-seed") && i + 1 < argc) seed = atol(argv[++i]);
        else if (!strcmp(argv[i], "-niter") && i + 1 < argc) niter = (unsigned)atoi(argv[++i]);
        else if (!strcmp(argv[i], "-double")) is_double = 1;
        else if (!strcmp(argv[i], "-piv")) pivot = 1;
        else if (!strcmp(argv[i], "-check")) check = 1;
        else if (!strcmp(argv[i], "-small-pivots")) small_pivots = 1;
    }
    if (n % nblocks) {
        fprintf(stderr, "size must be a multiple of nblocks (square tiles, as the reference LU assumes)\n");
        return 2;
    }
    cl_pivot_after_getrf = cl_pivot;
    cl_pivot_after_getrf.nbuffers = 2;
    cl_pivot_after_getrf.modes[0] = STARPU_RW;
    cl_pivot_after_getrf.modes[1] = STARPU_R;
    int ret = starpu_init(NULL);
    if (ret == -ENODEV) return 77;
    STARPU_CHECK_RETURN_VALUE(ret, "starpu_init");
    if (starpu_cuda_worker_get_count() == 0) {
        fprintf(stderr, "no CUDA worker: the GB300 LU codelets need one\n");
        starpu_shutdown();
        return 77;
    }
    const size_t es = is_double ? sizeof(double) : sizeof(float);
    void *A = NULL, *A0 = malloc(es * (size_t)n * n);
    starpu_malloc_flags(&A, es * (size_t)n * n, STARPU_MALLOC_PINNED);
    unsigned *ipiv = malloc(sizeof(unsigned) * n);
    lu_kernel_init((int)(n / nblocks));
    int bad = 0;
    double best = 1e300;
    for (unsigned it = 0; it < niter; ++it) {
        srand48(seed);
        for (unsigned j = 0; j < n; ++j)
            for (unsigned i = 0; i < n; ++i) {
                double v = drand48();
                if (i == j) v = (v + 1.0) * n;
                if (small_pivots && j <= i && (i % 97 == 5)) v = 0.0;
                if (is_double) ((double *)A)[(size_t)i + (size_t)j * n] = v;
                else ((float *)A)[(size_t)i + (size_t)j * n] = (float)v;
            }
        memcpy(A0, A, es * (size_t)n * n);
        for (unsigned i = 0; i < n; ++i) ipiv[i] = i;
        const double ms = factorise(A, ipiv);
        if (ms < best) best = ms;
        if (check) {
            const double e = check_factor(A0, A, ipiv);
            unsigned swaps = 0;
            for (unsigned i = 0; i < n; ++i) swaps += ipiv[i] != i;
            fprintf(stderr, "||A P - L U|| / (||A|| n) : %e (%u pivoting steps)\n", e, swaps);
            if (!(e <= 1e-4)) bad = 1;
        }
    }
    const double flop = 2.0 * (double)n * n * n / 3.0;
    printf("# size\tms\tGFlop/s\n%u\t%.1f\t%.1f\n", n, best, flop / best / 1e6);
    struct starpu_gb300_runtime_stats st;
    starpu_gb300_runtime_get_stats(&st);
    fprintf(stderr, "# tasks cpu=%lu cuda=%lu graph=%lu graphs=%lu\n", st.tasks_cpu, st.tasks_cuda, st.tasks_graph,
            st.graphs_launched);
    lu_kernel_fini();
    starpu_free_flags(A, es * (size_t)n * n, STARPU_MALLOC_PINNED);
    free(A0);
    free(ipiv);
    starpu_shutdown();
    return bad;
}
