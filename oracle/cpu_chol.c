/*
 * ORACLE / CPU BASELINE -- test and benchmark infrastructure only.
 *
 * A port of StarPU's CPU path for the tiled Cholesky: the CPU branches of the
 * four tile codelets (examples/cholesky/cholesky_kernels.c:75 SGEMM(N,T),
 * :169 SSYRK(L,N), :254 STRSM(R,L,T,N), :329-342 the sqrt / SSCAL / SSYR
 * POTRF loop used when the BLAS is not MKL) calling a Fortran BLAS exactly as
 * examples/common/blas.c:240-427 does, executed over host threads in the task
 * order and with the base priorities of examples/cholesky/cholesky_implicit.c
 * (:125-213, :244-318).  One BLAS thread per worker, like StarPU CPU workers.
 *
 * The BLAS is scipy's bundled OpenBLAS, whose Fortran symbols carry a
 * `scipy_` prefix; cpu_chol_init() dlopen()s it and binds the entry points.
 * The FP64 variant is the same DAG with D-precision BLAS (there is no FP64
 * codelet in the reference); its diagonal tile uses LAPACK dpotrf.
 */
#include <dlfcn.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef void (*sgemm_t)(const char *, const char *, const int *, const int *, const int *, const float *, const float *,
                        const int *, const float *, const int *, const float *, float *, const int *);
typedef void (*dgemm_t)(const char *, const char *, const int *, const int *, const int *, const double *,
                        const double *, const int *, const double *, const int *, const double *, double *,
                        const int *);
typedef void (*ssyrk_t)(const char *, const char *, const int *, const int *, const float *, const float *,
                        const int *, const float *, float *, const int *);
typedef void (*dsyrk_t)(const char *, const char *, const int *, const int *, const double *, const double *,
                        const int *, const double *, double *, const int *);
typedef void (*strsm_t)(const char *, const char *, const char *, const char *, const int *, const int *,
                        const float *, const float *, const int *, float *, const int *);
typedef void (*dtrsm_t)(const char *, const char *, const char *, const char *, const int *, const int *,
                        const double *, const double *, const int *, double *, const int *);
typedef void (*sscal_t)(const int *, const float *, float *, const int *);
typedef void (*ssyr_t)(const char *, const int *, const float *, const float *, const int *, float *, const int *);
typedef void (*dpotrf_t)(const char *, const int *, double *, const int *, int *);
typedef void (*dpotrs_t)(const char *, const int *, const int *, const double *, const int *, double *, const int *,
                         int *);
typedef void (*setnt_t)(int);

static struct {
    void *h;
    sgemm_t sgemm;
    dgemm_t dgemm;
    ssyrk_t ssyrk;
    dsyrk_t dsyrk;
    strsm_t strsm;
    dtrsm_t dtrsm;
    sscal_t sscal;
    ssyr_t ssyr;
    dpotrf_t dpotrf;
    dpotrs_t dpotrs;
    setnt_t set_threads;
} B;

static void *sym(const char *name)
{
    char buf[128];
    snprintf(buf, sizeof buf, "scipy_%s", name);
    void *p = dlsym(B.h, buf);
    if (!p) p = dlsym(B.h, name);
    return p;
}

/* Bind the BLAS entry points from the shared library at `path`.  0 on success. */
int cpu_chol_init(const char *path)
{
    if (B.h) return 0;
    B.h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!B.h) return -1;
    B.sgemm = (sgemm_t)sym("sgemm_");
    B.dgemm = (dgemm_t)sym("dgemm_");
    B.ssyrk = (ssyrk_t)sym("ssyrk_");
    B.dsyrk = (dsyrk_t)sym("dsyrk_");
    B.strsm = (strsm_t)sym("strsm_");
    B.dtrsm = (dtrsm_t)sym("dtrsm_");
    B.sscal = (sscal_t)sym("sscal_");
    B.ssyr = (ssyr_t)sym("ssyr_");
    B.dpotrf = (dpotrf_t)sym("dpotrf_");
    B.dpotrs = (dpotrs_t)sym("dpotrs_");
    B.set_threads = (setnt_t)sym("openblas_set_num_threads");
    if (!B.sgemm || !B.dgemm || !B.ssyrk || !B.dsyrk || !B.strsm || !B.dtrsm || !B.sscal || !B.ssyr || !B.dpotrf ||
        !B.dpotrs)
        return -2;
    return 0;
}

void cpu_chol_set_blas_threads(int n)
{
    if (B.set_threads) B.set_threads(n);
}

/* ------------------------------------------------------------- tasks */

enum { T_POTRF, T_TRSM, T_SYRK, T_GEMM };

typedef struct task {
    int kind, k, m, n;
    int prio;
    int ndeps;       /* remaining predecessors */
    int nsucc, capsucc;
    int *succ;
} task_t;

typedef struct {
    int nb, n, lda, is64;
    void *A;
    int sz[512], off[512];
    task_t *tasks;
    int ntasks;
    /* ready heap ordered by priority (max first), ties by submission index */
    int *heap, hn;
    int done, failed;
    pthread_mutex_t mu;
    pthread_cond_t cv;
} dag_t;

static int heap_less(dag_t *d, int a, int b)
{
    task_t *ta = &d->tasks[a], *tb = &d->tasks[b];
    if (ta->prio != tb->prio) return ta->prio < tb->prio;
    return a > b;
}

static void heap_push(dag_t *d, int t)
{
    int i = d->hn++;
    d->heap[i] = t;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (!heap_less(d, d->heap[p], d->heap[i])) break;
        int x = d->heap[p]; d->heap[p] = d->heap[i]; d->heap[i] = x;
        i = p;
    }
}

static int heap_pop(dag_t *d)
{
    int top = d->heap[0];
    d->heap[0] = d->heap[--d->hn];
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, r = l + 1, b = i;
        if (l < d->hn && heap_less(d, d->heap[b], d->heap[l])) b = l;
        if (r < d->hn && heap_less(d, d->heap[b], d->heap[r])) b = r;
        if (b == i) break;
        int x = d->heap[b]; d->heap[b] = d->heap[i]; d->heap[i] = x;
        i = b;
    }
    return top;
}

#define AT(d, i, j) ((d)->is64 ? (void *)((double *)(d)->A + (size_t)(i) + (size_t)(j) * (d)->lda) \
                               : (void *)((float *)(d)->A + (size_t)(i) + (size_t)(j) * (d)->lda))

static int run_task(dag_t *d, task_t *t)
{
    const int lda = d->lda;
    if (t->kind == T_POTRF) {
        int nx = d->sz[t->k];
        if (d->is64) {
            int info = 0;
            B.dpotrf("L", &nx, (double *)AT(d, d->off[t->k], d->off[t->k]), &lda, &info);
            return info;
        }
        /* cholesky_kernels.c:329-342 */
        float *s = (float *)AT(d, d->off[t->k], d->off[t->k]);
        for (int z = 0; z < nx; z++) {
            float lambda = sqrtf(s[z + (size_t)z * lda]);
            s[z + (size_t)z * lda] = lambda;
            if (!(lambda > 0.0f)) return z + 1;
            int rem = nx - z - 1, one = 1;
            float inv = 1.0f / lambda, m1 = -1.0f;
            B.sscal(&rem, &inv, &s[(z + 1) + (size_t)z * lda], &one);
            B.ssyr("L", &rem, &m1, &s[(z + 1) + (size_t)z * lda], &one, &s[(z + 1) + (size_t)(z + 1) * lda], &lda);
        }
        return 0;
    }
    if (t->kind == T_TRSM) { /* STRSM("R","L","T","N", nx21, ny21, 1, sub11, ld, sub21, ld) */
        int mm = d->sz[t->m], nn = d->sz[t->k];
        if (d->is64) {
            double one = 1.0;
            B.dtrsm("R", "L", "T", "N", &mm, &nn, &one, (double *)AT(d, d->off[t->k], d->off[t->k]), &lda,
                    (double *)AT(d, d->off[t->m], d->off[t->k]), &lda);
        } else {
            float one = 1.0f;
            B.strsm("R", "L", "T", "N", &mm, &nn, &one, (float *)AT(d, d->off[t->k], d->off[t->k]), &lda,
                    (float *)AT(d, d->off[t->m], d->off[t->k]), &lda);
        }
        return 0;
    }
    if (t->kind == T_SYRK) { /* SSYRK("L","N", dx, dz, -1, A_nk, ld, 1, A_nn, ld) */
        int nn = d->sz[t->n], kk = d->sz[t->k];
        if (d->is64) {
            double m1 = -1.0, p1 = 1.0;
            B.dsyrk("L", "N", &nn, &kk, &m1, (double *)AT(d, d->off[t->n], d->off[t->k]), &lda, &p1,
                    (double *)AT(d, d->off[t->n], d->off[t->n]), &lda);
        } else {
            float m1 = -1.0f, p1 = 1.0f;
            B.ssyrk("L", "N", &nn, &kk, &m1, (float *)AT(d, d->off[t->n], d->off[t->k]), &lda, &p1,
                    (float *)AT(d, d->off[t->n], d->off[t->n]), &lda);
        }
        return 0;
    }
    /* SGEMM("N","T", dy, dx, dz, -1, A_mk, ld, A_nk, ld, 1, A_mn, ld) */
    int mm = d->sz[t->m], nn = d->sz[t->n], kk = d->sz[t->k];
    if (d->is64) {
        double m1 = -1.0, p1 = 1.0;
        B.dgemm("N", "T", &mm, &nn, &kk, &m1, (double *)AT(d, d->off[t->m], d->off[t->k]), &lda,
                (double *)AT(d, d->off[t->n], d->off[t->k]), &lda, &p1, (double *)AT(d, d->off[t->m], d->off[t->n]),
                &lda);
    } else {
        float m1 = -1.0f, p1 = 1.0f;
        B.sgemm("N", "T", &mm, &nn, &kk, &m1, (float *)AT(d, d->off[t->m], d->off[t->k]), &lda,
                (float *)AT(d, d->off[t->n], d->off[t->k]), &lda, &p1, (float *)AT(d, d->off[t->m], d->off[t->n]),
                &lda);
    }
    return 0;
}

static void *worker(void *arg)
{
    dag_t *d = (dag_t *)arg;
    pthread_mutex_lock(&d->mu);
    for (;;) {
        while (d->hn == 0 && d->done < d->ntasks && !d->failed) pthread_cond_wait(&d->cv, &d->mu);
        if (d->done >= d->ntasks || d->failed) break;
        int ti = heap_pop(d);
        pthread_mutex_unlock(&d->mu);
        int info = run_task(d, &d->tasks[ti]);
        pthread_mutex_lock(&d->mu);
        if (info) {
            d->failed = d->off[d->tasks[ti].k] + info;
            pthread_cond_broadcast(&d->cv);
            break;
        }
        d->done++;
        task_t *t = &d->tasks[ti];
        for (int s = 0; s < t->nsucc; s++) {
            task_t *u = &d->tasks[t->succ[s]];
            if (--u->ndeps == 0) heap_push(d, t->succ[s]);
        }
        pthread_cond_broadcast(&d->cv);
    }
    pthread_mutex_unlock(&d->mu);
    return NULL;
}

static void add_edge(dag_t *d, int from, int to)
{
    task_t *f = &d->tasks[from];
    if (f->nsucc == f->capsucc) {
        f->capsucc = f->capsucc ? 2 * f->capsucc : 4;
        f->succ = (int *)realloc(f->succ, sizeof(int) * f->capsucc);
    }
    f->succ[f->nsucc++] = to;
    d->tasks[to].ndeps++;
}

/* Tiled right-looking Cholesky of the lower part of A on `nthreads` host
 * threads.  The dependency edges are the ones StarPU's sequential-consistency
 * rule derives from the access modes of cholesky_implicit.c's insert loop:
 *   POTRF(k)    <- SYRK(k-1,k)
 *   TRSM(m,k)   <- POTRF(k), GEMM(k-1,m,k)
 *   SYRK(k,n)   <- TRSM(n,k), SYRK(k-1,n)
 *   GEMM(k,m,n) <- TRSM(m,k), TRSM(n,k), GEMM(k-1,m,n)
 * Returns 0 or the LAPACK-style info of a failed pivot. */
static int potrf_dag(void *A, int n, int lda, int nb, int nthreads, int is64)
{
    if (nb < 1 || nb > 512 || nb > n) return -1;
    dag_t *d = (dag_t *)calloc(1, sizeof(dag_t));
    d->nb = nb; d->n = n; d->lda = lda; d->is64 = is64; d->A = A;
    for (int b = 0; b < nb; b++) {
        int base = n / nb, rem = n % nb;
        d->sz[b] = base + (b < rem ? 1 : 0);
        d->off[b] = b * base + (b < rem ? b : rem);
    }
    size_t nt = (size_t)nb + (size_t)nb * nb + (size_t)nb * nb + (size_t)nb * nb * nb;
    d->tasks = (task_t *)calloc(nt, sizeof(task_t));
    d->heap = (int *)malloc(nt * sizeof(int));
    int *ip = (int *)malloc(sizeof(int) * nb);
    int *it = (int *)malloc(sizeof(int) * nb * nb);         /* TRSM(m,k)  -> [k*nb+m] */
    int *is = (int *)malloc(sizeof(int) * nb * nb);         /* SYRK(k,n)  -> [k*nb+n] */
    int *ig = (int *)malloc(sizeof(int) * nb * nb * nb);    /* GEMM(k,m,n)-> [(k*nb+m)*nb+n] */
    int cnt = 0;
    for (int k = 0; k < nb; k++) {
        task_t *t = &d->tasks[cnt]; ip[k] = cnt++;
        t->kind = T_POTRF; t->k = k; t->prio = 2 * nb - 2 * k;
        for (int m = k + 1; m < nb; m++) {
            t = &d->tasks[cnt]; it[k * nb + m] = cnt++;
            t->kind = T_TRSM; t->k = k; t->m = m; t->prio = 2 * nb - 2 * k - m;
        }
        for (int nn = k + 1; nn < nb; nn++) {
            t = &d->tasks[cnt]; is[k * nb + nn] = cnt++;
            t->kind = T_SYRK; t->k = k; t->n = nn; t->prio = 2 * nb - 2 * k - nn;
            for (int m = nn + 1; m < nb; m++) {
                t = &d->tasks[cnt]; ig[(k * nb + m) * nb + nn] = cnt++;
                t->kind = T_GEMM; t->k = k; t->m = m; t->n = nn; t->prio = 2 * nb - 2 * k - m - nn;
            }
        }
    }
    d->ntasks = cnt;
    for (int k = 0; k < nb; k++) {
        if (k > 0) add_edge(d, is[(k - 1) * nb + k], ip[k]);
        for (int m = k + 1; m < nb; m++) {
            add_edge(d, ip[k], it[k * nb + m]);
            if (k > 0) add_edge(d, ig[((k - 1) * nb + m) * nb + k], it[k * nb + m]);
        }
        for (int nn = k + 1; nn < nb; nn++) {
            add_edge(d, it[k * nb + nn], is[k * nb + nn]);
            if (k > 0) add_edge(d, is[(k - 1) * nb + nn], is[k * nb + nn]);
            for (int m = nn + 1; m < nb; m++) {
                int g = ig[(k * nb + m) * nb + nn];
                add_edge(d, it[k * nb + m], g);
                add_edge(d, it[k * nb + nn], g);
                if (k > 0) add_edge(d, ig[((k - 1) * nb + m) * nb + nn], g);
            }
        }
    }
    for (int i = 0; i < cnt; i++)
        if (d->tasks[i].ndeps == 0) heap_push(d, i);
    pthread_mutex_init(&d->mu, NULL);
    pthread_cond_init(&d->cv, NULL);
    if (B.set_threads) B.set_threads(1);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, worker, d);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    int ret = d->failed;
    pthread_mutex_destroy(&d->mu);
    pthread_cond_destroy(&d->cv);
    for (int i = 0; i < cnt; i++) free(d->tasks[i].succ);
    free(th); free(ip); free(it); free(is); free(ig);
    free(d->tasks); free(d->heap); free(d);
    return ret;
}

int cpu_chol_potrf_tiled_f32(int n, float *A, int lda, int nblocks, int nthreads)
{
    if (!B.h) return -100;
    return potrf_dag(A, n, lda, nblocks, nthreads, 0);
}

int cpu_chol_potrf_tiled_f64(int n, double *A, int lda, int nblocks, int nthreads)
{
    if (!B.h) return -100;
    return potrf_dag(A, n, lda, nblocks, nthreads, 1);
}

/* LAPACK dpotrs with `nthreads` BLAS threads. */
int cpu_chol_potrs_f64(int n, int nrhs, const double *L, int ldl, double *Bm, int ldb, int nthreads)
{
    if (!B.h) return -100;
    int info = 0;
    if (B.set_threads) B.set_threads(nthreads < 1 ? 1 : nthreads);
    B.dpotrs("L", &n, &nrhs, L, &ldl, Bm, &ldb, &info);
    if (B.set_threads) B.set_threads(1);
    return info;
}
