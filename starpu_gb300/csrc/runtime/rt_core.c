/*
 * Runtime core: configuration, initialisation / shutdown, worker
 * enumeration, scheduling contexts, memory allocation, timing, and the
 * no-op profiling / tracing / bound entry points that drivers call.
 *
 * Environment variables honoured (StarPU's names, src/core/workers.c:1170-1354):
 *   STARPU_NCPU, STARPU_NCUDA, STARPU_SCHED (dmda only), STARPU_CALIBRATE,
 *   STARPU_PERF_MODEL_DIR, STARPU_HOSTNAME, STARPU_CUDA_PIPELINE;
 * and STARPU_GB300_GRAPH=0/1 (whole-DAG CUDA graphs when every worker is a
 * CUDA worker; default 1).
 */
#define _GNU_SOURCE
#include <errno.h>
#include <stdarg.h>
#include <string.h>
#include <sched.h>
#include <time.h>
#include <unistd.h>

#include "rt_internal.h"

struct rt_state rt;

static __thread int tls_worker = -1;
static __thread struct starpu_task *tls_task = NULL;

void rt_lock(void) { pthread_mutex_lock(&rt.lock); }
void rt_unlock(void) { pthread_mutex_unlock(&rt.lock); }
int rt_current_worker(void) { return tls_worker; }
void rt_set_current_worker(int id) { tls_worker = id; }
struct starpu_task *rt_current_task_get(void) { return tls_task; }
void rt_current_task_set(struct starpu_task *t) { tls_task = t; }

void starpu_gb300_abort_msg(const char *file, int line, const char *func, const char *fmt, ...)
{
    va_list ap;
    fprintf(stderr, "[starpu_gb300][%s:%d %s] ", file, line, func);
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    fprintf(stderr, "\n");
    fflush(stderr);
    abort();
}

double starpu_timing_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec * 1e6 + (double)ts.tv_nsec * 1e-3;
}

static int env_int(const char *name, int dflt)
{
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    return atoi(v);
}

int starpu_conf_init(struct starpu_conf *conf)
{
    if (!conf) return -EINVAL;
    memset(conf, 0, sizeof *conf);
    conf->magic = 42;
    conf->ncpus = -1;
    conf->ncuda = -1;
    conf->nhip = 0;
    conf->nopencl = 0;
    conf->calibrate = -1;
    return 0;
}

int starpu_get_env_number(const char *str)
{
    const char *v = getenv(str);
    if (!v) return -1;
    char *end;
    const long n = strtol(v, &end, 10);
    if (*end || n < 0) starpu_gb300_abort_msg(__FILE__, __LINE__, __func__,
                                              "The %s environment variable must contain a non-negative integer", str);
    return (int)n;
}

void starpu_usleep(float nb_micro_sec)
{
    if (nb_micro_sec <= 0) return;
    struct timespec ts;
    ts.tv_sec = (time_t)(nb_micro_sec / 1e6f);
    ts.tv_nsec = (long)((nb_micro_sec - (float)ts.tv_sec * 1e6f) * 1e3f);
    if (ts.tv_nsec >= 1000000000L) ts.tv_nsec = 999999999L;
    while (nanosleep(&ts, &ts) != 0 && errno == EINTR) {
    }
}

void starpu_sleep(float nb_sec) { starpu_usleep(nb_sec * 1e6f); }

/* every ready task is pushed as it becomes ready: nothing waits for this */
void starpu_do_schedule(void) {}

int starpu_worker_get_count_by_type(enum starpu_worker_archtype type)
{
    int n = 0;
    for (int i = 0; i < rt.nworkers; ++i) n += rt.workers[i].type == type;
    return n;
}

int starpu_conf_noworker(struct starpu_conf *conf)
{
    conf->ncpus = conf->ncuda = conf->nhip = conf->nopencl = 0;
    conf->nsycl = conf->nmax_fpga = conf->nmpi_sc = conf->ntcpip_sc = 0;
    return 0;
}

int starpu_init(struct starpu_conf *conf) { return starpu_initialize(conf, NULL, NULL); }

int starpu_initialize(struct starpu_conf *user_conf, int *argc, char ***argv)
{
    (void)argc;
    (void)argv;
    if (rt.initialized) {
        rt.initialized++;
        return 0;
    }
    struct starpu_conf c;
    if (user_conf) c = *user_conf;
    else starpu_conf_init(&c);

    const char *sched = getenv("STARPU_SCHED");
    if (sched && *sched && strcmp(sched, "dmda") && strcmp(sched, "dm") && strcmp(sched, "dmdas") &&
        strcmp(sched, "dmdar") && strcmp(sched, "eager") && strcmp(sched, "prio") && strcmp(sched, "heft"))
        fprintf(stderr, "[starpu_gb300] STARPU_SCHED=%s not provided, using dmda\n", sched);

    memset(&rt.stats, 0, sizeof rt.stats);
    pthread_mutex_init(&rt.lock, NULL);
    pthread_cond_init(&rt.all_done, NULL);
    rt.min_prio = INT_MIN;
    rt.max_prio = INT_MAX;
    rt.calibrate = (unsigned)env_int("STARPU_CALIBRATE", c.calibrate == (unsigned)-1 ? 0 : (int)c.calibrate);
    rt.transfer_us_per_byte = 1.0 / 50000.0; /* ~50 GB/s host <-> GPU */
    rt_perfmodel_init();

    int ndev = 0;
    int want_cuda = c.ncuda >= 0 ? c.ncuda : -1;
    want_cuda = env_int("STARPU_NCUDA", want_cuda);
    if (want_cuda != 0) {
        ndev = rt_cuda_init(want_cuda < 0 ? 1 : want_cuda);
        if (ndev < 0) ndev = 0;
    }
    int ncores = (int)sysconf(_SC_NPROCESSORS_ONLN);
    cpu_set_t set;
    if (sched_getaffinity(0, sizeof set, &set) == 0) ncores = CPU_COUNT(&set);
    int ncpu = c.ncpus >= 0 ? c.ncpus : ncores - ndev;
    ncpu = env_int("STARPU_NCPU", ncpu);
    if (ncpu < 0) ncpu = 0;
    if (ncpu + ndev > STARPU_NMAXWORKERS) ncpu = STARPU_NMAXWORKERS - ndev;
    if (ncpu + ndev == 0) return -ENODEV;

    rt.nworkers = 0;
    for (int d = 0; d < ndev; ++d) {
        struct rt_worker *w = &rt.workers[rt.nworkers];
        memset(w, 0, sizeof *w);
        w->id = rt.nworkers++;
        w->type = STARPU_CUDA_WORKER;
        w->devid = d;
    }
    for (int i = 0; i < ncpu; ++i) {
        struct rt_worker *w = &rt.workers[rt.nworkers];
        memset(w, 0, sizeof *w);
        w->id = rt.nworkers++;
        w->type = STARPU_CPU_WORKER;
        w->devid = i;
    }
    rt.ncuda = ndev;
    rt.ncpu = ncpu;
    rt.graph_mode = (ndev > 0 && ncpu == 0) ? env_int("STARPU_GB300_GRAPH", 1) : 0;
    /* STARPU_COMMUTE writers of one handle run in any order, one at a time,
     * where every worker is a CPU worker (they run their tasks synchronously);
     * with a CUDA worker they keep their submission order (a valid order of
     * commuting tasks).  STARPU_GB300_COMMUTE=0 keeps that order everywhere. */
    rt.relaxed_commute = ndev == 0 && env_int("STARPU_GB300_COMMUTE", 1) != 0;
    pthread_cond_init(&rt.commute_cond, NULL);
    for (int i = 0; i < rt.nworkers; ++i) {
        struct rt_worker *w = &rt.workers[i];
        w->dev.type = w->type;
        w->dev.devid = w->type == STARPU_CUDA_WORKER ? w->devid : 0;
        w->dev.ncores = 1;
        w->arch.ndevices = 1;
        w->arch.devices = &w->dev;
        pthread_cond_init(&w->cond, NULL);
    }
    rt.initialized = 1;
    rt.shutting_down = 0;
    for (int i = 0; i < rt.nworkers; ++i) {
        struct rt_worker *w = &rt.workers[i];
        if (w->type == STARPU_CUDA_WORKER) pthread_create(&w->thread, NULL, rt_cuda_worker_main, w);
        else pthread_create(&w->thread, NULL, rt_cpu_worker_main, w);
    }
    return 0;
}

int starpu_is_initialized(void) { return rt.initialized > 0; }

/* Driver pre-initialisation before starpu_init (src/core/workers.c:1614-1625):
 * the CPU and CUDA drivers of this runtime need none. */
void starpu_drivers_preinit(void) {}

void starpu_shutdown(void)
{
    if (!rt.initialized) return;
    if (--rt.initialized > 0) return;
    starpu_task_wait_for_all();
    starpu_profiling_worker_helper_display_summary();
    rt_lock();
    rt.shutting_down = 1;
    for (int i = 0; i < rt.nworkers; ++i) pthread_cond_broadcast(&rt.workers[i].cond);
    rt_unlock();
    for (int i = 0; i < rt.nworkers; ++i) pthread_join(rt.workers[i].thread, NULL);
    rt_perfmodel_save_all();
    for (int i = 0; i < rt.nworkers; ++i) {
        free(rt.workers[i].heap);
        rt.workers[i].heap = NULL;
        pthread_cond_destroy(&rt.workers[i].cond);
    }
    free(rt.pending);
    rt.pending = NULL;
    rt.npending = rt.cappending = 0;
    rt_cuda_shutdown();
    rt.nworkers = rt.ncpu = rt.ncuda = 0;
    rt_ctx_reset();
}

void starpu_pause(void)
{
    rt_lock();
    rt.paused = 1;
    rt_unlock();
}

void starpu_resume(void)
{
    rt_lock();
    rt.paused = 0;
    for (int i = 0; i < rt.nworkers; ++i) pthread_cond_broadcast(&rt.workers[i].cond);
    rt_unlock();
}

int starpu_asynchronous_copy_disabled(void) { return 0; }

/* ------------------------------------------------------------- workers */
unsigned starpu_worker_get_count(void) { return (unsigned)rt.nworkers; }
unsigned starpu_cpu_worker_get_count(void) { return (unsigned)rt.ncpu; }
unsigned starpu_cuda_worker_get_count(void) { return (unsigned)rt.ncuda; }
unsigned starpu_mpi_sc_worker_get_count(void) { return 0; }
unsigned starpu_tcpip_sc_worker_get_count(void) { return 0; }
unsigned starpu_hip_worker_get_count(void) { return 0; }
unsigned starpu_opencl_worker_get_count(void) { return 0; }
int starpu_worker_get_id(void) { return tls_worker; }

enum starpu_worker_archtype starpu_worker_get_type(int id)
{
    if (id < 0 || id >= rt.nworkers) return (enum starpu_worker_archtype)-1;
    return rt.workers[id].type;
}

int starpu_worker_get_devid(int id)
{
    if (id < 0 || id >= rt.nworkers) return -1;
    return rt.workers[id].devid;
}

void starpu_worker_get_name(int id, char *dst, size_t maxlen)
{
    if (id < 0 || id >= rt.nworkers) {
        snprintf(dst, maxlen, "invalid");
        return;
    }
    snprintf(dst, maxlen, "%s %d", rt.workers[id].type == STARPU_CUDA_WORKER ? "CUDA" : "CPU", rt.workers[id].devid);
}

struct starpu_perfmodel_arch *starpu_worker_get_perf_archtype(int workerid, unsigned sched_ctx_id)
{
    (void)sched_ctx_id;
    if (workerid < 0 || workerid >= rt.nworkers) return NULL;
    return &rt.workers[workerid].arch;
}

int starpu_worker_get_ids_by_type(enum starpu_worker_archtype type, int *workerids, unsigned maxsize)
{
    unsigned n = 0;
    for (int i = 0; i < rt.nworkers && n < maxsize; ++i)
        if (rt.workers[i].type == type) workerids[n++] = i;
    return (int)n;
}

/* parallel (combined) workers are not provided: every worker is a single unit */
int starpu_combined_worker_get_size(void) { return 1; }
int starpu_combined_worker_get_rank(void) { return 0; }

/* ------------------------------------------------ priorities and contexts */
int starpu_sched_get_min_priority(void) { return rt.initialized ? rt.min_prio : INT_MIN; }
int starpu_sched_get_max_priority(void) { return rt.initialized ? rt.max_prio : INT_MAX; }
int starpu_sched_set_min_priority(int p)
{
    rt.min_prio = p;
    return 0;
}
int starpu_sched_set_max_priority(int p)
{
    rt.max_prio = p;
    return 0;
}

/* ------------------------------------------------ scheduling contexts
 *
 * A context is a set of workers (src/core/sched_ctx.c): a task runs only on
 * the workers of its context -- the STARPU_SCHED_CTX it was given, else the
 * submitting thread's current context (starpu_sched_ctx_set_context), else
 * the initial context 0, which holds every worker (task.c:973-977,
 * sched_ctx.c:1689-1696).  Deleting a context hands its workers to its
 * inheritor, waits for the context's submitted tasks, then frees its id
 * (sched_ctx.c:1004-1079).  Every context uses the runtime's one policy
 * (dmda); a policy requested for a context is accepted and not used. */
struct rt_ctx {
    int used;
    unsigned inheritor; /* STARPU_NMAX_SCHED_CTXS: none */
    long nsubmitted;    /* submitted and not terminated */
    char member[STARPU_NMAXWORKERS];
};
static struct rt_ctx ctxs[STARPU_NMAX_SCHED_CTXS]; /* [0] is the initial context */
static __thread unsigned tls_ctx = STARPU_NMAX_SCHED_CTXS;

/* the context a task belongs to: an id that names no live context is the
 * initial one */
static unsigned ctx_live(unsigned id)
{
    return id > 0 && id < STARPU_NMAX_SCHED_CTXS && ctxs[id].used ? id : 0;
}

void rt_ctx_reset(void) { memset(ctxs, 0, sizeof ctxs); }

unsigned rt_ctx_resolve(struct starpu_task *t)
{
    unsigned id = t->sched_ctx;
    if (id == STARPU_NMAX_SCHED_CTXS) id = tls_ctx == STARPU_NMAX_SCHED_CTXS ? 0 : tls_ctx;
    return ctx_live(id);
}

/* called with the runtime lock held */
int rt_ctx_has_worker(unsigned id, int worker)
{
    id = ctx_live(id);
    return id == 0 || (worker >= 0 && worker < STARPU_NMAXWORKERS && ctxs[id].member[worker]);
}

/* called with the runtime lock held */
void rt_ctx_count(unsigned id, int delta)
{
    id = ctx_live(id);
    if (id) ctxs[id].nsubmitted += delta;
}

unsigned starpu_sched_ctx_create(int *workerids_ctx, int nworkers_ctx, const char *name, ...)
{
    (void)name;
    va_list ap;
    va_start(ap, name);
    int key;
    while ((key = va_arg(ap, int)) != 0) {
        if (key == STARPU_SCHED_CTX_POLICY_NAME) (void)va_arg(ap, const char *);
        else if (key == STARPU_SCHED_CTX_POLICY_STRUCT) (void)va_arg(ap, void *);
        else if (key == STARPU_SCHED_CTX_POLICY_MIN_PRIO || key == STARPU_SCHED_CTX_POLICY_MAX_PRIO) (void)va_arg(ap, int);
        else STARPU_ABORT_MSG("unknown starpu_sched_ctx_create argument %d", key);
    }
    va_end(ap);
    rt_lock();
    unsigned id = 1;
    while (id < STARPU_NMAX_SCHED_CTXS && ctxs[id].used) ++id;
    STARPU_ASSERT_MSG(id < STARPU_NMAX_SCHED_CTXS, "too many scheduling contexts (%d)", STARPU_NMAX_SCHED_CTXS);
    struct rt_ctx *c = &ctxs[id];
    memset(c, 0, sizeof *c);
    c->used = 1;
    c->inheritor = STARPU_NMAX_SCHED_CTXS;
    /* -1 workers: all of them; no list: workers 0 .. n-1 (sched_ctx.c:367-385) */
    const int n = nworkers_ctx == -1 ? rt.nworkers : nworkers_ctx;
    STARPU_ASSERT_MSG(n >= 0 && n <= rt.nworkers, "%d workers asked for a context, %d exist", n, rt.nworkers);
    for (int k = 0; k < n; ++k) {
        const int w = workerids_ctx && nworkers_ctx != -1 ? workerids_ctx[k] : k;
        STARPU_ASSERT_MSG(w >= 0 && w < rt.nworkers, "no worker %d", w);
        c->member[w] = 1;
    }
    rt_unlock();
    return id;
}

void starpu_sched_ctx_set_inheritor(unsigned id, unsigned inheritor)
{
    STARPU_ASSERT_MSG(id < STARPU_NMAX_SCHED_CTXS, "no scheduling context %u", id);
    rt_lock();
    ctxs[id].inheritor = inheritor;
    rt_unlock();
}

unsigned starpu_sched_ctx_get_inheritor(unsigned id)
{
    return id < STARPU_NMAX_SCHED_CTXS ? ctxs[id].inheritor : STARPU_NMAX_SCHED_CTXS;
}

void starpu_sched_ctx_delete(unsigned id)
{
    if (id == 0 || id >= STARPU_NMAX_SCHED_CTXS || !ctxs[id].used) return;
    rt_lock();
    struct rt_ctx *c = &ctxs[id];
    const unsigned inh = c->inheritor;
    for (unsigned k = 1; k < STARPU_NMAX_SCHED_CTXS; ++k)
        if (ctxs[k].used && ctxs[k].inheritor == id) ctxs[k].inheritor = inh;
    /* the workers move to a live inheritor (the initial context has them all) */
    if (inh > 0 && inh < STARPU_NMAX_SCHED_CTXS && ctxs[inh].used)
        for (int w = 0; w < rt.nworkers; ++w)
            if (c->member[w]) ctxs[inh].member[w] = 1;
    rt_unlock();
    rt_flush_and_wait();
    rt_lock();
    while (c->nsubmitted > 0) pthread_cond_wait(&rt.all_done, &rt.lock);
    c->used = 0;
    rt_unlock();
}

unsigned starpu_sched_ctx_get_nworkers(unsigned id)
{
    id = ctx_live(id);
    if (id == 0) return (unsigned)rt.nworkers;
    unsigned n = 0;
    for (int w = 0; w < rt.nworkers; ++w) n += ctxs[id].member[w] != 0;
    return n;
}

unsigned starpu_sched_ctx_contains_worker(int workerid, unsigned id)
{
    return workerid >= 0 && workerid < rt.nworkers && rt_ctx_has_worker(id, workerid);
}

void starpu_sched_ctx_set_context(unsigned *id) { tls_ctx = id ? *id : STARPU_NMAX_SCHED_CTXS; }
unsigned starpu_sched_ctx_get_context(void) { return tls_ctx; }

void starpu_reset_scheduler(void)
{
    rt_lock();
    for (int i = 0; i < rt.nworkers; ++i) rt.workers[i].expected_end = 0;
    rt_unlock();
}

static __thread long tls_iteration = -1;
void starpu_iteration_push(unsigned long iteration) { tls_iteration = (long)iteration; }
void starpu_iteration_pop(void) { tls_iteration = -1; }

/* ----------------------------------------------------------------- memory */
static size_t malloc_align = 64;

void starpu_malloc_set_align(size_t align)
{
    if (align > malloc_align) malloc_align = align;
}

int starpu_malloc_flags(void **A, size_t dim, int flags)
{
    if (!A) return -EINVAL;
    *A = NULL;
    if ((flags & STARPU_MALLOC_PINNED) && rt.ncuda > 0) {
        if (rt_cuda_host_alloc(A, dim ? dim : 1) == 0) return 0;
    }
    if (posix_memalign(A, malloc_align, dim ? dim : 1) != 0) return -ENOMEM;
    return 0;
}

int starpu_malloc(void **A, size_t dim) { return starpu_malloc_flags(A, dim, STARPU_MALLOC_PINNED); }

int starpu_free_flags(void *A, size_t dim, int flags)
{
    (void)dim;
    if (!A) return 0;
    if ((flags & STARPU_MALLOC_PINNED) && rt.ncuda > 0) {
        rt_cuda_host_free(A);
        return 0;
    }
    free(A);
    return 0;
}

int starpu_free(void *A) { return starpu_free_flags(A, 0, STARPU_MALLOC_PINNED); }
int starpu_free_noflag(void *A, size_t dim) { return starpu_free_flags(A, dim, 0); }

/* ------------------------------------------ vendor-library hooks (no-ops) */
void starpu_cublas_init(void) {}
void starpu_cublas_shutdown(void) {}
void starpu_cublas_set_stream(void) {}
void starpu_cusolver_init(void) {}
void starpu_cusolver_shutdown(void) {}
void starpu_hipblas_init(void) {}
void starpu_hipblas_shutdown(void) {}
void starpu_hipsolver_init(void) {}
void starpu_hipsolver_shutdown(void) {}

/* ----------------------------- tracing (FxT) and LP bound: not provided */
void starpu_fxt_start_profiling(void) {}
void starpu_fxt_stop_profiling(void) {}
void starpu_bound_start(int deps, int prio) { (void)deps; (void)prio; }
void starpu_bound_stop(void) {}
void starpu_bound_compute(double *res, double *integer_res, int integer)
{
    (void)integer;
    if (res) *res = 0.0;
    if (integer_res) *integer_res = 0.0;
}
void starpu_bound_print_lp(FILE *output)
{
    if (output) fprintf(output, "/* LP bound not provided by the GB300 runtime */\n");
}
void starpu_bound_print_mps(FILE *output)
{
    if (output) fprintf(output, "* MPS bound not provided by the GB300 runtime\n");
}
void starpu_bound_print(FILE *output, int integer)
{
    (void)integer;
    if (output) fprintf(output, "bound not provided by the GB300 runtime\n");
}

void starpu_bound_print_dot(FILE *output)
{
    if (output) fprintf(output, "/* task graph bound not provided by the GB300 runtime */\ndigraph G {}\n");
}

void starpu_profiling_bus_helper_display_summary(void)
{
    rt_lock();
    const unsigned long h2d = rt.stats.h2d_bytes, d2h = rt.stats.d2h_bytes;
    rt_unlock();
    fprintf(stderr, "\n#---------------------\nData transfer stats:\n");
    fprintf(stderr, "\tNUMA 0 -> CUDA 0\t%.4f MB\n", h2d / 1048576.0);
    fprintf(stderr, "\tCUDA 0 -> NUMA 0\t%.4f MB\n", d2h / 1048576.0);
    fprintf(stderr, "Total transfers: %.4f MB\n#---------------------\n", (h2d + d2h) / 1048576.0);
}

/* STARPU_WORKER_STATS=1: tasks run per worker, printed at shutdown to
 * stderr or STARPU_WORKER_STATS_FILE, in the layout of
 * profiling_helpers.c:88-181 without per-task profiling (time splits need
 * STARPU_PROFILING, which this runtime does not record) */
void starpu_profiling_worker_helper_display_summary(void)
{
    const char *on = getenv("STARPU_WORKER_STATS");
    if (!on || !atoi(on)) return;
    const char *path = getenv("STARPU_WORKER_STATS_FILE");
    FILE *f = path && *path ? fopen(path, "w") : stderr;
    if (!f) starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, "cannot open %s for the worker stats", path);
    fprintf(f, "\n#---------------------\nWorker stats:\n");
    for (int w = 0; w < rt.nworkers; ++w) {
        char name[64];
        starpu_worker_get_name(w, name, sizeof name);
        fprintf(f, "%-32s\n\t%d task(s)\n", name, (int)rt.workers[w].ntasks);
    }
    fprintf(f, "#---------------------\n");
    if (f != stderr) fclose(f);
}

static int profiling_status = 0;
int starpu_profiling_status_set(int status)
{
    int old = profiling_status;
    profiling_status = status;
    return old;
}
int starpu_profiling_status_get(void) { return profiling_status; }

void starpu_gb300_runtime_get_stats(struct starpu_gb300_runtime_stats *stats)
{
    rt_lock();
    if (stats) *stats = rt.stats;
    rt_unlock();
}

void starpu_gb300_runtime_reset_stats(void)
{
    rt_lock();
    memset(&rt.stats, 0, sizeof rt.stats);
    rt_unlock();
}
