/*
 * dmda scheduling and history-based performance models.
 *
 * Push (src/sched_policies/deque_modeling_policy_data_aware.c:604 semantics):
 * for every worker able to run the task, fitness = the worker's expected
 * availability + the expected transfer time of the data not valid on its
 * memory node + the expected length from the history model; the task goes to
 * the worker with the smallest fitness (uncalibrated archs predict 0, so they
 * get tasks and calibrate).  Each worker pops its queue by priority, then
 * submission order.
 *
 * History models (src/core/perfmodel/perfmodel_history.c): per symbol, per
 * arch (CPU / CUDA) and per footprint of the task's data shapes, the running
 * mean / deviation / count of measured execution times in microseconds.
 * They are loaded from and saved to
 *   $STARPU_PERF_MODEL_DIR/codelets/45/<symbol>.<hostname>
 * (default $STARPU_HOME/.starpu/sampling, then $HOME/.starpu/sampling) in the
 * version-45 text layout ("# hash size flops mean (us) dev (us) sum sum2 n").
 */
#include <math.h>
#include <sys/stat.h>
#include <unistd.h>

#include "rt_internal.h"

#define CALIBRATE_MINIMUM 10

/* ------------------------------------------------------------ queues */

static int job_before(const struct rt_job *a, const struct rt_job *b)
{
    if (a->task->priority != b->task->priority) return a->task->priority > b->task->priority;
    return a->seq < b->seq;
}

static void heap_push(struct rt_worker *w, struct rt_job *j)
{
    if (w->hn == w->hcap) {
        w->hcap = w->hcap ? 2 * w->hcap : 64;
        w->heap = realloc(w->heap, sizeof *w->heap * w->hcap);
    }
    int i = w->hn++;
    w->heap[i] = j;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (!job_before(w->heap[i], w->heap[p])) break;
        struct rt_job *x = w->heap[p];
        w->heap[p] = w->heap[i];
        w->heap[i] = x;
        i = p;
    }
}

static struct rt_job *heap_pop(struct rt_worker *w)
{
    if (!w->hn) return NULL;
    struct rt_job *top = w->heap[0];
    w->heap[0] = w->heap[--w->hn];
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, r = l + 1, b = i;
        if (l < w->hn && job_before(w->heap[l], w->heap[b])) b = l;
        if (r < w->hn && job_before(w->heap[r], w->heap[b])) b = r;
        if (b == i) break;
        struct rt_job *x = w->heap[b];
        w->heap[b] = w->heap[i];
        w->heap[i] = x;
        i = b;
    }
    return top;
}

static double transfer_time(struct starpu_task *t, struct rt_worker *w)
{
    int node = w->type == STARPU_CUDA_WORKER ? RT_NODE_GPU : RT_NODE_RAM;
    double bytes = 0;
    for (int i = 0; i < t->nbuffers; ++i) {
        starpu_data_handle_t h = t->handles[i];
        if (!h || !(t->modes[i] & STARPU_R)) continue;
        if (!h->valid[node]) bytes += (double)rt_data_size(h);
    }
    return bytes * rt.transfer_us_per_byte;
}

/* called with the runtime lock held */
void rt_sched_push(struct rt_job *j)
{
    struct starpu_task *t = j->task;
    double now = starpu_timing_now();
    int best = -1;
    double best_fit = INFINITY, best_len = 0;
    for (int i = 0; i < rt.nworkers; ++i) {
        struct rt_worker *w = &rt.workers[i];
        if (!rt_can_execute(w, t)) continue;
        double len = rt_expected_length(t, w->type);
        if (isnan(len)) len = 0;
        double avail = w->expected_end > now ? w->expected_end : now;
        double fit = avail + transfer_time(t, w) + len;
        if (fit < best_fit) {
            best_fit = fit;
            best = i;
            best_len = len;
        }
    }
    STARPU_ASSERT_MSG(best >= 0, "no worker can execute task %s", t->name ? t->name : "?");
    struct rt_worker *w = &rt.workers[best];
    double avail = w->expected_end > now ? w->expected_end : now;
    w->expected_end = avail + best_len;
    j->predicted = best_len;
    j->worker = best;
    t->predicted = best_len;
    heap_push(w, j);
    pthread_cond_signal(&w->cond);
}

/* called with the runtime lock held */
struct rt_job *rt_sched_pop(struct rt_worker *w)
{
    if (rt.paused) return NULL;
    return heap_pop(w);
}

/* ------------------------------------------------------- history models */

struct hist_entry {
    int arch;            /* 0 CPU, 1 CUDA */
    uint32_t footprint;
    size_t size;
    double flops;
    double sum, sum2;
    unsigned n;
    struct hist_entry *next;
};

struct starpu_perfmodel_history_state {
    struct hist_entry *entries;
    int dirty;
};

#define MAX_MODELS 256
static struct starpu_perfmodel *models[MAX_MODELS];
static int nmodels;
static pthread_mutex_t model_mu = PTHREAD_MUTEX_INITIALIZER;

void starpu_perfmodel_get_model_path(const char *symbol, char *path, size_t maxlen)
{
    const char *dir = getenv("STARPU_PERF_MODEL_DIR");
    char base[1024];
    if (dir && *dir) snprintf(base, sizeof base, "%s", dir);
    else {
        const char *home = getenv("STARPU_HOME");
        if (!home || !*home) home = getenv("HOME");
        if (!home) home = "/tmp";
        snprintf(base, sizeof base, "%s/.starpu/sampling", home);
    }
    char host[256];
    const char *h = getenv("STARPU_HOSTNAME");
    if (h && *h) snprintf(host, sizeof host, "%s", h);
    else if (gethostname(host, sizeof host) != 0) snprintf(host, sizeof host, "unknown");
    snprintf(path, maxlen, "%s/codelets/45/%s.%s", base, symbol, host);
}

static void mkdir_p(const char *path)
{
    char tmp[1024];
    snprintf(tmp, sizeof tmp, "%s", path);
    for (char *p = tmp + 1; *p; ++p)
        if (*p == '/') {
            *p = 0;
            mkdir(tmp, 0755);
            *p = '/';
        }
}

static struct hist_entry *find(struct starpu_perfmodel_history_state *s, int arch, uint32_t fp, int create)
{
    for (struct hist_entry *e = s->entries; e; e = e->next)
        if (e->arch == arch && e->footprint == fp) return e;
    if (!create) return NULL;
    struct hist_entry *e = calloc(1, sizeof *e);
    e->arch = arch;
    e->footprint = fp;
    e->next = s->entries;
    s->entries = e;
    return e;
}

/* Parse a file written by save_model (a sequence of "# DEV <arch>" blocks of
 * entry lines "hash size flops mean dev sum sum2 n"). */
static void load_model(struct starpu_perfmodel *m)
{
    char path[1200];
    starpu_perfmodel_get_model_path(m->symbol, path, sizeof path);
    FILE *f = fopen(path, "r");
    if (!f) return;
    char line[512];
    int arch = -1;
    while (fgets(line, sizeof line, f)) {
        int a;
        if (sscanf(line, "# device type %d", &a) == 1) {
            arch = a;
            continue;
        }
        if (line[0] == '#' || arch < 0) continue;
        unsigned fp;
        size_t size;
        double flops, mean, dev, sum, sum2;
        unsigned n;
        if (sscanf(line, "%x %zu %lf %lf %lf %lf %lf %u", &fp, &size, &flops, &mean, &dev, &sum, &sum2, &n) == 8) {
            struct hist_entry *e = find(m->state, arch, fp, 1);
            e->size = size;
            e->flops = flops;
            e->sum = sum;
            e->sum2 = sum2;
            e->n = n;
        }
    }
    fclose(f);
}

static void ensure_model(struct starpu_perfmodel *m)
{
    if (m->is_init) return;
    pthread_mutex_lock(&model_mu);
    if (!m->is_init) {
        m->state = calloc(1, sizeof *m->state);
        if (m->symbol) load_model(m);
        if (nmodels < MAX_MODELS) models[nmodels++] = m;
        m->is_loaded = 1;
        m->is_init = 1;
    }
    pthread_mutex_unlock(&model_mu);
}

static uint32_t task_footprint(struct starpu_task *t)
{
    uint32_t x = 0;
    for (int i = 0; i < t->nbuffers; ++i) {
        if (!t->handles[i] || (t->modes[i] & STARPU_NOFOOTPRINT) || (t->modes[i] & STARPU_SCRATCH)) continue;
        uint32_t f = rt_data_footprint(t->handles[i]);
        x = (x * 0x9E3779B1u) ^ f;
    }
    return x;
}

static size_t task_size(struct starpu_task *t)
{
    size_t s = 0;
    for (int i = 0; i < t->nbuffers; ++i)
        if (t->handles[i]) s += rt_data_size(t->handles[i]);
    return s;
}

double rt_expected_length(struct starpu_task *t, enum starpu_worker_archtype type)
{
    struct starpu_perfmodel *m = t->cl ? t->cl->model : NULL;
    if (!m || m->type != STARPU_HISTORY_BASED) return NAN;
    ensure_model(m);
    pthread_mutex_lock(&model_mu);
    struct hist_entry *e = find(m->state, type == STARPU_CUDA_WORKER ? 1 : 0, task_footprint(t), 0);
    double v = (e && e->n >= CALIBRATE_MINIMUM) ? e->sum / e->n : NAN;
    pthread_mutex_unlock(&model_mu);
    return v;
}

double starpu_task_expected_length(struct starpu_task *task, struct starpu_perfmodel_arch *arch, unsigned nimpl)
{
    (void)nimpl;
    if (!arch || arch->ndevices < 1) return NAN;
    return rt_expected_length(task, arch->devices[0].type);
}

double starpu_task_expected_data_transfer_time(unsigned memory_node, struct starpu_task *task)
{
    double bytes = 0;
    int node = memory_node == STARPU_MAIN_RAM ? RT_NODE_RAM : RT_NODE_GPU;
    for (int i = 0; i < task->nbuffers; ++i)
        if (task->handles[i] && (task->modes[i] & STARPU_R) && !task->handles[i]->valid[node])
            bytes += (double)rt_data_size(task->handles[i]);
    return bytes * rt.transfer_us_per_byte;
}

uint32_t starpu_task_footprint(struct starpu_perfmodel *model, struct starpu_task *task,
                               struct starpu_perfmodel_arch *arch, unsigned nimpl)
{
    (void)model;
    (void)arch;
    (void)nimpl;
    return task_footprint(task);
}

static void record(struct starpu_perfmodel *m, struct starpu_task *t, int arch, double us)
{
    ensure_model(m);
    pthread_mutex_lock(&model_mu);
    struct hist_entry *e = find(m->state, arch, task_footprint(t), 1);
    e->size = task_size(t);
    e->flops = t->flops;
    e->sum += us;
    e->sum2 += us * us;
    e->n++;
    m->state->dirty = 1;
    pthread_mutex_unlock(&model_mu);
}

void rt_perfmodel_feedback(struct starpu_task *t, enum starpu_worker_archtype type, double us)
{
    struct starpu_perfmodel *m = t->cl->model;
    if (!m || m->type != STARPU_HISTORY_BASED) return;
    record(m, t, type == STARPU_CUDA_WORKER ? 1 : 0, us);
}

void starpu_perfmodel_update_history(struct starpu_perfmodel *model, struct starpu_task *task,
                                     struct starpu_perfmodel_arch *arch, unsigned cpuid, unsigned nimpl,
                                     double measured)
{
    (void)cpuid;
    (void)nimpl;
    if (!model || !arch || arch->ndevices < 1) return;
    record(model, task, arch->devices[0].type == STARPU_CUDA_WORKER ? 1 : 0, measured);
}

static int save_model(struct starpu_perfmodel *m)
{
    if (!m->symbol || !m->state) return -EINVAL;
    char path[1200];
    starpu_perfmodel_get_model_path(m->symbol, path, sizeof path);
    mkdir_p(path);
    FILE *f = fopen(path, "w");
    if (!f) return -errno;
    fprintf(f, "##################\n# Performance Model Version\n45\n\n");
    for (int arch = 0; arch < 2; ++arch) {
        int cnt = 0;
        for (struct hist_entry *e = m->state->entries; e; e = e->next) cnt += e->arch == arch;
        if (!cnt) continue;
        fprintf(f, "####################\n# device type %d\n# (CPU - 0, CUDA - 1)\n# number of entries\n%d\n", arch,
                cnt);
        fprintf(f, "# hash\t\tsize\t\tflops\t\tmean (us)\tdev (us)\tsum\t\tsum2\t\tn\n");
        for (struct hist_entry *e = m->state->entries; e; e = e->next) {
            if (e->arch != arch) continue;
            double mean = e->n ? e->sum / e->n : 0;
            double var = e->n ? e->sum2 / e->n - mean * mean : 0;
            fprintf(f, "%08x\t%-15zu\t%-15e\t%-15e\t%-15e\t%-15e\t%-15e\t%u\n", e->footprint, e->size, e->flops, mean,
                    var > 0 ? sqrt(var) : 0.0, e->sum, e->sum2, e->n);
        }
        fprintf(f, "\n");
    }
    fclose(f);
    m->state->dirty = 0;
    return 0;
}

int starpu_save_history_based_model(struct starpu_perfmodel *model)
{
    ensure_model(model);
    pthread_mutex_lock(&model_mu);
    int rc = save_model(model);
    pthread_mutex_unlock(&model_mu);
    return rc;
}

void rt_perfmodel_save_all(void)
{
    pthread_mutex_lock(&model_mu);
    for (int i = 0; i < nmodels; ++i)
        if (models[i]->state && models[i]->state->dirty) save_model(models[i]);
    pthread_mutex_unlock(&model_mu);
}

int starpu_perfmodel_load_symbol(const char *symbol, struct starpu_perfmodel *model)
{
    memset(model, 0, sizeof *model);
    model->type = STARPU_HISTORY_BASED;
    model->symbol = strdup(symbol);
    ensure_model(model);
    return model->state->entries ? 0 : -ENOENT;
}

int starpu_perfmodel_unload_model(struct starpu_perfmodel *model)
{
    pthread_mutex_lock(&model_mu);
    for (int i = 0; i < nmodels; ++i)
        if (models[i] == model) {
            models[i] = models[--nmodels];
            break;
        }
    pthread_mutex_unlock(&model_mu);
    if (model->state) {
        struct hist_entry *e = model->state->entries;
        while (e) {
            struct hist_entry *n = e->next;
            free(e);
            e = n;
        }
        free(model->state);
        model->state = NULL;
    }
    model->is_init = 0;
    return 0;
}
