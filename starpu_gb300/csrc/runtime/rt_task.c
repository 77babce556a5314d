/*
 * Tasks: creation, starpu_task_insert argument parsing
 * (include/starpu_task_util.h semantics), implicit data dependencies
 * (sequential consistency: a writer depends on the last writer and every
 * reader since; a reader depends on the last writer -- the edges of
 * src/core/dependencies/implicit_data_deps.c), tags, termination and waits.
 */
#include <stdarg.h>

#include "rt_internal.h"

void starpu_codelet_init(struct starpu_codelet *cl) { memset(cl, 0, sizeof *cl); }

void starpu_task_init(struct starpu_task *t)
{
    memset(t, 0, sizeof *t);
    t->sequential_consistency = 1;
    t->detach = 1;
    t->priority = STARPU_DEFAULT_PRIO;
    t->status = STARPU_TASK_INIT;
    t->magic = 42;
    t->sched_ctx = STARPU_NMAX_SCHED_CTXS; /* the submitting thread's context */
}

struct starpu_task *starpu_task_create(void)
{
    struct starpu_task *t = malloc(sizeof *t);
    starpu_task_init(t);
    t->destroy = 1;
    return t;
}

void starpu_task_clean(struct starpu_task *t)
{
    if (t->cl_arg_free && t->cl_arg) free(t->cl_arg);
    if (t->callback_arg_free && t->callback_arg) free(t->callback_arg);
    if (t->prologue_callback_arg_free && t->prologue_callback_arg) free(t->prologue_callback_arg);
    free(t->declared_deps);
    t->cl_arg = NULL;
    t->callback_arg = NULL;
    t->prologue_callback_arg = NULL;
    t->declared_deps = NULL;
    t->ndeclared_deps = 0;
}

void starpu_task_destroy(struct starpu_task *t)
{
    if (!t) return;
    starpu_task_clean(t);
    free(t);
}

struct starpu_task *starpu_task_get_current(void) { return rt_current_task_get(); }

int starpu_task_nsubmitted(void) { return (int)rt.nsubmitted; }

int starpu_task_nready(void)
{
    int n = 0;
    rt_lock();
    for (int i = 0; i < rt.nworkers; ++i) n += rt.workers[i].hn;
    rt_unlock();
    return n;
}

/* ----------------------------------------------------------------- tags */

struct tag_entry {
    starpu_tag_t id;
    struct rt_job *job;     /* last submitted task with this tag (NULL once done) */
    struct starpu_task *task; /* that task, kept after it is done (starpu_tag_get_task) */
    int done;               /* completed (or notified from the application) */
    starpu_tag_t *deps;
    int ndeps;
    struct rt_job **waiters; /* tasks waiting for this tag before any task carrying it was submitted */
    int nwaiters, capwaiters;
    struct tag_entry *next;
};

static void tag_add_waiter(struct tag_entry *e, struct rt_job *j)
{
    if (e->nwaiters == e->capwaiters) {
        e->capwaiters = e->capwaiters ? 2 * e->capwaiters : 4;
        e->waiters = realloc(e->waiters, sizeof *e->waiters * e->capwaiters);
    }
    e->waiters[e->nwaiters++] = j;
    j->ndeps++;
}

/* called with the runtime lock held when tag e becomes done */
static void tag_release_waiters(struct tag_entry *e)
{
    for (int i = 0; i < e->nwaiters; ++i) {
        struct rt_job *u = e->waiters[i];
        if (--u->ndeps == 0 && !rt.graph_mode) {
            u->task->status = STARPU_TASK_READY;
            rt_sched_push(u);
        }
    }
    e->nwaiters = 0;
}

#define TAG_BUCKETS 4096
static struct tag_entry *tags[TAG_BUCKETS];
static pthread_cond_t tag_cond = PTHREAD_COND_INITIALIZER;

static struct tag_entry *tag_get(starpu_tag_t id, int create)
{
    unsigned b = (unsigned)((id ^ (id >> 29) ^ (id >> 47)) % TAG_BUCKETS);
    for (struct tag_entry *e = tags[b]; e; e = e->next)
        if (e->id == id) return e;
    if (!create) return NULL;
    struct tag_entry *e = calloc(1, sizeof *e);
    e->id = id;
    e->next = tags[b];
    tags[b] = e;
    return e;
}

void starpu_tag_declare_deps_array(starpu_tag_t id, unsigned ndeps, starpu_tag_t *array)
{
    rt_lock();
    struct tag_entry *e = tag_get(id, 1);
    e->deps = realloc(e->deps, sizeof(starpu_tag_t) * (e->ndeps + ndeps));
    for (unsigned i = 0; i < ndeps; ++i) e->deps[e->ndeps++] = array[i];
    rt_unlock();
}

void starpu_tag_declare_deps(starpu_tag_t id, unsigned ndeps, ...)
{
    starpu_tag_t *a = malloc(sizeof(starpu_tag_t) * (ndeps ? ndeps : 1));
    va_list ap;
    va_start(ap, ndeps);
    for (unsigned i = 0; i < ndeps; ++i) a[i] = va_arg(ap, starpu_tag_t);
    va_end(ap);
    starpu_tag_declare_deps_array(id, ndeps, a);
    free(a);
}

int starpu_tag_wait_array(unsigned ntags, starpu_tag_t *id)
{
    rt_flush_and_wait();
    rt_lock();
    for (unsigned i = 0; i < ntags; ++i) {
        struct tag_entry *e = tag_get(id[i], 1);
        while (!e->done) pthread_cond_wait(&tag_cond, &rt.lock);
    }
    rt_unlock();
    return 0;
}

int starpu_tag_wait(starpu_tag_t id) { return starpu_tag_wait_array(1, &id); }

void starpu_tag_remove(starpu_tag_t id)
{
    rt_lock();
    struct tag_entry *e = tag_get(id, 0);
    if (e) {
        e->done = 0;
        e->job = NULL;
        free(e->deps);
        e->deps = NULL;
        e->ndeps = 0;
    }
    rt_unlock();
}

void starpu_tag_notify_from_apps(starpu_tag_t id)
{
    rt_lock();
    struct tag_entry *e = tag_get(id, 1);
    e->done = 1;
    tag_release_waiters(e);
    pthread_cond_broadcast(&tag_cond);
    rt_unlock();
    rt_drain();
}

/* rt_submit flags: no data or tag dependencies; already counted as submitted
 * (a regenerated task) */
enum { SUBMIT_NODEPS = 1, SUBMIT_COUNTED = 2 };
static int rt_submit(struct starpu_task *t, int flags);
static void pack_value(void **buf, size_t *size, const void *p, size_t sz);

/* ---------------------------------------------------------- dependencies */

static void add_edge(struct rt_job *from, struct rt_job *to)
{
    if (!from || from == to || from->terminated) return;
    if (from->nsucc && from->succ[from->nsucc - 1] == to) return; /* same pair twice in a row */
    if (from->nsucc == from->capsucc) {
        from->capsucc = from->capsucc ? 2 * from->capsucc : 4;
        from->succ = realloc(from->succ, sizeof *from->succ * from->capsucc);
    }
    from->succ[from->nsucc++] = to;
    to->ndeps++;
    if (to->nprev == to->capprev) {
        to->capprev = to->capprev ? 2 * to->capprev : 4;
        to->prev = realloc(to->prev, sizeof *to->prev * to->capprev);
    }
    to->prev[to->nprev++] = from;
}

/* Explicit task dependencies (src/core/dependencies/task_deps.c semantics):
 * a declared predecessor that is done adds nothing, a submitted one an edge;
 * one not submitted yet holds the dependent (counted with its tag waits, so
 * that graph mode keeps it pending) until the predecessor is submitted. */
struct task_waiter {
    struct starpu_task *pred;
    struct rt_job *job;
    struct task_waiter *next;
};
static struct task_waiter *task_waiters; /* guarded by the runtime lock */

void starpu_task_declare_deps_array(struct starpu_task *task, unsigned ndeps, struct starpu_task *task_array[])
{
    if (!ndeps) return;
    STARPU_ASSERT_MSG(!task->starpu_private, "dependencies must be declared before the task is submitted");
    task->declared_deps = realloc(task->declared_deps, sizeof *task->declared_deps * (task->ndeclared_deps + ndeps));
    memcpy(task->declared_deps + task->ndeclared_deps, task_array, sizeof *task_array * ndeps);
    task->ndeclared_deps += ndeps;
}

void starpu_task_declare_deps(struct starpu_task *task, unsigned ndeps, ...)
{
    if (!ndeps) return;
    struct starpu_task **deps = malloc(sizeof *deps * ndeps);
    va_list ap;
    va_start(ap, ndeps);
    for (unsigned i = 0; i < ndeps; ++i) deps[i] = va_arg(ap, struct starpu_task *);
    va_end(ap);
    starpu_task_declare_deps_array(task, ndeps, deps);
    free(deps);
}

/* called with the runtime lock held, as job j of its task is submitted */
static void link_declared_deps(struct rt_job *j)
{
    struct starpu_task *t = j->task;
    for (unsigned i = 0; i < t->ndeclared_deps; ++i) {
        struct starpu_task *p = t->declared_deps[i];
        if (!p || p == t || p->status == STARPU_TASK_FINISHED) continue;
        if (p->starpu_private) {
            add_edge(p->starpu_private, j);
        } else {
            struct task_waiter *w = malloc(sizeof *w);
            w->pred = p;
            w->job = j;
            w->next = task_waiters;
            task_waiters = w;
            j->ndeps++;
            j->tag_waits++;
        }
    }
}

/* called with the runtime lock held, as job j of its task is submitted:
 * tasks that declared a dependency on it before now wait for it */
static void link_waiting_successors(struct rt_job *j)
{
    for (struct task_waiter **pw = &task_waiters; *pw;) {
        struct task_waiter *w = *pw;
        if (w->pred != j->task) {
            pw = &w->next;
            continue;
        }
        add_edge(j, w->job);
        w->job->ndeps--;
        w->job->tag_waits--;
        *pw = w->next;
        free(w);
    }
}

static void add_commuter(starpu_data_handle_t h, struct rt_job *j)
{
    if (h->ncommuters == h->capcommuters) {
        h->capcommuters = h->capcommuters ? 2 * h->capcommuters : 8;
        h->commuters = realloc(h->commuters, sizeof *h->commuters * h->capcommuters);
    }
    h->commuters[h->ncommuters++] = j;
}

/* Commuting writers of one handle run one at a time: a task takes the busy
 * flag of each handle it writes with STARPU_COMMUTE before it runs (in
 * handle-address order, so two tasks never wait for each other) and gives
 * them back when it is done.  Called with the runtime lock held. */
static int commute_handles(struct starpu_task *t, starpu_data_handle_t *hs)
{
    int n = 0;
    for (int i = 0; i < t->nbuffers; ++i) {
        starpu_data_handle_t h = t->handles[i];
        if (!h || !(t->modes[i] & STARPU_COMMUTE) || !(t->modes[i] & STARPU_W)) continue;
        int k = n;
        while (k > 0 && (uintptr_t)hs[k - 1] > (uintptr_t)h) {
            hs[k] = hs[k - 1];
            --k;
        }
        if (k > 0 && hs[k - 1] == h) { /* the same handle twice */
            for (int q = k; q < n; ++q) hs[q] = hs[q + 1];
            continue;
        }
        hs[k] = h;
        ++n;
    }
    return n;
}

void rt_commute_acquire(struct starpu_task *t)
{
    starpu_data_handle_t hs[STARPU_NMAXBUFS];
    const int n = commute_handles(t, hs);
    for (int k = 0; k < n; ++k) {
        while (hs[k]->commute_busy) pthread_cond_wait(&rt.commute_cond, &rt.lock);
        hs[k]->commute_busy = 1;
    }
}

void rt_commute_release(struct starpu_task *t)
{
    starpu_data_handle_t hs[STARPU_NMAXBUFS];
    const int n = commute_handles(t, hs);
    for (int k = 0; k < n; ++k) hs[k]->commute_busy = 0;
    if (n) pthread_cond_broadcast(&rt.commute_cond);
}

/* End dependencies on other tasks (starpu_task_dep.h): `task` terminates
 * only once each of them has.  A task done already adds nothing; one
 * submitted releases `task` when it terminates; one not submitted yet is
 * recorded until it is. */
struct end_waiter {
    struct starpu_task *pred, *task;
    struct end_waiter *next;
};
static struct end_waiter *end_waiters; /* guarded by the runtime lock */

static void add_end_release(struct rt_job *j, struct starpu_task *task)
{
    if (j->nend_release == j->capend_release) {
        j->capend_release = j->capend_release ? 2 * j->capend_release : 4;
        j->end_release = realloc(j->end_release, sizeof *j->end_release * j->capend_release);
    }
    j->end_release[j->nend_release++] = task;
}

void starpu_task_declare_end_deps_array(struct starpu_task *task, unsigned ndeps, struct starpu_task *task_array[])
{
    rt_lock();
    for (unsigned i = 0; i < ndeps; ++i) {
        struct starpu_task *p = task_array[i];
        if (!p || p == task || p->status == STARPU_TASK_FINISHED) continue;
        task->nb_termination_call_required++;
        if (p->starpu_private) {
            add_end_release(p->starpu_private, task);
        } else {
            struct end_waiter *w = malloc(sizeof *w);
            w->pred = p;
            w->task = task;
            w->next = end_waiters;
            end_waiters = w;
        }
    }
    rt_unlock();
}

void starpu_task_declare_end_deps(struct starpu_task *task, unsigned ndeps, ...)
{
    if (!ndeps) return;
    struct starpu_task **deps = malloc(sizeof *deps * ndeps);
    va_list ap;
    va_start(ap, ndeps);
    for (unsigned i = 0; i < ndeps; ++i) deps[i] = va_arg(ap, struct starpu_task *);
    va_end(ap);
    starpu_task_declare_end_deps_array(task, ndeps, deps);
    free(deps);
}

/* runtime lock held, as job j of its task is submitted */
static void link_end_waiters(struct rt_job *j)
{
    for (struct end_waiter **pw = &end_waiters; *pw;) {
        struct end_waiter *w = *pw;
        if (w->pred != j->task) {
            pw = &w->next;
            continue;
        }
        add_end_release(j, w->task);
        *pw = w->next;
        free(w);
    }
}

static void add_reader(starpu_data_handle_t h, struct rt_job *j)
{
    if (h->nreaders == h->capreaders) {
        h->capreaders = h->capreaders ? 2 * h->capreaders : 8;
        h->readers = realloc(h->readers, sizeof *h->readers * h->capreaders);
    }
    h->readers[h->nreaders++] = j;
}

int rt_can_execute(struct rt_worker *w, struct starpu_task *t)
{
    struct starpu_codelet *cl = t->cl;
    if (!cl) return 1;
    uint32_t where = t->where ? t->where : cl->where;
    if (w->type == STARPU_CUDA_WORKER) {
        if (where && !(where & STARPU_CUDA)) return 0;
        if (!cl->cuda_funcs[0]) return 0;
    } else {
        if (where && !(where & STARPU_CPU)) return 0;
        if (!cl->cpu_funcs[0]) return 0;
    }
    if (t->execute_on_a_specific_worker && (int)t->workerid != w->id) return 0;
    if (cl->can_execute && !cl->can_execute((unsigned)w->id, t, 0)) return 0;
    return 1;
}

static int rt_submit(struct starpu_task *t, int flags)
{
    const int nodeps = flags & SUBMIT_NODEPS;
    STARPU_ASSERT(rt.initialized);
    if (t->cl) {
        int nb = t->cl->nbuffers >= 0 ? t->cl->nbuffers : t->nbuffers;
        t->nbuffers = nb;
        STARPU_ASSERT_MSG(nb <= STARPU_NMAXBUFS, "too many buffers (%d)", nb);
        for (int i = 0; i < nb; ++i)
            if (!t->modes[i]) t->modes[i] = t->cl->modes[i];
    }
    t->sched_ctx = rt_ctx_resolve(t);
    STARPU_ASSERT_MSG(!rt.graph_mode || (!t->prologue_callback_func && t->where != STARPU_NOWHERE),
                      "prologue callbacks and STARPU_NOWHERE tasks need task-by-task execution "
                      "(STARPU_GB300_GRAPH=0, or a CPU worker beside the CUDA worker)");
    if (t->cl && t->where != STARPU_NOWHERE) {
        /* a worker of the task's context must be able to run it
         * (workers.c _starpu_worker_exists) */
        int ok = 0;
        rt_lock();
        for (int w = 0; w < rt.nworkers && !ok; ++w)
            ok = rt_can_execute(&rt.workers[w], t) && rt_ctx_has_worker(t->sched_ctx, w);
        rt_unlock();
        if (!ok) return -ENODEV;
    }
    struct rt_job *j = calloc(1, sizeof *j);
    j->task = t;
    j->worker = -1;
    j->heap_index = -1;
    t->starpu_private = j;
    t->status = STARPU_TASK_BLOCKED;
    int sync = t->synchronous;

    rt_lock();
    j->seq = rt.seq++;
    if (!(flags & SUBMIT_COUNTED)) {
        rt.nsubmitted++;
        rt_ctx_count(t->sched_ctx, +1);
    }
    j->ndeps = 1; /* held until submission completes */
    if (t->sequential_consistency && !nodeps) {
        for (int i = 0; i < t->nbuffers; ++i) {
            starpu_data_handle_t h = t->handles[i];
            enum starpu_data_access_mode m = t->modes[i];
            if (!h || !h->seq_consistency || (m & STARPU_SCRATCH) || (m & STARPU_REDUX)) continue;
            if ((m & STARPU_W) && (m & STARPU_COMMUTE) && rt.relaxed_commute) {
                /* after the last plain writer and the readers since, in any
                 * order with the other commuting writers
                 * (implicit_data_deps.c) */
                add_edge(h->last_writer, j);
                for (int r = 0; r < h->nreaders; ++r) add_edge(h->readers[r], j);
                add_commuter(h, j);
            } else if (m & STARPU_W) {
                add_edge(h->last_writer, j);
                for (int r = 0; r < h->nreaders; ++r) add_edge(h->readers[r], j);
                for (int c = 0; c < h->ncommuters; ++c) add_edge(h->commuters[c], j);
                h->nreaders = 0;
                h->ncommuters = 0;
                h->last_writer = j;
            } else if (m & STARPU_R) {
                add_edge(h->last_writer, j);
                for (int c = 0; c < h->ncommuters; ++c) add_edge(h->commuters[c], j);
                add_reader(h, j);
            }
        }
    }
    if (t->use_tag && !nodeps) {
        struct tag_entry *e = tag_get(t->tag_id, 1);
        for (int d = 0; d < e->ndeps; ++d) {
            struct tag_entry *p = tag_get(e->deps[d], 1);
            if (p->done) continue;
            if (p->job) add_edge(p->job, j);
            else {
                tag_add_waiter(p, j); /* its task is not submitted yet */
                j->tag_waits++;
            }
        }
        e->job = j;
        e->task = t;
        e->done = 0;
        /* tasks that waited for this tag before it had a task now depend on it */
        for (int w = 0; w < e->nwaiters; ++w) {
            struct rt_job *u = e->waiters[w];
            add_edge(j, u);
            u->ndeps--;
            u->tag_waits--;
        }
        e->nwaiters = 0;
        j->tag = t->tag_id;
        j->has_tag = 1;
    }
    if (!nodeps && t->ndeclared_deps) link_declared_deps(j);
    if (task_waiters) link_waiting_successors(j);
    if (end_waiters) link_end_waiters(j);
    if (rt.graph_mode) {
        if (rt.npending == rt.cappending) {
            rt.cappending = rt.cappending ? 2 * rt.cappending : 1024;
            rt.pending = realloc(rt.pending, sizeof *rt.pending * rt.cappending);
        }
        j->graph_slot = rt.npending;
        rt.pending[rt.npending++] = j;
        j->ndeps--;
    } else if (--j->ndeps == 0) {
        t->status = STARPU_TASK_READY;
        rt_sched_push(j);
    }
    rt_unlock();
    rt_drain();
    if (sync) starpu_task_wait(t);
    return 0;
}

int starpu_task_submit(struct starpu_task *t) { return rt_submit(t, 0); }

/* task.c:1577: no data or tag dependencies -- the caller holds the data */
int starpu_task_submit_nodeps(struct starpu_task *t) { return rt_submit(t, SUBMIT_NODEPS); }

void rt_drain(void)
{
    for (;;) {
        rt_lock();
        struct rt_job *j = rt.defer_head;
        if (j) {
            rt.defer_head = j->defer_next;
            if (!rt.defer_head) rt.defer_tail = NULL;
        }
        rt_unlock();
        if (!j) return;
        struct starpu_task *t = j->task;
        if (t->prologue_callback_func && !j->prologue_done) {
            j->prologue_done = 1;
            struct starpu_task *prev = rt_current_task_get();
            rt_current_task_set(t);
            t->prologue_callback_func(t->prologue_callback_arg);
            rt_current_task_set(prev);
        }
        if (t->where == STARPU_NOWHERE) {
            rt_job_terminate(j, 0.0); /* nothing to run (sched_policy.c:676) */
        } else {
            rt_lock();
            rt_sched_push(j);
            rt_unlock();
        }
    }
}

/* before or after the task's submission (jobs.c:355-361) */
void starpu_task_end_dep_add(struct starpu_task *t, int nb_deps)
{
    rt_lock();
    t->nb_termination_call_required += nb_deps;
    rt_unlock();
}

void starpu_task_end_dep_release(struct starpu_task *t)
{
    struct rt_job *j = t->starpu_private;
    STARPU_ASSERT_MSG(j, "starpu_task_end_dep_release on a task that is not submitted");
    rt_job_terminate(j, 0.0);
}

/* Called with the runtime lock NOT held, after the job's work completed. */
void rt_job_terminate(struct rt_job *j, double measured_us)
{
    struct starpu_task *t = j->task;
    if (t->cl && t->cl->model && measured_us > 0) {
        int w = j->worker;
        rt_perfmodel_feedback(t, &rt.workers[w >= 0 ? w : 0].arch, measured_us);
    }
    /* a termination held by starpu_task_end_dep_add needs one more call per
     * added dependency (jobs.c:363-373) */
    rt_lock();
    if (t->nb_termination_call_required > 0) {
        t->nb_termination_call_required--;
        rt_unlock();
        return;
    }
    rt_unlock();
    if (t->callback_func) {
        struct starpu_task *prev = rt_current_task_get();
        rt_current_task_set(t);
        t->callback_func(t->callback_arg);
        rt_current_task_set(prev);
    }
    /* a task still marked regenerate after its callback runs again
     * (jobs.c): this run's job is released first, the task stays counted as
     * submitted (so waits for all tasks do not end in between), then it is
     * submitted anew */
    const int regen = t->regenerate;
    if (regen) STARPU_ASSERT_MSG(t->detach && !t->synchronous, "a regenerated task must be detached and asynchronous");
    rt_lock();
    j->terminated = 1;
    if (!regen) t->status = STARPU_TASK_FINISHED;
    for (int i = 0; i < t->nbuffers; ++i)
        if (t->handles[i]) rt_data_forget_job(t->handles[i], j);
    for (int s = 0; s < j->nsucc; ++s) {
        struct rt_job *u = j->succ[s];
        for (int p = 0; p < u->nprev; ++p) /* keep predecessor lists free of finished jobs */
            if (u->prev[p] == j) {
                u->prev[p] = u->prev[--u->nprev];
                --p;
            }
        if (--u->ndeps == 0 && !rt.graph_mode) {
            u->task->status = STARPU_TASK_READY;
            rt_sched_push(u);
        }
    }
    if (j->has_tag) {
        struct tag_entry *e = tag_get(j->tag, 1);
        if (e->job == j) {
            e->done = 1;
            e->job = NULL;
            tag_release_waiters(e);
        }
        pthread_cond_broadcast(&tag_cond);
    }
    int destroy = !regen && t->destroy && t->detach;
    struct starpu_task **release = j->end_release;
    const int nrelease = j->nend_release;
    t->starpu_private = NULL;
    free(j->succ);
    free(j->prev);
    free(j);
    if (!regen) {
        rt.nsubmitted--;
        rt_ctx_count(t->sched_ctx, -1);
    }
    pthread_cond_broadcast(&rt.all_done);
    rt_unlock();
    for (int k = 0; k < nrelease; ++k) starpu_task_end_dep_release(release[k]);
    free(release);
    if (regen) {
        t->starpu_private = NULL;
        const int rc = rt_submit(t, SUBMIT_COUNTED);
        STARPU_ASSERT_MSG(rc == 0, "regenerating task %s failed (%d)", t->name ? t->name : "?", rc);
    }
    if (destroy) starpu_task_destroy(t);
    rt_drain();
}

/* Graph mode: hand the pending jobs to the CUDA driver as one graph, in a
 * topological order of their edges (submission order where it is one).
 * Jobs still waiting for a tag that has no task yet -- and every job that
 * depends on them -- stay pending for a later flush. */
void rt_flush_and_wait(void)
{
    if (!rt.graph_mode) return;
    rt_lock();
    int n = rt.npending;
    if (!n) {
        rt_unlock();
        return;
    }
    struct rt_job **pend = rt.pending;
    /* mark: 1 = in this batch, 2 = deferred */
    char *state = calloc(n, 1);
    for (int k = 0; k < n; ++k) pend[k]->graph_slot = k;
    for (int k = 0; k < n; ++k) {
        struct rt_job *j = pend[k];
        int defer = j->tag_waits > 0;
        for (int p = 0; p < j->nprev && !defer; ++p) {
            struct rt_job *q = j->prev[p];
            if (!q->terminated && q->graph_slot >= 0 && q->graph_slot < n && pend[q->graph_slot] == q &&
                state[q->graph_slot] == 2)
                defer = 1;
        }
        state[k] = defer ? 2 : 1;
    }
    /* Kahn's algorithm over in-batch edges, smallest submission index first */
    int *indeg = calloc(n, sizeof(int));
    struct rt_job **batch = malloc(sizeof *batch * n);
    struct rt_job **keep = malloc(sizeof *keep * n);
    int nb = 0, nk = 0;
    for (int k = 0; k < n; ++k) {
        if (state[k] != 1) continue;
        struct rt_job *j = pend[k];
        for (int p = 0; p < j->nprev; ++p) {
            struct rt_job *q = j->prev[p];
            if (!q->terminated && q->graph_slot >= 0 && q->graph_slot < n && pend[q->graph_slot] == q &&
                state[q->graph_slot] == 1)
                indeg[k]++;
        }
    }
    int *ready = malloc(sizeof(int) * n);
    int nr = 0;
    for (int k = 0; k < n; ++k)
        if (state[k] == 1 && indeg[k] == 0) ready[nr++] = k;
    while (nr > 0) {
        /* pop the smallest index (ready is kept sorted by insertion below) */
        int best = 0;
        for (int i = 1; i < nr; ++i)
            if (ready[i] < ready[best]) best = i;
        int k = ready[best];
        ready[best] = ready[--nr];
        batch[nb++] = pend[k];
        struct rt_job *j = pend[k];
        for (int s = 0; s < j->nsucc; ++s) {
            struct rt_job *u = j->succ[s];
            int us = u->graph_slot;
            if (us >= 0 && us < n && pend[us] == u && state[us] == 1 && --indeg[us] == 0) ready[nr++] = us;
        }
    }
    for (int k = 0; k < n; ++k)
        if (state[k] == 2) keep[nk++] = pend[k];
    STARPU_ASSERT_MSG(nb + nk == n, "task graph has a cycle");
    rt.pending = keep;
    rt.npending = nk;
    rt.cappending = n;
    for (int k = 0; k < nk; ++k) keep[k]->graph_slot = k;
    free(pend);
    free(state);
    free(indeg);
    free(ready);
    rt_unlock();
    if (nb) rt_cuda_graph_flush(batch, nb);
    free(batch);
}

int starpu_task_wait_for_all(void)
{
    if (!rt.initialized) return 0;
    rt_flush_and_wait();
    rt_lock();
    while (rt.nsubmitted > 0) pthread_cond_wait(&rt.all_done, &rt.lock);
    rt_unlock();
    return 0;
}

int starpu_task_wait_for_n_submitted(unsigned n)
{
    rt_flush_and_wait();
    rt_lock();
    while (rt.nsubmitted > (long)n) pthread_cond_wait(&rt.all_done, &rt.lock);
    rt_unlock();
    return 0;
}

int starpu_task_wait(struct starpu_task *t)
{
    rt_flush_and_wait();
    rt_lock();
    while (t->status != STARPU_TASK_FINISHED) pthread_cond_wait(&rt.all_done, &rt.lock);
    rt_unlock();
    return 0;
}

int starpu_task_wait_array(struct starpu_task **tasks, unsigned nb_tasks)
{
    for (unsigned i = 0; i < nb_tasks; ++i) {
        const int rc = starpu_task_wait(tasks[i]);
        if (rc) return rc;
    }
    return 0;
}

/* ----------------------------------------------------------- task_insert */

static int build_task(struct starpu_task *t, struct starpu_codelet *cl, va_list ap)
{
    t->cl = cl;
    int nb = 0;
    int type;
    int got_value = 0, got_cl_args = 0, bad_mix = 0; /* STARPU_VALUE and STARPU_CL_ARGS exclude each other */
    while ((type = va_arg(ap, int)) != 0) {
        if ((type & ~((1 << STARPU_MODE_SHIFT) - 1)) == 0) {
            /* an access mode (possibly with flags) followed by a handle */
            starpu_data_handle_t h = va_arg(ap, starpu_data_handle_t);
            STARPU_ASSERT_MSG(nb < STARPU_NMAXBUFS, "too many data in task_insert");
            t->handles[nb] = h;
            t->modes[nb] = (enum starpu_data_access_mode)type;
            nb++;
        } else if (type == STARPU_DATA_ARRAY) {
            starpu_data_handle_t *hs = va_arg(ap, starpu_data_handle_t *);
            int n = va_arg(ap, int);
            for (int i = 0; i < n; ++i, ++nb) {
                t->handles[nb] = hs[i];
                t->modes[nb] = cl->modes[nb];
            }
        } else if (type == STARPU_DATA_MODE_ARRAY) {
            struct starpu_data_descr *ds = va_arg(ap, struct starpu_data_descr *);
            int n = va_arg(ap, int);
            for (int i = 0; i < n; ++i, ++nb) {
                t->handles[nb] = ds[i].handle;
                t->modes[nb] = ds[i].mode;
            }
        } else if (type == STARPU_VALUE) {
            void *p = va_arg(ap, void *);
            size_t sz = va_arg(ap, size_t);
            if (got_cl_args) {
                bad_mix = 1;
                continue;
            }
            pack_value(&t->cl_arg, &t->cl_arg_size, p, sz); /* as starpu_codelet_pack_args packs */
            t->cl_arg_free = 1;
            got_value = 1;
        } else if (type == STARPU_CL_ARGS || type == STARPU_CL_ARGS_NFREE) {
            void *arg = va_arg(ap, void *);
            const size_t size = va_arg(ap, size_t);
            if (got_value) {
                bad_mix = 1;
                continue;
            }
            t->cl_arg = arg;
            t->cl_arg_size = size;
            t->cl_arg_free = type == STARPU_CL_ARGS;
            got_cl_args = 1;
        } else if (type == STARPU_CALLBACK) {
            t->callback_func = va_arg(ap, void (*)(void *));
        } else if (type == STARPU_CALLBACK_WITH_ARG) {
            t->callback_func = va_arg(ap, void (*)(void *));
            t->callback_arg = va_arg(ap, void *);
        } else if (type == STARPU_CALLBACK_ARG) {
            t->callback_arg = va_arg(ap, void *);
        } else if (type == STARPU_PROLOGUE_CALLBACK) {
            t->prologue_callback_func = va_arg(ap, void (*)(void *));
        } else if (type == STARPU_PROLOGUE_CALLBACK_ARG || type == STARPU_PROLOGUE_CALLBACK_ARG_NFREE) {
            t->prologue_callback_arg = va_arg(ap, void *);
            t->prologue_callback_arg_free = type == STARPU_PROLOGUE_CALLBACK_ARG;
        } else if (type == STARPU_PRIORITY) {
            t->priority = va_arg(ap, int);
        } else if (type == STARPU_FLOPS) {
            t->flops = va_arg(ap, double);
        } else if (type == STARPU_NAME) {
            t->name = va_arg(ap, const char *);
        } else if (type == STARPU_TAG || type == STARPU_TAG_ONLY) {
            t->tag_id = va_arg(ap, starpu_tag_t);
            t->use_tag = type == STARPU_TAG;
        } else if (type == STARPU_EXECUTE_ON_WORKER) {
            int w = va_arg(ap, int);
            if (w >= 0) {
                t->execute_on_a_specific_worker = 1;
                t->workerid = (unsigned)w;
            }
        } else if (type == STARPU_EXECUTE_WHERE) {
            t->where = (uint32_t)va_arg(ap, unsigned long long);
        } else if (type == STARPU_SCHED_CTX) {
            t->sched_ctx = va_arg(ap, unsigned);
        } else if (type == STARPU_TASK_SYNCHRONOUS) {
            t->synchronous = va_arg(ap, int);
        } else if (type == STARPU_SEQUENTIAL_CONSISTENCY) {
            t->sequential_consistency = va_arg(ap, unsigned);
        } else if (type == STARPU_TASK_COLOR) {
            (void)va_arg(ap, int);
        } else if (type == STARPU_POSSIBLY_PARALLEL) {
            (void)va_arg(ap, unsigned);
        } else if (type == STARPU_TASK_NO_SUBMITORDER) {
            t->no_submitorder = va_arg(ap, unsigned);
        } else if (type == STARPU_EXECUTE_ON_NODE || type == STARPU_EXECUTE_ON_DATA) {
            (void)va_arg(ap, void *);
        } else {
            fprintf(stderr, "[starpu_gb300] unsupported task_insert argument %d\n", type);
            return -EINVAL;
        }
    }
    if (bad_mix) {
        fprintf(stderr, "[starpu_gb300] STARPU_CL_ARGS and STARPU_VALUE cannot be used in the same call\n");
        return -EINVAL;
    }
    t->nbuffers = nb;
    if (cl && cl->nbuffers >= 0)
        STARPU_ASSERT_MSG(cl->nbuffers == nb, "codelet %s expects %d buffers, %d given", cl->name ? cl->name : "?",
                          cl->nbuffers, nb);
    return 0;
}

struct starpu_task *starpu_task_build(struct starpu_codelet *cl, ...)
{
    struct starpu_task *t = starpu_task_create();
    va_list ap;
    va_start(ap, cl);
    int rc = build_task(t, cl, ap);
    va_end(ap);
    if (rc) {
        starpu_task_destroy(t);
        return NULL;
    }
    return t;
}

static int vinsert(struct starpu_codelet *cl, va_list ap)
{
    struct starpu_task *t = starpu_task_create();
    int rc = build_task(t, cl, ap);
    if (rc) {
        starpu_task_destroy(t);
        return rc;
    }
    rc = starpu_task_submit(t);
    if (rc) starpu_task_destroy(t);
    return rc;
}

int starpu_task_insert(struct starpu_codelet *cl, ...)
{
    va_list ap;
    va_start(ap, cl);
    int rc = vinsert(cl, ap);
    va_end(ap);
    return rc;
}

int starpu_insert_task(struct starpu_codelet *cl, ...)
{
    va_list ap;
    va_start(ap, cl);
    int rc = vinsert(cl, ap);
    va_end(ap);
    return rc;
}

/* Unpack STARPU_VALUE arguments in order: each destination pointer receives
 * the bytes of the corresponding packed value. */
/* Packed STARPU_VALUE arguments (task_insert_utils.c, task_insert.c:54-104):
 * an int count, then per value its size_t length and its bytes.  Unpacking
 * fills at most `count` destinations and stops early at a 0 / NULL one, so
 * callers may or may not end their list with 0. */
static void pack_value(void **buf, size_t *size, const void *p, size_t sz)
{
    char *b = *buf;
    size_t n = *size;
    if (n == 0) {
        b = malloc(sizeof(int));
        const int zero = 0;
        memcpy(b, &zero, sizeof zero);
        n = sizeof(int);
    }
    b = realloc(b, n + sizeof sz + sz);
    memcpy(b + n, &sz, sizeof sz);
    memcpy(b + n + sizeof sz, p, sz);
    int count;
    memcpy(&count, b, sizeof count);
    ++count;
    memcpy(b, &count, sizeof count);
    *buf = b;
    *size = n + sizeof sz + sz;
}

/* returns the number of values consumed; *pos is left after them */
static int unpack_values(const char *arg, size_t *pos, int count, va_list ap)
{
    int k = 0;
    for (; k < count; ++k) {
        void *dst = va_arg(ap, void *);
        if (!dst) break;
        size_t sz;
        memcpy(&sz, arg + *pos, sizeof sz);
        memcpy(dst, arg + *pos + sizeof sz, sz);
        *pos += sizeof sz + sz;
    }
    return k;
}

void starpu_codelet_unpack_args(void *cl_arg, ...)
{
    int count;
    memcpy(&count, cl_arg, sizeof count);
    size_t pos = sizeof count;
    va_list ap;
    va_start(ap, cl_arg);
    unpack_values((const char *)cl_arg, &pos, count, ap);
    va_end(ap);
}

void starpu_codelet_pack_args(void **arg_buffer, size_t *arg_buffer_size, ...)
{
    va_list ap;
    va_start(ap, arg_buffer_size);
    void *buf = NULL;
    size_t n = 0;
    int type;
    while ((type = va_arg(ap, int)) != 0) {
        STARPU_ASSERT_MSG(type == STARPU_VALUE, "starpu_codelet_pack_args takes STARPU_VALUE arguments");
        const void *p = va_arg(ap, const void *);
        const size_t sz = va_arg(ap, size_t);
        pack_value(&buf, &n, p, sz);
    }
    va_end(ap);
    *arg_buffer = buf;
    *arg_buffer_size = n;
}

/* Unpacks the first values and writes the others, packed again (count
 * first), into `buffer` for a later starpu_codelet_unpack_args. */
void starpu_codelet_unpack_args_and_copyleft(void *cl_arg, void *buffer, size_t buffer_size, ...)
{
    const char *arg = cl_arg;
    int count;
    memcpy(&count, arg, sizeof count);
    size_t pos = sizeof count;
    va_list ap;
    va_start(ap, buffer_size);
    const int used = unpack_values(arg, &pos, count, ap);
    va_end(ap);
    if (!buffer_size) return;
    const int left = count - used;
    size_t rest = 0;
    for (int k = 0, q = (int)pos; k < left; ++k) {
        size_t sz;
        memcpy(&sz, arg + q, sizeof sz);
        rest += sizeof sz + sz;
        q += (int)(sizeof sz + sz);
    }
    STARPU_ASSERT_MSG(sizeof left + rest <= buffer_size, "%zu bytes of arguments left, the buffer holds %zu",
                      sizeof left + rest, buffer_size);
    memcpy(buffer, &left, sizeof left);
    memcpy((char *)buffer + sizeof left, arg + pos, rest);
}

/* ------------------------------------------------------- fault tolerance
 *
 * src/core/task.c:2474-2575.  starpu_task_ft_prologue, given as a task's
 * prologue callback, turns that task into a meta task: it keeps its data
 * dependencies and runs nothing (STARPU_NOWHERE); a copy submitted without
 * dependencies does the work, and the copy's callback (check_ft) either
 * releases the meta task's termination or submits another copy when the work
 * called starpu_task_ft_failed. */

static void ft_check_support(const struct starpu_task *t)
{
    for (int i = 0; i < t->nbuffers; ++i)
        STARPU_ASSERT_MSG(t->modes[i] == STARPU_R || t->modes[i] == STARPU_W,
                          "starpu_task_failed is only supported for tasks with access modes STARPU_R and STARPU_W");
}

struct starpu_task *starpu_task_ft_create_retry(const struct starpu_task *meta_task,
                                                const struct starpu_task *template_task, void (*check_ft)(void *))
{
    STARPU_ASSERT_MSG(!meta_task->cl_arg_free || !meta_task->cl_arg, "not supported yet");
    STARPU_ASSERT_MSG(!meta_task->callback_func, "not supported");
    struct starpu_task *n = starpu_task_create();
    *n = *template_task;
    n->prologue_callback_func = NULL;
    n->prologue_callback_arg = NULL;
    n->prologue_callback_arg_free = 0;
    n->cl_arg_free = 0; /* the meta task keeps its argument */
    n->callback_func = check_ft;
    n->callback_arg = (void *)meta_task;
    n->callback_arg_free = 0;
    n->use_tag = 0;
    n->synchronous = 0;
    n->destroy = 1;
    n->regenerate = 0;
    n->no_submitorder = 1;
    n->failed = 0;
    n->nb_termination_call_required = 0;
    n->declared_deps = NULL;
    n->ndeclared_deps = 0;
    n->status = STARPU_TASK_INIT;
    n->starpu_private = NULL;
    return n;
}

static void default_check_ft(void *arg)
{
    struct starpu_task *meta_task = arg;
    struct starpu_task *current = starpu_task_get_current();
    if (!current->failed) {
        starpu_task_ft_success(meta_task);
        return;
    }
    struct starpu_task *n = starpu_task_ft_create_retry(meta_task, current, default_check_ft);
    const int rc = starpu_task_submit_nodeps(n);
    STARPU_ASSERT(!rc);
}

void starpu_task_ft_prologue(void *arg)
{
    struct starpu_task *meta_task = starpu_task_get_current();
    void (*check_ft)(void *) = arg ? (void (*)(void *))arg : default_check_ft;
    struct starpu_task *n = starpu_task_ft_create_retry(meta_task, meta_task, check_ft);
    /* the meta task's termination waits for the work's success; held before
     * the work is submitted, so that a fast success cannot come first */
    starpu_task_end_dep_add(meta_task, 1);
    meta_task->where = STARPU_NOWHERE;
    const int rc = starpu_task_submit_nodeps(n);
    STARPU_ASSERT(!rc);
}

void starpu_task_ft_failed(struct starpu_task *t)
{
    ft_check_support(t);
    t->failed = 1;
}

void starpu_task_ft_success(struct starpu_task *meta_task) { starpu_task_end_dep_release(meta_task); }

void starpu_codelet_nop_func(void *descr[], void *arg)
{
    (void)descr;
    (void)arg;
}

struct starpu_codelet starpu_codelet_nop = {
    .cpu_funcs = {starpu_codelet_nop_func},
    .cuda_funcs = {starpu_codelet_nop_func},
    .nbuffers = 0,
};

/* the last task submitted with tag `id`, also once it is done; NULL when
 * none was (tags.c) */
struct starpu_task *starpu_tag_get_task(starpu_tag_t id)
{
    rt_lock();
    struct tag_entry *e = tag_get(id, 0);
    struct starpu_task *t = e ? e->task : NULL;
    rt_unlock();
    return t;
}

/* the distinct tasks that wait for `task` (submitted, not terminated):
 * their count, of which the first `ndeps` go to task_array (task.c) */
int starpu_task_get_task_succs(struct starpu_task *task, unsigned ndeps, struct starpu_task *task_array[])
{
    rt_lock();
    struct rt_job *j = task->starpu_private;
    int n = 0;
    for (int k = 0; j && k < j->nsucc; ++k) {
        struct starpu_task *u = j->succ[k]->task;
        int seen = 0;
        for (int q = 0; q < k && !seen; ++q) seen = j->succ[q]->task == u;
        if (seen) continue;
        if ((unsigned)n < ndeps) task_array[n] = u;
        ++n;
    }
    rt_unlock();
    return n;
}
