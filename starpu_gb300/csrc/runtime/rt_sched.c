/*
 * dmda scheduling and history-based performance models.
 *
 * Push (src/sched_policies/deque_modeling_policy_data_aware.c:604 semantics):
 * for every worker able to run the task, fitness = the worker's expected
 * availability + the expected transfer time of the data not valid on its
 * memory node + the expected length from the codelet's performance model
 * (history, regression or cost function, for the worker); the task goes to
 * the worker with the smallest fitness (uncalibrated archs predict 0, so they
 * get tasks and calibrate).  Each worker pops its queue by priority, then
 * submission order.
 *
 * The performance models the expected lengths come from are in rt_perfmodel.c.
 */
#include <math.h>
#include <sys/stat.h>
#include <unistd.h>

#include "rt_internal.h"

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
    /* a prologue callback runs as the task becomes ready, before it is
     * scheduled (sched_policy.c:583-588); a STARPU_NOWHERE task needs no
     * worker.  Both may call back into the runtime: rt_drain takes them
     * outside the lock. */
    if ((t->prologue_callback_func && !j->prologue_done) || t->where == STARPU_NOWHERE) {
        j->defer_next = NULL;
        if (rt.defer_tail) rt.defer_tail->defer_next = j;
        else rt.defer_head = j;
        rt.defer_tail = j;
        return;
    }
    double now = starpu_timing_now();
    int best = -1;
    double best_fit = INFINITY, best_len = 0;
    for (int i = 0; i < rt.nworkers; ++i) {
        struct rt_worker *w = &rt.workers[i];
        if (!rt_can_execute(w, t) || !rt_ctx_has_worker(t->sched_ctx, i)) continue;
        double len = starpu_task_worker_expected_length(t, (unsigned)i, 0, 0);
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

/* ------------------------------------------------------- transfer model */

double starpu_task_expected_data_transfer_time(unsigned memory_node, struct starpu_task *task)
{
    double bytes = 0;
    int node = memory_node == STARPU_MAIN_RAM ? RT_NODE_RAM : RT_NODE_GPU;
    for (int i = 0; i < task->nbuffers; ++i)
        if (task->handles[i] && (task->modes[i] & STARPU_R) && !task->handles[i]->valid[node])
            bytes += (double)rt_data_size(task->handles[i]);
    return bytes * rt.transfer_us_per_byte;
}
