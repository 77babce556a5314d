/*
 * CUDA driver of the runtime (the counterpart of src/drivers/cuda/driver_cuda.c).
 *
 * Per-task mode (CPU and CUDA workers together, or STARPU_GB300_GRAPH=0):
 * the worker thread runs ready tasks on its own non-blocking stream with up to
 * STARPU_CUDA_PIPELINE (default 2) tasks in flight, stages input tiles with
 * 2D copies on that stream, brackets every codelet call with CUDA events and
 * feeds the measured time to the history model (driver_cuda.c:2135-2303).
 *
 * Graph mode (every worker is a CUDA worker): the tasks submitted before a
 * synchronisation point form one DAG; the data it reads are staged (a whole
 * partitioned matrix in one copy when possible), then the DAG is recorded as a
 * CUDA graph by stream capture: each task's codelet enqueues its kernels on a
 * stream of a pool, edges between tasks on different streams are event waits,
 * and the graph is instantiated and launched once.  Independent tasks of the
 * DAG therefore run concurrently on the device, and the per-task host work of
 * the reference driver (event polling, job bookkeeping) leaves the critical path.
 */
#include <cuda_runtime_api.h>

#include "rt_internal.h"

#define POOL_STREAMS 8

static __thread cudaStream_t tls_stream = NULL;
static cudaStream_t transfer_stream = NULL;
static cudaStream_t capture_origin = NULL;
static cudaStream_t pool[POOL_STREAMS];
static cudaEvent_t *ev_pool = NULL;
static int ev_pool_n = 0;
static int cuda_ndev = 0;

cudaStream_t starpu_cuda_get_local_stream(void) { return tls_stream; }

void starpu_cuda_report_error(const char *func, const char *file, int line, cudaError_t status)
{
    starpu_gb300_abort_msg(file, line, func, "CUDA error %d: %s", (int)status, cudaGetErrorString(status));
}

int rt_cuda_init(int ncuda)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return 0;
    }
    if (ncuda > count) ncuda = count;
    if (ncuda > 1) ncuda = 1; /* one GPU per process: the multi-GPU path is replicas */
    if (cudaSetDevice(0) != cudaSuccess) return 0;
    if (cudaStreamCreateWithFlags(&transfer_stream, cudaStreamNonBlocking) != cudaSuccess) return 0;
    cudaStreamCreateWithFlags(&capture_origin, cudaStreamNonBlocking);
    for (int i = 0; i < POOL_STREAMS; ++i) cudaStreamCreateWithFlags(&pool[i], cudaStreamNonBlocking);
    cuda_ndev = ncuda;
    return ncuda;
}

void rt_cuda_shutdown(void)
{
    if (!cuda_ndev) return;
    for (int i = 0; i < ev_pool_n; ++i) cudaEventDestroy(ev_pool[i]);
    free(ev_pool);
    ev_pool = NULL;
    ev_pool_n = 0;
    for (int i = 0; i < POOL_STREAMS; ++i) cudaStreamDestroy(pool[i]);
    cudaStreamDestroy(capture_origin);
    cudaStreamDestroy(transfer_stream);
    cuda_ndev = 0;
}

void *rt_cuda_alloc(size_t bytes)
{
    void *p = NULL;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return NULL;
    }
    return p;
}

void rt_cuda_free(void *p) { cudaFree(p); }

int rt_cuda_host_alloc(void **p, size_t bytes)
{
    if (cudaMallocHost(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return 0;
}

void rt_cuda_host_free(void *p) { cudaFreeHost(p); }

void *rt_cuda_transfer_stream(void) { return transfer_stream; }

int rt_cuda_sync_transfer_stream(void) { return cudaStreamSynchronize(transfer_stream) == cudaSuccess ? 0 : -EIO; }

int rt_cuda_copy_2d(int to_gpu, void *dst, size_t dld, const void *src, size_t sld, size_t width_bytes, size_t rows,
                    void *stream)
{
    cudaError_t e = cudaMemcpy2DAsync(dst, dld, src, sld, width_bytes, rows,
                                      to_gpu ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                                      stream ? (cudaStream_t)stream : transfer_stream);
    return e == cudaSuccess ? 0 : -EIO;
}

/* ------------------------------------------------------ per-task mode */

struct inflight {
    struct rt_job *j;
    cudaEvent_t e0, e1;
};

static void stage_for_gpu(struct rt_job *j, cudaStream_t s)
{
    struct starpu_task *t = j->task;
    for (int i = 0; i < t->nbuffers; ++i) {
        starpu_data_handle_t h = t->handles[i];
        if (!h) continue;
        int rc = rt_data_fetch(h, RT_NODE_GPU, t->modes[i], s);
        STARPU_ASSERT_MSG(rc == 0, "cannot fetch data %d of task %s to the GPU (%d)", i, t->name ? t->name : "?", rc);
        t->interfaces[i] = rt_data_interface(h, RT_NODE_GPU);
    }
}

static void complete(struct rt_worker *w, struct inflight *f)
{
    cudaEventSynchronize(f->e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, f->e0, f->e1);
    struct starpu_task *t = f->j->task;
    rt_lock();
    for (int i = 0; i < t->nbuffers; ++i)
        if (t->handles[i] && (t->modes[i] & STARPU_W)) rt_data_after_write(t->handles[i], RT_NODE_GPU);
    rt.stats.tasks_cuda++;
    w->ntasks++;
    rt_unlock();
    rt_job_terminate(f->j, (double)ms * 1e3);
}

void *rt_cuda_worker_main(void *arg)
{
    struct rt_worker *w = arg;
    rt_set_current_worker(w->id);
    cudaSetDevice(w->devid);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    tls_stream = s;
    int depth = 2;
    const char *p = getenv("STARPU_CUDA_PIPELINE");
    if (p && atoi(p) > 0) depth = atoi(p);
    if (depth > 16) depth = 16;
    struct inflight fl[16];
    for (int i = 0; i < depth; ++i) {
        cudaEventCreate(&fl[i].e0);
        cudaEventCreate(&fl[i].e1);
    }
    int head = 0, count = 0;
    rt_lock();
    for (;;) {
        struct rt_job *j = (count < depth) ? rt_sched_pop(w) : NULL;
        if (!j) {
            if (count > 0) {
                rt_unlock();
                complete(w, &fl[head]);
                head = (head + 1) % depth;
                count--;
                rt_lock();
                continue;
            }
            if (rt.shutting_down) break;
            pthread_cond_wait(&w->cond, &rt.lock);
            continue;
        }
        stage_for_gpu(j, s);
        rt_unlock();
        struct inflight *f = &fl[(head + count) % depth];
        f->j = j;
        struct starpu_task *t = j->task;
        rt_current_task_set(t);
        cudaEventRecord(f->e0, s);
        t->cl->cuda_funcs[0](t->interfaces, t->cl_arg);
        cudaEventRecord(f->e1, s);
        rt_current_task_set(NULL);
        if (!(t->cl->cuda_flags[0] & STARPU_CUDA_ASYNC)) cudaStreamSynchronize(s);
        count++;
        rt_lock();
    }
    rt_unlock();
    for (int i = 0; i < depth; ++i) {
        cudaEventDestroy(fl[i].e0);
        cudaEventDestroy(fl[i].e1);
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return NULL;
}

/* --------------------------------------------------------- graph mode */

static void ensure_events(int n)
{
    if (ev_pool_n >= n) return;
    ev_pool = realloc(ev_pool, sizeof *ev_pool * n);
    for (int i = ev_pool_n; i < n; ++i) cudaEventCreateWithFlags(&ev_pool[i], cudaEventDisableTiming);
    ev_pool_n = n;
}

/* One copy for a whole partitioned root whose every leaf must move host -> GPU. */
static int leaves_need_h2d(starpu_data_handle_t h)
{
    if (!h->partitioned) return h->valid[RT_NODE_RAM] && !h->valid[RT_NODE_GPU];
    for (unsigned i = 0; i < h->nchildren; ++i)
        if (!leaves_need_h2d(h->children[i])) return 0;
    return 1;
}

static void mark_leaves(starpu_data_handle_t h)
{
    if (!h->partitioned) {
        h->valid[RT_NODE_GPU] = 1;
        return;
    }
    for (unsigned i = 0; i < h->nchildren; ++i) mark_leaves(h->children[i]);
}

static void bulk_stage(struct rt_job **jobs, int n, cudaStream_t s)
{
    for (int k = 0; k < n; ++k) {
        struct starpu_task *t = jobs[k]->task;
        for (int i = 0; i < t->nbuffers; ++i) {
            starpu_data_handle_t h = t->handles[i];
            if (!h || h->root == h || h->id == STARPU_VARIABLE_INTERFACE_ID) continue;
            struct _starpu_data_state *r = h->root;
            if (!r->partitioned || !leaves_need_h2d(r)) continue;
            /* allocate the root on the GPU through one of its leaves, then copy the root */
            if (rt_data_fetch(h, RT_NODE_GPU, STARPU_W, s)) continue;
            size_t es = r->elemsize;
            if (rt_cuda_copy_2d(1, (void *)r->mat[RT_NODE_GPU].ptr, r->mat[RT_NODE_GPU].ld * es,
                                (const void *)r->mat[RT_NODE_RAM].ptr, r->mat[RT_NODE_RAM].ld * es,
                                r->mat[0].nx * es, r->mat[0].ny, s) == 0) {
                mark_leaves(r);
                rt.stats.h2d_bytes += r->mat[0].nx * r->mat[0].ny * es;
            }
        }
    }
}

static void run_sequential(struct rt_job **jobs, int n, cudaStream_t s)
{
    tls_stream = s;
    for (int k = 0; k < n; ++k) {
        struct starpu_task *t = jobs[k]->task;
        rt_current_task_set(t);
        t->cl->cuda_funcs[0](t->interfaces, t->cl_arg);
        rt_current_task_set(NULL);
        if (!(t->cl->cuda_flags[0] & STARPU_CUDA_ASYNC)) cudaStreamSynchronize(s);
    }
    cudaStreamSynchronize(s);
    rt.stats.tasks_cuda += n;
}

int rt_cuda_graph_flush(struct rt_job **jobs, int n)
{
    cudaSetDevice(rt.workers[0].devid);
    int prev_worker = rt_current_worker();
    cudaStream_t prev_stream = tls_stream;
    rt_set_current_worker(rt.workers[0].id);
    cudaStream_t origin = capture_origin;

    /* 1. stage inputs and simulate the writes in submission order */
    rt_lock();
    bulk_stage(jobs, n, origin);
    int all_async = 1;
    for (int k = 0; k < n; ++k) {
        struct starpu_task *t = jobs[k]->task;
        stage_for_gpu(jobs[k], origin);
        for (int i = 0; i < t->nbuffers; ++i)
            if (t->handles[i] && (t->modes[i] & STARPU_W)) rt_data_after_write(t->handles[i], RT_NODE_GPU);
        if (!t->cl || !t->cl->cuda_funcs[0]) STARPU_ABORT_MSG("graph mode: task %s has no CUDA implementation", t->name ? t->name : "?");
        all_async &= (t->cl->cuda_flags[0] & STARPU_CUDA_ASYNC) != 0;
    }
    rt_unlock();

    double t_build0 = starpu_timing_now();
    int graphed = 0;
    cudaGraph_t graph = NULL;
    cudaGraphExec_t exec = NULL;
    if (all_async) {
        ensure_events(n + POOL_STREAMS + 1);
        int *stream_of = malloc(sizeof(int) * n);
        int tail[POOL_STREAMS];
        int used[POOL_STREAMS];
        for (int i = 0; i < POOL_STREAMS; ++i) {
            tail[i] = -1;
            used[i] = 0;
        }
        cudaEvent_t fork = ev_pool[n];
        int rr = 0;
        cudaError_t err = cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) err = cudaEventRecord(fork, origin);
        for (int k = 0; k < n && err == cudaSuccess; ++k) {
            struct rt_job *j = jobs[k];
            j->graph_slot = k;
            /* prefer the stream whose last task is one of our predecessors */
            int s = -1;
            for (int p = j->nprev - 1; p >= 0 && s < 0; --p) {
                int ps = stream_of[j->prev[p]->graph_slot];
                if (tail[ps] == j->prev[p]->graph_slot) s = ps;
            }
            if (s < 0) {
                s = rr;
                rr = (rr + 1) % POOL_STREAMS;
            }
            if (!used[s]) {
                err = cudaStreamWaitEvent(pool[s], fork, 0);
                used[s] = 1;
            }
            for (int p = 0; p < j->nprev && err == cudaSuccess; ++p) {
                int ps = j->prev[p]->graph_slot;
                if (stream_of[ps] != s || tail[s] != ps) err = cudaStreamWaitEvent(pool[s], ev_pool[ps], 0);
            }
            if (err != cudaSuccess) break;
            tls_stream = pool[s];
            struct starpu_task *t = j->task;
            rt_current_task_set(t);
            t->cl->cuda_funcs[0](t->interfaces, t->cl_arg);
            rt_current_task_set(NULL);
            err = cudaEventRecord(ev_pool[k], pool[s]);
            stream_of[k] = s;
            tail[s] = k;
        }
        for (int i = 0; i < POOL_STREAMS && err == cudaSuccess; ++i) {
            if (!used[i]) continue;
            cudaEvent_t jn = ev_pool[n + 1 + i];  /* join events follow the fork event */
            err = cudaEventRecord(jn, pool[i]);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(origin, jn, 0);
        }
        cudaError_t e2 = cudaStreamEndCapture(origin, &graph);
        if (err == cudaSuccess) err = e2;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&exec, graph, 0);
        free(stream_of);
        if (err == cudaSuccess) {
            graphed = 1;
        } else {
            cudaGetLastError();
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            exec = NULL;
            graph = NULL;
            fprintf(stderr, "[starpu_gb300] graph capture failed (%s); running the %d tasks one by one\n",
                    cudaGetErrorString(err), n);
        }
    }
    double t_build1 = starpu_timing_now();
    if (graphed) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, origin);
        cudaGraphLaunch(exec, origin);
        cudaEventRecord(b, origin);
        cudaStreamSynchronize(origin);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        rt_lock();
        rt.stats.graphs_launched++;
        rt.stats.tasks_graph += n;
        rt.stats.graph_build_us += t_build1 - t_build0;
        rt.stats.graph_exec_us += ms * 1e3;
        rt_unlock();
    } else {
        run_sequential(jobs, n, origin);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) starpu_cuda_report_error(__func__, __FILE__, __LINE__, e);
    tls_stream = prev_stream;
    rt_set_current_worker(prev_worker);
    for (int k = 0; k < n; ++k) rt_job_terminate(jobs[k], 0.0);
    return 0;
}
