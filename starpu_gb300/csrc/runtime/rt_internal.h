/*
 * Internal structures of the StarPU-API runtime of libstarpu_gb300.so.
 *
 * Design (GB300-first rather than a port of StarPU's runtime):
 *  - one global runtime lock protects handles, dependencies and queues (the
 *    submission loop is single-threaded and tasks are coarse tiles);
 *  - data handles hold one interface per memory node (node 0 = host RAM,
 *    node 1 = the GPU); tiles of a partitioned matrix are views into their
 *    root's buffer on every node, so the root is one allocation in HBM and a
 *    whole factorisation can run in place;
 *  - sequential consistency (last writer + readers since) gives the implicit
 *    RAW / WAR / WAW edges of StarPU's core/dependencies/implicit_data_deps.c;
 *  - workers: host threads running cpu_funcs, and one CUDA worker per GPU
 *    that either runs ready tasks one by one on its stream (StarPU's driver)
 *    or, when every worker is a CUDA worker, records the whole DAG submitted
 *    before a synchronisation point as one CUDA graph (stream capture over a
 *    pool of streams, one event per task for the edges) and launches it;
 *  - scheduling: dmda-style (expected finish time = worker availability +
 *    transfer + history-model length), priority-ordered worker queues;
 *  - history perfmodels per (symbol, architecture combination,
 *    implementation, footprint), persisted in the version-45 text layout
 *    under $STARPU_PERF_MODEL_DIR/codelets/45/ (rt_perfmodel.c).
 */
#ifndef RT_INTERNAL_H
#define RT_INTERNAL_H

#include <pthread.h>
#include <stdint.h>

#include "starpu.h"

#define RT_NODES 2
#define RT_NODE_RAM 0
#define RT_NODE_GPU 1

struct rt_job;

struct _starpu_data_state {
    enum starpu_data_interface_id id;
    int home_node;
    size_t elemsize;
    struct starpu_matrix_interface mat[RT_NODES];    /* matrix / vector views per node */
    struct starpu_variable_interface var[RT_NODES];  /* variable per node */
    struct starpu_vector_interface vec[RT_NODES];    /* a vector's codelet view of mat[] */
    int valid[RT_NODES];
    int allocated[RT_NODES];
    void *owned[RT_NODES];      /* buffers this handle allocated (roots only) */
    size_t owned_size[RT_NODES];
    struct _starpu_data_state *parent, *root;
    size_t row_off, col_off;    /* element offsets of this view inside the root */
    unsigned nchildren;
    struct _starpu_data_state **children;
    int partitioned;
    /* sequential consistency */
    int seq_consistency;        /* implicit dependencies on this handle (inherited by children) */
    struct rt_job *last_writer;
    struct rt_job **readers;
    int nreaders, capreaders;
    /* STARPU_COMMUTE writers since the last plain writer (rt.relaxed_commute):
     * unordered among themselves, run one at a time (commute_busy) */
    struct rt_job **commuters;
    int ncommuters, capcommuters;
    int commute_busy;
    struct starpu_task **acquired;  /* pending starpu_data_acquire_cb accesses, released in order */
    int nacquired, capacquired;
    char name[48];
};

struct rt_job {
    struct starpu_task *task;
    uint64_t seq;
    int ndeps;
    struct rt_job **succ;
    int nsucc, capsucc;
    int nprev_graph;            /* graph mode: predecessors still pending in the same flush */
    struct rt_job **prev;       /* graph mode: predecessors (for event edges) */
    int nprev, capprev;
    int terminated;
    int worker;
    double predicted;           /* us */
    double start_us;
    int graph_slot;             /* graph mode: index in the flush */
    int stream_slot;
    int heap_index;
    starpu_tag_t tag;
    int has_tag;
    int tag_waits;              /* tags awaited whose task is not submitted yet */
    int prologue_done;
    struct rt_job *defer_next;  /* queue of ready jobs whose prologue / NOWHERE step runs unlocked */
    struct starpu_task **end_release; /* tasks whose termination also waits for this one */
    int nend_release, capend_release;
};

struct rt_worker {
    int id;
    enum starpu_worker_archtype type;
    int devid;
    struct starpu_perfmodel_arch arch;
    struct starpu_perfmodel_device dev;
    pthread_t thread;
    pthread_cond_t cond;
    struct rt_job **heap;       /* ready queue, max priority first */
    int hn, hcap;
    double expected_end;        /* us, dmda availability */
    unsigned long ntasks;
};

struct rt_state {
    int initialized;
    int shutting_down;
    pthread_mutex_t lock;
    pthread_cond_t all_done;
    struct rt_worker workers[STARPU_NMAXWORKERS];
    int nworkers, ncpu, ncuda;
    int graph_mode;             /* CUDA-only runs: whole-DAG CUDA graphs */
    int default_seq_consistency;
    int relaxed_commute;        /* STARPU_COMMUTE writers unordered (runs without a CUDA worker) */
    pthread_cond_t commute_cond;
    int paused;
    uint64_t seq;
    long nsubmitted;            /* submitted and not terminated */
    int min_prio, max_prio;
    unsigned calibrate;
    double transfer_us_per_byte;
    /* graph mode: jobs submitted since the last flush, in submission order */
    struct rt_job **pending;
    int npending, cappending;
    /* ready jobs with a prologue callback to run or no worker to run on
     * (STARPU_NOWHERE): handled by rt_drain outside the lock */
    struct rt_job *defer_head, *defer_tail;
    struct starpu_gb300_runtime_stats stats;
};

extern struct rt_state rt;

/* rt_core.c */
void rt_lock(void);
void rt_unlock(void);
int rt_current_worker(void);
void rt_set_current_worker(int id);
struct starpu_task *rt_current_task_get(void);
void rt_current_task_set(struct starpu_task *t);

/* rt_data.c */
int rt_data_node_ready(starpu_data_handle_t h, int node);
int rt_data_fetch(starpu_data_handle_t h, int node, enum starpu_data_access_mode mode, void *stream);
void rt_data_after_write(starpu_data_handle_t h, int node);
void *rt_data_interface(starpu_data_handle_t h, int node);
size_t rt_data_size(starpu_data_handle_t h);
uint32_t rt_data_footprint(starpu_data_handle_t h);
void rt_data_forget_job(starpu_data_handle_t h, struct rt_job *j);

/* rt_task.c */
void rt_job_terminate(struct rt_job *j, double measured_us);
int rt_can_execute(struct rt_worker *w, struct starpu_task *t);
void rt_flush_and_wait(void);

/* rt_core.c: scheduling contexts (rt_ctx_has_worker / rt_ctx_count with the
 * runtime lock held) */
unsigned rt_ctx_resolve(struct starpu_task *t);
int rt_ctx_has_worker(unsigned ctx, int worker);
void rt_ctx_count(unsigned ctx, int delta);
void rt_ctx_reset(void);

/* rt_task.c: the busy flags of a task's STARPU_COMMUTE handles (runtime lock held) */
void rt_commute_acquire(struct starpu_task *t);
void rt_commute_release(struct starpu_task *t);

/* rt_task.c: runs the deferred prologues and NOWHERE terminations; call it
 * without the lock after any section that may have pushed jobs */
void rt_drain(void);

/* rt_sched.c */
void rt_sched_push(struct rt_job *j);
struct rt_job *rt_sched_pop(struct rt_worker *w);
void rt_perfmodel_feedback(struct starpu_task *t, struct starpu_perfmodel_arch *arch, double us);
void rt_perfmodel_init(void);
void rt_perfmodel_save_all(void);

/* rt_cuda.c */
int rt_cuda_init(int ncuda);
void rt_cuda_shutdown(void);
void *rt_cuda_worker_main(void *arg);
int rt_cuda_graph_flush(struct rt_job **jobs, int n);
int rt_cuda_copy_2d(int to_gpu, void *dst, size_t dld, const void *src, size_t sld, size_t width_bytes, size_t rows,
                    void *stream);
void *rt_cuda_alloc(size_t bytes);
void rt_cuda_free(void *p);
void *rt_cuda_transfer_stream(void);
int rt_cuda_sync_transfer_stream(void);
int rt_cuda_host_alloc(void **p, size_t bytes);
void rt_cuda_host_free(void *p);

/* rt_cpu.c */
void *rt_cpu_worker_main(void *arg);

#endif /* RT_INTERNAL_H */
