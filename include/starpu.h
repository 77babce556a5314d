/*
 * starpu.h -- StarPU C API subset implemented by libstarpu_gb300.so.
 *
 * These are this project's own declarations of the part of StarPU's public
 * API that the tiled Cholesky drivers use (examples/cholesky/cholesky_implicit.c,
 * cholesky_kernels.c, examples/sched_ctx_utils/sched_ctx_utils.c and
 * examples/common/blas.c), so that those sources compile and link unchanged.
 * Names, constants, struct field names and semantics follow StarPU's
 * include/starpu_task.h, starpu_task_util.h, starpu_data.h,
 * starpu_data_interfaces.h, starpu_data_filters.h, starpu_perfmodel.h,
 * starpu_sched_ctx.h, starpu_stdlib.h, starpu_util.h and starpu_thread_util.h;
 * binary layouts are this library's own (sources are recompiled against it).
 */
#ifndef STARPU_H
#define STARPU_H

#include <assert.h>
#include <errno.h>
#include <limits.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "starpu_config.h"

#ifdef STARPU_USE_CUDA
#include <cuda_runtime.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ====================================================================== util */

#define STARPU_ATTRIBUTE_UNUSED __attribute__((unused))
#define STARPU_ATTRIBUTE_NORETURN __attribute__((noreturn))
#define STARPU_MIN(a, b) ((a) < (b) ? (a) : (b))
#define STARPU_MAX(a, b) ((a) < (b) ? (b) : (a))
#define STARPU_UNLIKELY(x) __builtin_expect(!!(x), 0)
#define STARPU_LIKELY(x) __builtin_expect(!!(x), 1)

void starpu_gb300_abort_msg(const char *file, int line, const char *func, const char *fmt, ...)
    __attribute__((noreturn, format(printf, 4, 5)));

#define STARPU_ABORT() starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, "aborted")
#define STARPU_ABORT_MSG(...) starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, __VA_ARGS__)
#define STARPU_ASSERT(x)                                                                                  \
    do {                                                                                                  \
        if (STARPU_UNLIKELY(!(x))) starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, "assertion `%s' failed", #x); \
    } while (0)
#define STARPU_ASSERT_MSG(x, ...)                                                                         \
    do {                                                                                                  \
        if (STARPU_UNLIKELY(!(x))) starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, __VA_ARGS__);     \
    } while (0)
#define STARPU_CHECK_RETURN_VALUE(err, message)                                                           \
    do {                                                                                                  \
        if (STARPU_UNLIKELY((err) != 0))                                                                  \
            starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, "unexpected value %d returned by %s",   \
                                   (int)(err), message);                                                   \
    } while (0)
#define STARPU_CHECK_RETURN_VALUE_IS(err, value, message)                                                 \
    do {                                                                                                  \
        if (STARPU_UNLIKELY((err) != (value)))                                                            \
            starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, "unexpected value %d returned by %s",   \
                                   (int)(err), message);                                                   \
    } while (0)

/* microseconds since an arbitrary origin (CLOCK_MONOTONIC) */
double starpu_timing_now(void);

/* =================================================================== threads */

typedef pthread_t starpu_pthread_t;
typedef pthread_attr_t starpu_pthread_attr_t;
typedef pthread_mutex_t starpu_pthread_mutex_t;
typedef pthread_mutexattr_t starpu_pthread_mutexattr_t;
typedef pthread_cond_t starpu_pthread_cond_t;
typedef pthread_key_t starpu_pthread_key_t;
typedef pthread_barrier_t starpu_pthread_barrier_t;

#define _STARPU_PTHREAD_CHECK(call, what)                                                                 \
    do {                                                                                                  \
        int _p_ret = (call);                                                                              \
        if (STARPU_UNLIKELY(_p_ret != 0))                                                                 \
            starpu_gb300_abort_msg(__FILE__, __LINE__, __func__, "%s failed: %s", what, strerror(_p_ret)); \
    } while (0)
#define STARPU_PTHREAD_CREATE(thread, attr, routine, arg) \
    _STARPU_PTHREAD_CHECK(pthread_create(thread, attr, routine, arg), "pthread_create")
#define STARPU_PTHREAD_JOIN(thread, retval) _STARPU_PTHREAD_CHECK(pthread_join(thread, retval), "pthread_join")
#define STARPU_PTHREAD_MUTEX_INITIALIZER PTHREAD_MUTEX_INITIALIZER
#define STARPU_PTHREAD_COND_INITIALIZER PTHREAD_COND_INITIALIZER
#define STARPU_PTHREAD_MUTEX_INIT(mutex, attr) _STARPU_PTHREAD_CHECK(pthread_mutex_init(mutex, attr), "pthread_mutex_init")
#define STARPU_PTHREAD_MUTEX_DESTROY(mutex) _STARPU_PTHREAD_CHECK(pthread_mutex_destroy(mutex), "pthread_mutex_destroy")
#define STARPU_PTHREAD_MUTEX_LOCK(mutex) _STARPU_PTHREAD_CHECK(pthread_mutex_lock(mutex), "pthread_mutex_lock")
#define STARPU_PTHREAD_MUTEX_UNLOCK(mutex) _STARPU_PTHREAD_CHECK(pthread_mutex_unlock(mutex), "pthread_mutex_unlock")
#define STARPU_PTHREAD_COND_INIT(cond, attr) _STARPU_PTHREAD_CHECK(pthread_cond_init(cond, attr), "pthread_cond_init")
#define STARPU_PTHREAD_COND_DESTROY(cond) _STARPU_PTHREAD_CHECK(pthread_cond_destroy(cond), "pthread_cond_destroy")
#define STARPU_PTHREAD_COND_SIGNAL(cond) _STARPU_PTHREAD_CHECK(pthread_cond_signal(cond), "pthread_cond_signal")
#define STARPU_PTHREAD_COND_BROADCAST(cond) _STARPU_PTHREAD_CHECK(pthread_cond_broadcast(cond), "pthread_cond_broadcast")
#define STARPU_PTHREAD_COND_WAIT(cond, mutex) _STARPU_PTHREAD_CHECK(pthread_cond_wait(cond, mutex), "pthread_cond_wait")
#define STARPU_PTHREAD_KEY_CREATE(key, destr) _STARPU_PTHREAD_CHECK(pthread_key_create(key, destr), "pthread_key_create")
#define STARPU_PTHREAD_KEY_DELETE(key) _STARPU_PTHREAD_CHECK(pthread_key_delete(key), "pthread_key_delete")
#define STARPU_PTHREAD_SETSPECIFIC(key, ptr) _STARPU_PTHREAD_CHECK(pthread_setspecific(key, ptr), "pthread_setspecific")
#define STARPU_PTHREAD_GETSPECIFIC(key) pthread_getspecific(key)
#define STARPU_PTHREAD_BARRIER_INIT(b, attr, count) _STARPU_PTHREAD_CHECK(pthread_barrier_init(b, attr, count), "pthread_barrier_init")
#define STARPU_PTHREAD_BARRIER_DESTROY(b) _STARPU_PTHREAD_CHECK(pthread_barrier_destroy(b), "pthread_barrier_destroy")
#define STARPU_PTHREAD_BARRIER_WAIT(b) do { int _bw = pthread_barrier_wait(b); STARPU_ASSERT(_bw == 0 || _bw == PTHREAD_BARRIER_SERIAL_THREAD); } while (0)

/* ====================================================================== data */

#define STARPU_MAIN_RAM 0

enum starpu_data_access_mode {
    STARPU_NONE = 0,
    STARPU_R = (1 << 0),
    STARPU_W = (1 << 1),
    STARPU_RW = (STARPU_R | STARPU_W),
    STARPU_SCRATCH = (1 << 2),
    STARPU_REDUX = (1 << 3),
    STARPU_COMMUTE = (1 << 4),
    STARPU_SSEND = (1 << 5),
    STARPU_LOCALITY = (1 << 6),
    STARPU_MPI_REDUX = (1 << 7),
    STARPU_NOPLAN = (1 << 8),
    STARPU_UNMAP = (1 << 9),
    STARPU_NOFOOTPRINT = (1 << 10),
    STARPU_ACCESS_MODE_MAX = (1 << 11)
};

struct _starpu_data_state;
typedef struct _starpu_data_state *starpu_data_handle_t;

enum starpu_data_interface_id {
    STARPU_UNKNOWN_INTERFACE_ID = -1,
    STARPU_MATRIX_INTERFACE_ID = 0,
    STARPU_BLOCK_INTERFACE_ID = 1,
    STARPU_VECTOR_INTERFACE_ID = 2,
    STARPU_CSR_INTERFACE_ID = 3,
    STARPU_BCSR_INTERFACE_ID = 4,
    STARPU_VARIABLE_INTERFACE_ID = 5,
    STARPU_VOID_INTERFACE_ID = 6,
    STARPU_MULTIFORMAT_INTERFACE_ID = 7,
    STARPU_COO_INTERFACE_ID = 8,
    STARPU_TENSOR_INTERFACE_ID = 9,
    STARPU_NDIM_INTERFACE_ID = 10,
    STARPU_MAX_INTERFACE_ID = 11
};

/* Dense matrix: nx elements along x (contiguous), ny along y, ld elements
 * between the starts of consecutive y indices (column-major: nx = rows). */
struct starpu_matrix_interface {
    enum starpu_data_interface_id id;
    uintptr_t ptr;
    uintptr_t dev_handle;
    size_t offset;
    size_t nx;
    size_t ny;
    size_t ld;
    size_t elemsize;
    size_t allocsize;
};

struct starpu_variable_interface {
    enum starpu_data_interface_id id;
    uintptr_t ptr;
    uintptr_t dev_handle;
    size_t offset;
    size_t elemsize;
};

struct starpu_vector_interface {
    enum starpu_data_interface_id id;
    uintptr_t ptr;
    uintptr_t dev_handle;
    size_t offset;
    size_t nx;
    size_t elemsize;
    size_t allocsize;
    size_t slice_base;
};

#define STARPU_MATRIX_GET_PTR(interface) (((struct starpu_matrix_interface *)(interface))->ptr)
#define STARPU_MATRIX_GET_DEV_HANDLE(interface) (((struct starpu_matrix_interface *)(interface))->dev_handle)
#define STARPU_MATRIX_GET_OFFSET(interface) (((struct starpu_matrix_interface *)(interface))->offset)
#define STARPU_MATRIX_GET_NX(interface) (((struct starpu_matrix_interface *)(interface))->nx)
#define STARPU_MATRIX_GET_NY(interface) (((struct starpu_matrix_interface *)(interface))->ny)
#define STARPU_MATRIX_GET_LD(interface) (((struct starpu_matrix_interface *)(interface))->ld)
#define STARPU_MATRIX_GET_ELEMSIZE(interface) (((struct starpu_matrix_interface *)(interface))->elemsize)
#define STARPU_MATRIX_GET_ALLOCSIZE(interface) (((struct starpu_matrix_interface *)(interface))->allocsize)
#define STARPU_VARIABLE_GET_PTR(interface) (((struct starpu_variable_interface *)(interface))->ptr)
#define STARPU_VARIABLE_GET_OFFSET(interface) (((struct starpu_variable_interface *)(interface))->offset)
#define STARPU_VARIABLE_GET_ELEMSIZE(interface) (((struct starpu_variable_interface *)(interface))->elemsize)
#define STARPU_VARIABLE_GET_DEV_HANDLE(interface) (((struct starpu_variable_interface *)(interface))->dev_handle)
#define STARPU_VECTOR_GET_PTR(interface) (((struct starpu_vector_interface *)(interface))->ptr)
#define STARPU_VECTOR_GET_NX(interface) (((struct starpu_vector_interface *)(interface))->nx)
#define STARPU_VECTOR_GET_ELEMSIZE(interface) (((struct starpu_vector_interface *)(interface))->elemsize)

/* registration (home_node = STARPU_MAIN_RAM, or -1 for data without a home copy) */
void starpu_matrix_data_register(starpu_data_handle_t *handle, int home_node, uintptr_t ptr, size_t ld, size_t nx,
                                 size_t ny, size_t elemsize);
void starpu_variable_data_register(starpu_data_handle_t *handle, int home_node, uintptr_t ptr, size_t size);
void starpu_vector_data_register(starpu_data_handle_t *handle, int home_node, uintptr_t ptr, size_t nx,
                                 size_t elemsize);
void starpu_data_unregister(starpu_data_handle_t handle);
void starpu_data_unregister_no_coherency(starpu_data_handle_t handle);
void starpu_data_set_name(starpu_data_handle_t handle, const char *name);
void starpu_data_set_coordinates(starpu_data_handle_t handle, unsigned dimensions, ...);
void starpu_data_set_default_sequential_consistency_flag(unsigned flag);
unsigned starpu_data_get_default_sequential_consistency_flag(void);
void starpu_data_set_sequential_consistency_flag(starpu_data_handle_t handle, unsigned flag);
unsigned starpu_data_get_sequential_consistency_flag(starpu_data_handle_t handle);
void starpu_data_wont_use(starpu_data_handle_t handle);
void starpu_data_invalidate(starpu_data_handle_t handle);
int starpu_data_acquire(starpu_data_handle_t handle, enum starpu_data_access_mode mode);
void starpu_data_release(starpu_data_handle_t handle);
/* asynchronous acquisition: `callback` runs once the data is available in
 * RAM; the access lasts until starpu_data_release */
int starpu_data_acquire_cb(starpu_data_handle_t handle, enum starpu_data_access_mode mode, void (*callback)(void *),
                           void *arg);
size_t starpu_data_get_size(starpu_data_handle_t handle);
uint32_t starpu_data_get_footprint(starpu_data_handle_t handle);
void *starpu_data_get_local_ptr(starpu_data_handle_t handle);
enum starpu_data_interface_id starpu_data_get_interface_id(starpu_data_handle_t handle);
size_t starpu_matrix_get_nx(starpu_data_handle_t handle);
size_t starpu_matrix_get_ny(starpu_data_handle_t handle);
size_t starpu_matrix_get_local_ld(starpu_data_handle_t handle);
uintptr_t starpu_matrix_get_local_ptr(starpu_data_handle_t handle);
size_t starpu_matrix_get_elemsize(starpu_data_handle_t handle);

/* ------------------------------------------------------------------ filters */
struct starpu_data_filter {
    void (*filter_func)(void *father_interface, void *child_interface, struct starpu_data_filter *, unsigned id,
                        unsigned nparts);
    unsigned nchildren;
    unsigned (*get_nchildren)(struct starpu_data_filter *, starpu_data_handle_t initial_handle);
    struct starpu_data_interface_ops *(*get_child_ops)(struct starpu_data_filter *, unsigned id);
    unsigned filter_arg;
    void *filter_arg_ptr;
};

void starpu_matrix_filter_block(void *father_interface, void *child_interface, struct starpu_data_filter *f,
                                unsigned id, unsigned nparts);
void starpu_matrix_filter_vertical_block(void *father_interface, void *child_interface, struct starpu_data_filter *f,
                                         unsigned id, unsigned nparts);
/* vectors: nx split into nparts blocks, the remainder to the first ones */
void starpu_vector_filter_block(void *father_interface, void *child_interface, struct starpu_data_filter *f,
                                unsigned id, unsigned nparts);
void starpu_filter_nparts_compute_chunk_size_and_offset(unsigned n, unsigned nparts, size_t elemsize, unsigned id,
                                                        size_t blocksize, size_t *chunk_size, size_t *offset);
void starpu_data_partition(starpu_data_handle_t initial_handle, struct starpu_data_filter *f);
void starpu_data_map_filters(starpu_data_handle_t root_data, unsigned nfilters, ...);
starpu_data_handle_t starpu_data_get_sub_data(starpu_data_handle_t root_data, unsigned depth, ...);
starpu_data_handle_t starpu_data_get_child(starpu_data_handle_t handle, unsigned i);
int starpu_data_get_nb_children(starpu_data_handle_t handle);
void starpu_data_unpartition(starpu_data_handle_t root_data, unsigned gathering_node);

/* ===================================================================== tasks */

#define STARPU_NOWHERE ((1ULL) << 0)
#define STARPU_WORKER_TO_MASK(a) ((1ULL) << ((a) + 1))

enum starpu_worker_archtype {
    STARPU_CPU_WORKER = 0,
    STARPU_CUDA_WORKER = 1,
    STARPU_OPENCL_WORKER = 2,
    STARPU_MAX_FPGA_WORKER = 4,
    STARPU_MPI_SC_WORKER = 5,
    STARPU_TCPIP_SC_WORKER = 6,
    STARPU_HIP_WORKER = 7,
    STARPU_SYCL_WORKER = 8,
    STARPU_NARCH = 9,
    STARPU_ANY_WORKER = 255
};

#define STARPU_CPU STARPU_WORKER_TO_MASK(STARPU_CPU_WORKER)
#define STARPU_CUDA STARPU_WORKER_TO_MASK(STARPU_CUDA_WORKER)
#define STARPU_OPENCL STARPU_WORKER_TO_MASK(STARPU_OPENCL_WORKER)
#define STARPU_HIP STARPU_WORKER_TO_MASK(STARPU_HIP_WORKER)

#define STARPU_CUDA_ASYNC (1 << 0)
#define STARPU_HIP_ASYNC (1 << 0)
#define STARPU_OPENCL_ASYNC (1 << 0)

enum starpu_codelet_type { STARPU_SEQ = 0, STARPU_SPMD, STARPU_FORKJOIN };

typedef void (*starpu_cpu_func_t)(void **, void *);
typedef void (*starpu_cuda_func_t)(void **, void *);
typedef void (*starpu_hip_func_t)(void **, void *);
typedef void (*starpu_opencl_func_t)(void **, void *);

struct starpu_task;
struct starpu_perfmodel;

struct starpu_codelet {
    uint32_t where;
    int (*can_execute)(unsigned workerid, struct starpu_task *task, unsigned nimpl);
    enum starpu_codelet_type type;
    int max_parallelism;
    starpu_cpu_func_t cpu_funcs[STARPU_MAXIMPLEMENTATIONS];
    starpu_cuda_func_t cuda_funcs[STARPU_MAXIMPLEMENTATIONS];
    char cuda_flags[STARPU_MAXIMPLEMENTATIONS];
    starpu_hip_func_t hip_funcs[STARPU_MAXIMPLEMENTATIONS];
    char hip_flags[STARPU_MAXIMPLEMENTATIONS];
    starpu_opencl_func_t opencl_funcs[STARPU_MAXIMPLEMENTATIONS];
    char opencl_flags[STARPU_MAXIMPLEMENTATIONS];
    const char *cpu_funcs_name[STARPU_MAXIMPLEMENTATIONS];
    int nbuffers;
    enum starpu_data_access_mode modes[STARPU_NMAXBUFS];
    enum starpu_data_access_mode *dyn_modes;
    unsigned specific_nodes;
    int nodes[STARPU_NMAXBUFS];
    struct starpu_perfmodel *model;
    struct starpu_perfmodel *energy_model;
    unsigned long per_worker_stats[STARPU_NMAXWORKERS];
    const char *name;
    unsigned color;
    int flags;
    int checked;
};

typedef uint64_t starpu_tag_t;

enum starpu_task_status {
    STARPU_TASK_INIT,
    STARPU_TASK_BLOCKED,
    STARPU_TASK_READY,
    STARPU_TASK_RUNNING,
    STARPU_TASK_FINISHED,
    STARPU_TASK_BLOCKED_ON_TAG,
    STARPU_TASK_BLOCKED_ON_TASK,
    STARPU_TASK_BLOCKED_ON_DATA,
    STARPU_TASK_STOPPED
};

struct starpu_task {
    const char *name;
    struct starpu_codelet *cl;
    uint32_t where;
    int nbuffers;
    starpu_data_handle_t handles[STARPU_NMAXBUFS];
    void *interfaces[STARPU_NMAXBUFS];
    enum starpu_data_access_mode modes[STARPU_NMAXBUFS];
    void *cl_arg;
    size_t cl_arg_size;
    unsigned cl_arg_free;
    void (*callback_func)(void *);
    void *callback_arg;
    unsigned callback_arg_free;
    void (*prologue_callback_func)(void *); /* run when the task becomes ready, before scheduling */
    void *prologue_callback_arg;
    unsigned prologue_callback_arg_free;
    unsigned use_tag;
    starpu_tag_t tag_id;
    unsigned sequential_consistency;
    unsigned synchronous;
    int priority;
    unsigned execute_on_a_specific_worker;
    unsigned workerid;
    unsigned detach;
    unsigned destroy;
    unsigned regenerate;
    unsigned no_submitorder;
    enum starpu_task_status status;
    unsigned sched_ctx;
    int hypervisor_tag;
    double flops;
    double predicted;
    double predicted_transfer;
    unsigned long magic;
    void *sched_data;
    unsigned color;        /* display colour of the task in traces */
    unsigned failed;       /* set by starpu_task_ft_failed */
    int nb_termination_call_required; /* starpu_task_end_dep_add calls not yet released */
    struct starpu_task **declared_deps; /* runtime-private: starpu_task_declare_deps_array */
    unsigned ndeclared_deps;
    void *starpu_private;  /* runtime job */
};

#define STARPU_TASK_INVALID 0
#define STARPU_VARIABLE_NBUFFERS (-1) /* the task's own nbuffers */

/* a codelet that does nothing, on every kind of worker */
extern struct starpu_codelet starpu_codelet_nop;
void starpu_codelet_nop_func(void *descr[], void *arg);
#define STARPU_DEFAULT_PRIO 0

void starpu_task_init(struct starpu_task *task);
struct starpu_task *starpu_task_create(void);
void starpu_task_clean(struct starpu_task *task);
void starpu_task_destroy(struct starpu_task *task);
int starpu_task_submit(struct starpu_task *task);
int starpu_task_wait(struct starpu_task *task);
int starpu_task_wait_array(struct starpu_task **tasks, unsigned nb_tasks);
#define STARPU_TASK_GET_NBUFFERS(task) ((unsigned)((task)->cl->nbuffers == STARPU_VARIABLE_NBUFFERS ? (task)->nbuffers : (task)->cl->nbuffers))
#define STARPU_TASK_GET_HANDLE(task, i) ((task)->handles[i])
#define STARPU_TASK_GET_MODE(task, i) ((task)->cl->nbuffers == STARPU_VARIABLE_NBUFFERS || !(task)->cl->modes[i] ? (task)->modes[i] : (task)->cl->modes[i])
int starpu_task_wait_for_all(void);
int starpu_task_wait_for_n_submitted(unsigned n);
int starpu_task_nsubmitted(void);
int starpu_task_nready(void);
struct starpu_task *starpu_task_get_current(void);
/* explicit task dependencies (starpu_task_dep.h): before `task` is submitted;
 * the tasks it waits for may be submitted before or after it, or be done */
void starpu_task_declare_deps_array(struct starpu_task *task, unsigned ndeps, struct starpu_task *task_array[]);
void starpu_task_declare_deps(struct starpu_task *task, unsigned ndeps, ...);
/* `task` terminates only once these tasks have too (done, submitted or not yet) */
void starpu_task_declare_end_deps_array(struct starpu_task *task, unsigned ndeps, struct starpu_task *task_array[]);
void starpu_task_declare_end_deps(struct starpu_task *task, unsigned ndeps, ...);
int starpu_task_get_task_succs(struct starpu_task *task, unsigned ndeps, struct starpu_task *task_array[]);
struct starpu_task *starpu_tag_get_task(starpu_tag_t id);
/* submission without data or tag dependencies (the caller already holds the data) */
int starpu_task_submit_nodeps(struct starpu_task *task);
/* termination of `task` waits for nb_deps more starpu_task_end_dep_release calls */
void starpu_task_end_dep_add(struct starpu_task *task, int nb_deps);
void starpu_task_end_dep_release(struct starpu_task *task);

/* fault tolerance (src/core/task.c): a task given starpu_task_ft_prologue as
 * prologue becomes a meta task that holds its data and runs nothing; a copy
 * of it does the work, and its callback (check_ft) either releases the meta
 * task (starpu_task_ft_success) or submits another copy when the work
 * reported starpu_task_ft_failed.  Only STARPU_R and STARPU_W accesses. */
void starpu_task_ft_prologue(void *check_ft);
struct starpu_task *starpu_task_ft_create_retry(const struct starpu_task *meta_task,
                                                const struct starpu_task *template_task, void (*check_ft)(void *));
void starpu_task_ft_failed(struct starpu_task *task);
void starpu_task_ft_success(struct starpu_task *meta_task);
void starpu_codelet_init(struct starpu_codelet *cl);
void starpu_iteration_push(unsigned long iteration);
void starpu_iteration_pop(void);

/* ------------------------------------------------------------- task_insert */
#define STARPU_MODE_SHIFT 17
#define STARPU_VALUE (1 << STARPU_MODE_SHIFT)
#define STARPU_CALLBACK (2 << STARPU_MODE_SHIFT)
#define STARPU_CALLBACK_WITH_ARG (3 << STARPU_MODE_SHIFT)
#define STARPU_CALLBACK_ARG (4 << STARPU_MODE_SHIFT)
#define STARPU_PRIORITY (5 << STARPU_MODE_SHIFT)
#define STARPU_EXECUTE_ON_NODE (6 << STARPU_MODE_SHIFT)
#define STARPU_EXECUTE_ON_DATA (7 << STARPU_MODE_SHIFT)
#define STARPU_DATA_ARRAY (8 << STARPU_MODE_SHIFT)
#define STARPU_DATA_MODE_ARRAY (9 << STARPU_MODE_SHIFT)
#define STARPU_TAG (11 << STARPU_MODE_SHIFT)
#define STARPU_FLOPS (13 << STARPU_MODE_SHIFT)
#define STARPU_SCHED_CTX (14 << STARPU_MODE_SHIFT)
#define STARPU_EXECUTE_ON_WORKER (19 << STARPU_MODE_SHIFT)
#define STARPU_EXECUTE_WHERE (20 << STARPU_MODE_SHIFT)
#define STARPU_TAG_ONLY (21 << STARPU_MODE_SHIFT)
#define STARPU_POSSIBLY_PARALLEL (22 << STARPU_MODE_SHIFT)
#define STARPU_NAME (25 << STARPU_MODE_SHIFT)
#define STARPU_CL_ARGS (26 << STARPU_MODE_SHIFT)
#define STARPU_CL_ARGS_NFREE (27 << STARPU_MODE_SHIFT)
#define STARPU_TASK_COLOR (29 << STARPU_MODE_SHIFT)
#define STARPU_TASK_SYNCHRONOUS (31 << STARPU_MODE_SHIFT)
#define STARPU_SEQUENTIAL_CONSISTENCY (35 << STARPU_MODE_SHIFT)
#define STARPU_TASK_NO_SUBMITORDER (37 << STARPU_MODE_SHIFT)
#define STARPU_PROLOGUE_CALLBACK (15 << STARPU_MODE_SHIFT)
#define STARPU_PROLOGUE_CALLBACK_ARG (16 << STARPU_MODE_SHIFT)
#define STARPU_PROLOGUE_CALLBACK_ARG_NFREE (40 << STARPU_MODE_SHIFT)

struct starpu_data_descr {
    starpu_data_handle_t handle;
    enum starpu_data_access_mode mode;
};

int starpu_task_insert(struct starpu_codelet *cl, ...);
int starpu_insert_task(struct starpu_codelet *cl, ...);
struct starpu_task *starpu_task_build(struct starpu_codelet *cl, ...);
void starpu_codelet_unpack_args(void *cl_arg, ...);
void starpu_codelet_pack_args(void **arg_buffer, size_t *arg_buffer_size, ...);
void starpu_codelet_unpack_args_and_copyleft(void *cl_arg, void *buffer, size_t buffer_size, ...);

/* ====================================================================== tags */
void starpu_tag_declare_deps(starpu_tag_t id, unsigned ndeps, ...);
void starpu_tag_declare_deps_array(starpu_tag_t id, unsigned ndeps, starpu_tag_t *array);
int starpu_tag_wait(starpu_tag_t id);
int starpu_tag_wait_array(unsigned ntags, starpu_tag_t *id);
void starpu_tag_remove(starpu_tag_t id);
void starpu_tag_notify_from_apps(starpu_tag_t id);

/* ================================================================ perfmodels */
enum starpu_perfmodel_type {
    STARPU_PERFMODEL_INVALID = 0,
    STARPU_PER_WORKER,
    STARPU_PER_ARCH,
    STARPU_COMMON,
    STARPU_HISTORY_BASED,
    STARPU_REGRESSION_BASED,
    STARPU_NL_REGRESSION_BASED,
    STARPU_MULTIPLE_REGRESSION_BASED
};

struct starpu_perfmodel_device {
    enum starpu_worker_archtype type;
    int devid;
    int ncores;
};

struct starpu_perfmodel_arch {
    int ndevices;
    struct starpu_perfmodel_device *devices;
};

struct starpu_perfmodel_history_state;

struct starpu_perfmodel {
    enum starpu_perfmodel_type type;
    double (*cost_function)(struct starpu_task *, unsigned nimpl);
    double (*arch_cost_function)(struct starpu_task *, struct starpu_perfmodel_arch *arch, unsigned nimpl);
    double (*worker_cost_function)(struct starpu_task *, unsigned workerid, unsigned nimpl);
    size_t (*size_base)(struct starpu_task *, unsigned nimpl);
    uint32_t (*footprint)(struct starpu_task *);
    const char *symbol;
    unsigned is_loaded;
    unsigned benchmarking;
    unsigned is_init;
    struct starpu_perfmodel_history_state *state;
};

double starpu_task_expected_length(struct starpu_task *task, struct starpu_perfmodel_arch *arch, unsigned nimpl);
double starpu_task_worker_expected_length(struct starpu_task *task, unsigned workerid, unsigned sched_ctx_id,
                                          unsigned nimpl);
double starpu_worker_get_relative_speedup(struct starpu_perfmodel_arch *perf_arch);
double starpu_task_expected_data_transfer_time(unsigned memory_node, struct starpu_task *task);
uint32_t starpu_task_footprint(struct starpu_perfmodel *model, struct starpu_task *task,
                               struct starpu_perfmodel_arch *arch, unsigned nimpl);
void starpu_perfmodel_init(struct starpu_perfmodel *model);
int starpu_perfmodel_deinit(struct starpu_perfmodel *model);
/* 0 on success, 1 when no file exists for the symbol or it is malformed */
int starpu_perfmodel_load_file(const char *filename, struct starpu_perfmodel *model);
int starpu_perfmodel_load_symbol(const char *symbol, struct starpu_perfmodel *model);
int starpu_perfmodel_unload_model(struct starpu_perfmodel *model);
/* the existing model file for `symbol`, "" when there is none */
void starpu_perfmodel_get_model_path(const char *symbol, char *path, size_t maxlen);
/* where the model file for `symbol` is written (its directory is created) */
void starpu_perfmodel_get_model_path_default_location(const char *symbol, char *path, size_t maxlen);
int starpu_save_history_based_model(struct starpu_perfmodel *model);
void starpu_perfmodel_update_history(struct starpu_perfmodel *model, struct starpu_task *task,
                                     struct starpu_perfmodel_arch *arch, unsigned cpuid, unsigned nimpl,
                                     double measured);
void starpu_perfmodel_update_history_n(struct starpu_perfmodel *model, struct starpu_task *task,
                                       struct starpu_perfmodel_arch *arch, unsigned cpuid, unsigned nimpl,
                                       double average_measured, unsigned number);
double starpu_perfmodel_history_based_expected_perf(struct starpu_perfmodel *model, struct starpu_perfmodel_arch *arch,
                                                    uint32_t footprint);

/* perfmodel tooling (tools/starpu_perfmodel_display.c, tools/starpu_perfmodel_plot.c) */
void starpu_drivers_preinit(void);
void starpu_perfmodel_initialize(void);
void starpu_perfmodel_free_sampling(void);
int starpu_perfmodel_list(FILE *output);
void starpu_perfmodel_directory(FILE *output);
void starpu_perfmodel_dump_xml(FILE *output, struct starpu_perfmodel *model);
void starpu_perfmodel_print(struct starpu_perfmodel *model, struct starpu_perfmodel_arch *arch, unsigned nimpl,
                            char *parameter, uint32_t *footprint, FILE *output);
int starpu_perfmodel_print_all(struct starpu_perfmodel *model, char *arch, char *parameter, uint32_t *footprint,
                               FILE *output);
int starpu_perfmodel_print_estimations(struct starpu_perfmodel *model, uint32_t footprint, FILE *output);
int starpu_perfmodel_list_combs(FILE *output, struct starpu_perfmodel *model);
int starpu_perfmodel_get_narch_combs(void);
int starpu_perfmodel_arch_comb_add(int ndevices, struct starpu_perfmodel_device *devices);
int starpu_perfmodel_arch_comb_get(int ndevices, struct starpu_perfmodel_device *devices);
struct starpu_perfmodel_arch *starpu_perfmodel_arch_comb_fetch(int comb);
const char *starpu_perfmodel_get_archtype_name(enum starpu_worker_archtype archtype);
void starpu_perfmodel_get_arch_name(struct starpu_perfmodel_arch *arch, char *archname, size_t maxlen, unsigned nimpl);
/* GB300 addition behind the plot tool: writes the gnuplot script `gp_path`
 * and its averages file `avg_path` for a loaded model (only_comb < 0: every
 * combination); 0 or -errno */
int starpu_gb300_perfmodel_plot(struct starpu_perfmodel *model, struct starpu_perfmodel *energy_model,
                                const char *symbol, const char *energy_symbol, int only_comb, int gflops, int energy,
                                const char *gp_path, const char *avg_path);

/* =================================================================== workers */
unsigned starpu_worker_get_count(void);
unsigned starpu_cpu_worker_get_count(void);
unsigned starpu_cuda_worker_get_count(void);
/* workers driving MPI / TCP-IP server-client sinks: none in this runtime */
unsigned starpu_mpi_sc_worker_get_count(void);
unsigned starpu_tcpip_sc_worker_get_count(void);
unsigned starpu_hip_worker_get_count(void);
unsigned starpu_opencl_worker_get_count(void);
int starpu_worker_get_id(void);
enum starpu_worker_archtype starpu_worker_get_type(int id);
int starpu_worker_get_devid(int id);
void starpu_worker_get_name(int id, char *dst, size_t maxlen);
struct starpu_perfmodel_arch *starpu_worker_get_perf_archtype(int workerid, unsigned sched_ctx_id);
int starpu_combined_worker_get_size(void);
int starpu_combined_worker_get_rank(void);
int starpu_worker_get_ids_by_type(enum starpu_worker_archtype type, int *workerids, unsigned maxsize);

/* =========================================================== sched contexts */
#define STARPU_SCHED_CTX_POLICY_NAME (1 << 16)
#define STARPU_SCHED_CTX_POLICY_STRUCT (2 << 16)
#define STARPU_SCHED_CTX_POLICY_MIN_PRIO (3 << 16)
#define STARPU_SCHED_CTX_POLICY_MAX_PRIO (4 << 16)

int starpu_sched_get_min_priority(void);
int starpu_sched_get_max_priority(void);
int starpu_sched_set_min_priority(int min_prio);
int starpu_sched_set_max_priority(int max_prio);
#define STARPU_MIN_PRIO (starpu_sched_get_min_priority())
#define STARPU_MAX_PRIO (starpu_sched_get_max_priority())

/* contexts 1 .. STARPU_NMAX_SCHED_CTXS - 1 (0 is the initial context, every
 * worker); STARPU_NMAX_SCHED_CTXS also means "no context" */
#define STARPU_NMAX_SCHED_CTXS 10
unsigned starpu_sched_ctx_create(int *workerids_ctx, int nworkers_ctx, const char *sched_ctx_name, ...);
void starpu_sched_ctx_delete(unsigned sched_ctx_id);
void starpu_sched_ctx_set_inheritor(unsigned sched_ctx_id, unsigned inheritor);
unsigned starpu_sched_ctx_get_inheritor(unsigned sched_ctx_id);
void starpu_sched_ctx_set_context(unsigned *sched_ctx_id);
unsigned starpu_sched_ctx_get_context(void);
unsigned starpu_sched_ctx_get_nworkers(unsigned sched_ctx_id);
unsigned starpu_sched_ctx_contains_worker(int workerid, unsigned sched_ctx_id);
void starpu_reset_scheduler(void);

/* ============================================================= init / conf */
struct starpu_conf {
    int magic;
    const char *sched_policy_name;
    void *sched_policy;
    int ncpus;
    int ncuda;
    int nhip;
    int nopencl;
    unsigned calibrate;
    unsigned bus_calibrate;
    int single_combined_worker;
    int disable_asynchronous_copy;
    int precedence_over_environment_variables;
    int nsycl, nmax_fpga, nmpi_sc, ntcpip_sc; /* accepted; this runtime has no such workers */
};

int starpu_conf_init(struct starpu_conf *conf);
int starpu_conf_noworker(struct starpu_conf *conf);

/* integer environment variables (starpu_helper.h): -1 when unset; a value
 * that is not a non-negative integer aborts */
int starpu_get_env_number(const char *str);
void starpu_usleep(float nb_micro_sec);
void starpu_do_schedule(void);
void starpu_sleep(float nb_sec);
int starpu_worker_get_count_by_type(enum starpu_worker_archtype type);
/* a handle without data, for dependencies only */
void starpu_void_data_register(starpu_data_handle_t *handle);
#define STARPU_ATOMIC_ADD(ptr, value) (__sync_fetch_and_add((ptr), (value)) + (value))
#define STARPU_ATTRIBUTE_ALIGNED(size) __attribute__((aligned(size)))
static inline int starpu_get_env_number_default(const char *str, int defval)
{
    const int n = starpu_get_env_number(str);
    return n == -1 ? defval : n;
}
#define starpu_getenv_number(s) starpu_get_env_number(s)
#define starpu_getenv_number_default(s, d) starpu_get_env_number_default(s, d)
int starpu_init(struct starpu_conf *conf);
int starpu_initialize(struct starpu_conf *user_conf, int *argc, char ***argv);
int starpu_is_initialized(void);
void starpu_shutdown(void);
void starpu_pause(void);
void starpu_resume(void);
int starpu_asynchronous_copy_disabled(void);

/* =========================================================== memory alloc */
#define STARPU_MALLOC_PINNED ((1ULL) << 1)
#define STARPU_MALLOC_COUNT ((1ULL) << 2)
#define STARPU_MALLOC_NORECLAIM ((1ULL) << 3)
#define STARPU_MEMORY_WAIT ((1ULL) << 4)
#define STARPU_MEMORY_OVERFLOW ((1ULL) << 5)
#define STARPU_MALLOC_SIMULATION_FOLDED ((1ULL) << 6)
#define STARPU_MALLOC_SIMULATION_UNIQUE ((1ULL) << 7)

int starpu_malloc(void **A, size_t dim);
int starpu_free(void *A);
int starpu_malloc_flags(void **A, size_t dim, int flags);
int starpu_free_flags(void *A, size_t dim, int flags);
int starpu_free_noflag(void *A, size_t dim);
void starpu_malloc_set_align(size_t align);

/* ========================================= profiling / tracing / bound stubs */
void starpu_fxt_start_profiling(void);
void starpu_fxt_stop_profiling(void);
void starpu_bound_start(int deps, int prio);
void starpu_bound_stop(void);
void starpu_bound_compute(double *res, double *integer_res, int integer);
void starpu_bound_print_lp(FILE *output);
void starpu_bound_print_mps(FILE *output);
void starpu_bound_print(FILE *output, int integer);
#define STARPU_PROFILING_DISABLE 0
#define STARPU_PROFILING_ENABLE 1
int starpu_profiling_status_set(int status);
int starpu_profiling_status_get(void);
/* prints the runtime's host<->device transfer totals (starpu_profiling.h) */
void starpu_profiling_bus_helper_display_summary(void);
/* with STARPU_WORKER_STATS=1: tasks run per worker (also printed at shutdown) */
void starpu_profiling_worker_helper_display_summary(void);
void starpu_bound_print_dot(FILE *output);

/* ================================================= random numbers (starpu_rand.h) */
#define starpu_srand48(seed) srand48(seed)
#define starpu_drand48() drand48()

/* ============================================================ GB300 extras
 * Statistics of the runtime's CUDA execution (no StarPU counterpart). */
struct starpu_gb300_runtime_stats {
    unsigned long tasks_cpu;       /* tasks run by CPU workers */
    unsigned long tasks_cuda;      /* tasks run by the CUDA worker, per task */
    unsigned long tasks_graph;     /* tasks run inside captured CUDA graphs */
    unsigned long graphs_launched; /* whole-DAG graphs launched */
    double graph_build_us;         /* host time to capture + instantiate */
    double graph_exec_us;          /* device time of the launched graphs */
    unsigned long h2d_bytes, d2h_bytes;
};
void starpu_gb300_runtime_get_stats(struct starpu_gb300_runtime_stats *stats);
void starpu_gb300_runtime_reset_stats(void);

#ifdef __cplusplus
}
#endif

#include "starpu_cuda.h"

#endif /* STARPU_H */
