/*
 * Data handles, tile filters and coherency between host RAM and the GPU.
 *
 * Matrix semantics follow StarPU's matrix interface (include/starpu_data_interfaces.h:1213):
 * nx contiguous elements (rows, column-major), ny columns, ld >= nx.  The two
 * block filters split along nx (starpu_matrix_filter_block) or ny
 * (starpu_matrix_filter_vertical_block) with the remainder going to the first
 * chunks (src/datawizard/interfaces/matrix_filters.c:22-104,
 * src/datawizard/filters.c:1655-1679).  On the GPU a root matrix is one dense
 * allocation (ld = nx) and every tile is a view into it, so tile copies are
 * 2D copies and a whole partitioned matrix can be staged with one copy.
 */
#include <stdarg.h>

#include "rt_internal.h"

static int default_seq = 1;

static void init_handle(struct _starpu_data_state *h)
{
    memset(h, 0, sizeof *h);
    h->root = h;
    h->seq_consistency = default_seq;
}

void starpu_data_set_default_sequential_consistency_flag(unsigned flag) { default_seq = flag != 0; }
unsigned starpu_data_get_default_sequential_consistency_flag(void) { return (unsigned)default_seq; }
void starpu_data_set_sequential_consistency_flag(starpu_data_handle_t h, unsigned flag)
{
    h->seq_consistency = flag != 0;
}
unsigned starpu_data_get_sequential_consistency_flag(starpu_data_handle_t h) { return (unsigned)h->seq_consistency; }

/* coordinates only label data for traces / MPI placement: accepted and ignored */
void starpu_data_set_coordinates(starpu_data_handle_t h, unsigned dimensions, ...)
{
    (void)h;
    (void)dimensions;
}

void starpu_matrix_data_register(starpu_data_handle_t *handle, int home_node, uintptr_t ptr, size_t ld, size_t nx,
                                 size_t ny, size_t elemsize)
{
    STARPU_ASSERT(handle);
    STARPU_ASSERT_MSG(ld >= nx, "ld (%zu) must be >= nx (%zu)", ld, nx);
    struct _starpu_data_state *h = calloc(1, sizeof *h);
    init_handle(h);
    h->id = STARPU_MATRIX_INTERFACE_ID;
    h->home_node = home_node;
    h->elemsize = elemsize;
    for (int n = 0; n < RT_NODES; ++n) {
        h->mat[n].id = STARPU_MATRIX_INTERFACE_ID;
        h->mat[n].nx = nx;
        h->mat[n].ny = ny;
        h->mat[n].elemsize = elemsize;
        h->mat[n].ld = (n == RT_NODE_RAM) ? ld : nx;
    }
    if (home_node == STARPU_MAIN_RAM) {
        h->mat[RT_NODE_RAM].ptr = ptr;
        h->mat[RT_NODE_RAM].allocsize = ld * ny * elemsize;
        h->valid[RT_NODE_RAM] = 1;
        h->allocated[RT_NODE_RAM] = 1;
    }
    *handle = h;
}

void starpu_vector_data_register(starpu_data_handle_t *handle, int home_node, uintptr_t ptr, size_t nx,
                                 size_t elemsize)
{
    starpu_matrix_data_register(handle, home_node, ptr, nx ? nx : 1, nx, 1, elemsize);
    (*handle)->id = STARPU_VECTOR_INTERFACE_ID;
}

void starpu_variable_data_register(starpu_data_handle_t *handle, int home_node, uintptr_t ptr, size_t size)
{
    struct _starpu_data_state *h = calloc(1, sizeof *h);
    init_handle(h);
    h->id = STARPU_VARIABLE_INTERFACE_ID;
    h->home_node = home_node;
    h->elemsize = size;
    for (int n = 0; n < RT_NODES; ++n) {
        h->var[n].id = STARPU_VARIABLE_INTERFACE_ID;
        h->var[n].elemsize = size;
    }
    if (home_node == STARPU_MAIN_RAM) {
        h->var[RT_NODE_RAM].ptr = ptr;
        h->valid[RT_NODE_RAM] = 1;
        h->allocated[RT_NODE_RAM] = 1;
    }
    *handle = h;
}

/* a handle that carries no data (void_interface.c): a zero-byte variable at
 * a static host address, valid in RAM from the start, so tasks order on it
 * and no copy ever moves a byte */
void starpu_void_data_register(starpu_data_handle_t *handle)
{
    static char nothing;
    starpu_variable_data_register(handle, STARPU_MAIN_RAM, (uintptr_t)&nothing, 0);
}

void starpu_data_set_name(starpu_data_handle_t handle, const char *name)
{
    if (handle && name) snprintf(handle->name, sizeof handle->name, "%s", name);
}

size_t rt_data_size(starpu_data_handle_t h)
{
    if (h->id == STARPU_VARIABLE_INTERFACE_ID) return h->elemsize;
    return h->mat[0].nx * h->mat[0].ny * h->elemsize;
}

size_t starpu_data_get_size(starpu_data_handle_t handle) { return rt_data_size(handle); }

/* FNV-1a over the shape: tasks on equally shaped data share history entries
 * (the role of matrix_interface.c:184's footprint). */
uint32_t rt_data_footprint(starpu_data_handle_t h)
{
    uint64_t v[3];
    v[0] = h->id == STARPU_VARIABLE_INTERFACE_ID ? h->elemsize : h->mat[0].nx;
    v[1] = h->id == STARPU_VARIABLE_INTERFACE_ID ? 0 : h->mat[0].ny;
    v[2] = h->elemsize;
    uint32_t x = 2166136261u;
    const unsigned char *p = (const unsigned char *)v;
    for (size_t i = 0; i < sizeof v; ++i) {
        x ^= p[i];
        x *= 16777619u;
    }
    return x;
}

uint32_t starpu_data_get_footprint(starpu_data_handle_t handle) { return rt_data_footprint(handle); }
enum starpu_data_interface_id starpu_data_get_interface_id(starpu_data_handle_t h) { return h->id; }
size_t starpu_matrix_get_nx(starpu_data_handle_t h) { return h->mat[0].nx; }
size_t starpu_matrix_get_ny(starpu_data_handle_t h) { return h->mat[0].ny; }
size_t starpu_matrix_get_elemsize(starpu_data_handle_t h) { return h->elemsize; }

size_t starpu_matrix_get_local_ld(starpu_data_handle_t h)
{
    int w = rt_current_worker();
    int node = (w >= 0 && rt.workers[w].type == STARPU_CUDA_WORKER) ? RT_NODE_GPU : RT_NODE_RAM;
    return h->mat[node].ld;
}

uintptr_t starpu_matrix_get_local_ptr(starpu_data_handle_t h)
{
    int w = rt_current_worker();
    int node = (w >= 0 && rt.workers[w].type == STARPU_CUDA_WORKER) ? RT_NODE_GPU : RT_NODE_RAM;
    return h->mat[node].ptr;
}

void *starpu_data_get_local_ptr(starpu_data_handle_t h)
{
    if (h->id == STARPU_VARIABLE_INTERFACE_ID) {
        int w = rt_current_worker();
        int node = (w >= 0 && rt.workers[w].type == STARPU_CUDA_WORKER) ? RT_NODE_GPU : RT_NODE_RAM;
        return (void *)h->var[node].ptr;
    }
    return (void *)starpu_matrix_get_local_ptr(h);
}

/* --------------------------------------------------------------- filters */

void starpu_filter_nparts_compute_chunk_size_and_offset(unsigned n, unsigned nparts, size_t elemsize, unsigned id,
                                                        size_t blocksize, size_t *chunk_size, size_t *offset)
{
    size_t base = n / nparts, rem = n % nparts;
    *chunk_size = base + (id < rem ? 1 : 0);
    if (offset) *offset = ((size_t)id * base + (id < rem ? id : rem)) * blocksize * elemsize;
}

static void matrix_block(int along_y, void *father, void *child, unsigned id, unsigned nparts)
{
    struct starpu_matrix_interface *p = father, *c = child;
    size_t nn = along_y ? p->ny : p->nx;
    STARPU_ASSERT_MSG(nparts <= nn, "cannot split %zu elements in %u parts", nn, nparts);
    size_t chunk, off;
    starpu_filter_nparts_compute_chunk_size_and_offset((unsigned)nn, nparts, p->elemsize, id, along_y ? p->ld : 1,
                                                       &chunk, &off);
    *c = *p;
    if (along_y) c->ny = chunk;
    else c->nx = chunk;
    if (p->ptr) c->ptr = p->ptr + off;
    c->offset = p->offset + off;
    c->allocsize = c->ld * c->ny * c->elemsize;
}

void starpu_matrix_filter_block(void *father, void *child, struct starpu_data_filter *f, unsigned id, unsigned nparts)
{
    (void)f;
    matrix_block(0, father, child, id, nparts);
}

void starpu_matrix_filter_vertical_block(void *father, void *child, struct starpu_data_filter *f, unsigned id,
                                         unsigned nparts)
{
    (void)f;
    matrix_block(1, father, child, id, nparts);
}

/* nx split into nparts blocks, the remainder going to the first ones
 * (vector_filters.c); the runtime hands its filters the nx x 1 matrix view */
void starpu_vector_filter_block(void *father, void *child, struct starpu_data_filter *f, unsigned id, unsigned nparts)
{
    (void)f;
    matrix_block(0, father, child, id, nparts);
}

void starpu_data_partition(starpu_data_handle_t h, struct starpu_data_filter *f)
{
    STARPU_ASSERT_MSG(h->id == STARPU_MATRIX_INTERFACE_ID || h->id == STARPU_VECTOR_INTERFACE_ID,
                      "only matrix and vector handles can be partitioned");
    STARPU_ASSERT_MSG(!h->partitioned, "handle already partitioned");
    unsigned n = f->get_nchildren ? f->get_nchildren(f, h) : f->nchildren;
    STARPU_ASSERT(n > 0);
    starpu_task_wait_for_all();
    h->children = calloc(n, sizeof *h->children);
    h->nchildren = n;
    for (unsigned i = 0; i < n; ++i) {
        struct _starpu_data_state *c = calloc(1, sizeof *c);
        init_handle(c);
        c->id = h->id;
        c->home_node = h->home_node;
        c->elemsize = h->elemsize;
        c->parent = h;
        c->root = h->root;
        c->seq_consistency = h->seq_consistency;
        /* the child's RAM view, computed by the filter from the parent's */
        struct starpu_matrix_interface pr = h->mat[RT_NODE_RAM];
        pr.offset = 0;
        f->filter_func(&pr, &c->mat[RT_NODE_RAM], f, i, n);
        size_t rel = c->mat[RT_NODE_RAM].offset / h->elemsize;
        size_t pld = h->mat[RT_NODE_RAM].ld;
        c->row_off = h->row_off + rel % pld;
        c->col_off = h->col_off + rel / pld;
        c->mat[RT_NODE_RAM].offset = 0;
        c->mat[RT_NODE_RAM].allocsize = c->mat[RT_NODE_RAM].ld * c->mat[RT_NODE_RAM].ny * c->elemsize;
        c->mat[RT_NODE_GPU] = c->mat[RT_NODE_RAM];
        c->mat[RT_NODE_GPU].ptr = 0;
        for (int nd = 0; nd < RT_NODES; ++nd) {
            c->valid[nd] = h->valid[nd];
            c->allocated[nd] = h->allocated[nd];
        }
        if (h->allocated[RT_NODE_GPU]) {
            const struct _starpu_data_state *r = h->root;
            c->mat[RT_NODE_GPU].ld = r->mat[RT_NODE_GPU].ld;
            c->mat[RT_NODE_GPU].ptr = r->mat[RT_NODE_GPU].ptr + (c->row_off + c->col_off * r->mat[RT_NODE_GPU].ld) * c->elemsize;
        }
        h->children[i] = c;
    }
    h->partitioned = 1;
}

void starpu_data_map_filters(starpu_data_handle_t root, unsigned nfilters, ...)
{
    va_list ap;
    va_start(ap, nfilters);
    struct starpu_data_filter **fs = calloc(nfilters ? nfilters : 1, sizeof *fs);
    for (unsigned i = 0; i < nfilters; ++i) fs[i] = va_arg(ap, struct starpu_data_filter *);
    va_end(ap);
    if (nfilters == 0) {
        free(fs);
        return;
    }
    starpu_data_partition(root, fs[0]);
    /* apply the remaining filters recursively to every child */
    for (unsigned i = 0; i < root->nchildren && nfilters > 1; ++i) {
        struct _starpu_data_state *c = root->children[i];
        if (nfilters == 2) {
            starpu_data_partition(c, fs[1]);
        } else {
            /* deeper maps: partition level by level */
            starpu_data_partition(c, fs[1]);
            for (unsigned j = 0; j < c->nchildren; ++j) {
                for (unsigned l = 2; l < nfilters; ++l) starpu_data_partition(c->children[j], fs[l]);
            }
        }
    }
    free(fs);
}

starpu_data_handle_t starpu_data_get_child(starpu_data_handle_t h, unsigned i)
{
    STARPU_ASSERT_MSG(h->partitioned && i < h->nchildren, "no child %u", i);
    return h->children[i];
}

int starpu_data_get_nb_children(starpu_data_handle_t h) { return h->partitioned ? (int)h->nchildren : 0; }

starpu_data_handle_t starpu_data_get_sub_data(starpu_data_handle_t root, unsigned depth, ...)
{
    va_list ap;
    va_start(ap, depth);
    starpu_data_handle_t h = root;
    for (unsigned d = 0; d < depth; ++d) {
        unsigned i = va_arg(ap, unsigned);
        h = starpu_data_get_child(h, i);
    }
    va_end(ap);
    return h;
}

/* ------------------------------------------------------------- coherency */

static int ensure_gpu_alloc(starpu_data_handle_t h)
{
    if (h->allocated[RT_NODE_GPU]) return 0;
    if (h->id == STARPU_VARIABLE_INTERFACE_ID) {
        void *p = rt_cuda_alloc(h->elemsize ? h->elemsize : 1);
        if (!p) return -ENOMEM;
        h->var[RT_NODE_GPU].ptr = (uintptr_t)p;
        h->owned[RT_NODE_GPU] = p;
        h->allocated[RT_NODE_GPU] = 1;
        return 0;
    }
    struct _starpu_data_state *r = h->root;
    if (!r->allocated[RT_NODE_GPU]) {
        size_t bytes = r->mat[0].nx * r->mat[0].ny * r->elemsize;
        void *p = rt_cuda_alloc(bytes ? bytes : 1);
        if (!p) return -ENOMEM;
        r->mat[RT_NODE_GPU].ptr = (uintptr_t)p;
        r->mat[RT_NODE_GPU].ld = r->mat[0].nx;
        r->owned[RT_NODE_GPU] = p;
        r->owned_size[RT_NODE_GPU] = bytes;
        r->allocated[RT_NODE_GPU] = 1;
    }
    if (h != r) {
        h->mat[RT_NODE_GPU].ld = r->mat[RT_NODE_GPU].ld;
        h->mat[RT_NODE_GPU].ptr = r->mat[RT_NODE_GPU].ptr + (h->row_off + h->col_off * r->mat[RT_NODE_GPU].ld) * h->elemsize;
        h->allocated[RT_NODE_GPU] = 1;
    }
    return 0;
}

static int ensure_ram_alloc(starpu_data_handle_t h)
{
    if (h->allocated[RT_NODE_RAM]) return 0;
    if (h->id == STARPU_VARIABLE_INTERFACE_ID) {
        void *p = calloc(1, h->elemsize ? h->elemsize : 1);
        if (!p) return -ENOMEM;
        h->var[RT_NODE_RAM].ptr = (uintptr_t)p;
        h->owned[RT_NODE_RAM] = p;
        h->allocated[RT_NODE_RAM] = 1;
        return 0;
    }
    struct _starpu_data_state *r = h->root;
    if (!r->allocated[RT_NODE_RAM]) {
        size_t bytes = r->mat[0].nx * r->mat[0].ny * r->elemsize;
        void *p = NULL;
        if (posix_memalign(&p, 64, bytes ? bytes : 1)) return -ENOMEM;
        r->mat[RT_NODE_RAM].ptr = (uintptr_t)p;
        r->mat[RT_NODE_RAM].ld = r->mat[0].nx;
        r->owned[RT_NODE_RAM] = p;
        r->allocated[RT_NODE_RAM] = 1;
    }
    if (h != r) {
        h->mat[RT_NODE_RAM].ld = r->mat[RT_NODE_RAM].ld;
        h->mat[RT_NODE_RAM].ptr = r->mat[RT_NODE_RAM].ptr + (h->row_off + h->col_off * r->mat[RT_NODE_RAM].ld) * h->elemsize;
        h->allocated[RT_NODE_RAM] = 1;
    }
    return 0;
}

static int copy_between(starpu_data_handle_t h, int to, void *stream)
{
    const int from = 1 - to;
    int rc;
    if (h->id == STARPU_VARIABLE_INTERFACE_ID) {
        rc = rt_cuda_copy_2d(to == RT_NODE_GPU, (void *)h->var[to].ptr, h->elemsize, (const void *)h->var[from].ptr,
                             h->elemsize, h->elemsize, 1, stream);
    } else {
        const struct starpu_matrix_interface *d = &h->mat[to], *s = &h->mat[from];
        rc = rt_cuda_copy_2d(to == RT_NODE_GPU, (void *)d->ptr, d->ld * h->elemsize, (const void *)s->ptr,
                             s->ld * h->elemsize, d->nx * h->elemsize, d->ny, stream);
    }
    if (!rc) {
        if (to == RT_NODE_GPU) rt.stats.h2d_bytes += rt_data_size(h);
        else rt.stats.d2h_bytes += rt_data_size(h);
    }
    return rc;
}

int rt_data_node_ready(starpu_data_handle_t h, int node) { return h->valid[node]; }

/* Make h usable on `node` for `mode`: allocate there and, if the access
 * reads, copy the valid replica in (on `stream` for the GPU; synchronously
 * for host RAM).  Returns 0 or a negative errno. */
int rt_data_fetch(starpu_data_handle_t h, int node, enum starpu_data_access_mode mode, void *stream)
{
    int rc = node == RT_NODE_GPU ? ensure_gpu_alloc(h) : ensure_ram_alloc(h);
    if (rc) return rc;
    if ((mode & STARPU_R) && !h->valid[node] && h->valid[1 - node]) {
        rc = copy_between(h, node, node == RT_NODE_GPU ? stream : rt_cuda_transfer_stream());
        if (rc) return rc;
        if (node == RT_NODE_RAM) rt_cuda_sync_transfer_stream();
        h->valid[node] = 1;
    }
    return 0;
}

void rt_data_after_write(starpu_data_handle_t h, int node)
{
    h->valid[node] = 1;
    h->valid[1 - node] = 0;
}

void *rt_data_interface(starpu_data_handle_t h, int node)
{
    if (h->id == STARPU_VARIABLE_INTERFACE_ID) return &h->var[node];
    if (h->id == STARPU_VECTOR_INTERFACE_ID) {
        /* a vector is kept as an nx x 1 matrix; its codelets read the vector
         * interface's layout (elemsize where a matrix has ny) */
        const struct starpu_matrix_interface *m = &h->mat[node];
        struct starpu_vector_interface *v = &h->vec[node];
        v->id = STARPU_VECTOR_INTERFACE_ID;
        v->ptr = m->ptr;
        v->dev_handle = m->dev_handle;
        v->offset = m->offset;
        v->nx = m->nx;
        v->elemsize = m->elemsize;
        v->allocsize = m->nx * m->elemsize;
        v->slice_base = 0;
        return v;
    }
    return &h->mat[node];
}

void rt_data_forget_job(starpu_data_handle_t h, struct rt_job *j)
{
    if (h->last_writer == j) h->last_writer = NULL;
    for (int i = 0; i < h->nreaders; ++i)
        if (h->readers[i] == j) {
            h->readers[i] = h->readers[--h->nreaders];
            --i;
        }
    for (int i = 0; i < h->ncommuters; ++i)
        if (h->commuters[i] == j) {
            h->commuters[i] = h->commuters[--h->ncommuters];
            --i;
        }
}

/* Bring every child's data to `node`; returns whether all children are valid on the other node. */
static int gather(starpu_data_handle_t h, int node)
{
    if (!h->partitioned) {
        if (!h->valid[node] && h->valid[1 - node]) {
            if (node == RT_NODE_RAM) ensure_ram_alloc(h);
            else ensure_gpu_alloc(h);
            copy_between(h, node, rt_cuda_transfer_stream());
            rt_cuda_sync_transfer_stream();
            h->valid[node] = 1;
        }
        return h->valid[1 - node];
    }
    int all_other = 1;
    for (unsigned i = 0; i < h->nchildren; ++i) all_other &= gather(h->children[i], node);
    return all_other;
}

static void free_children(starpu_data_handle_t h)
{
    for (unsigned i = 0; i < h->nchildren; ++i) {
        struct _starpu_data_state *c = h->children[i];
        if (c->partitioned) free_children(c);
        free(c->readers);
        free(c->commuters);
        free(c);
    }
    free(h->children);
    h->children = NULL;
    h->nchildren = 0;
    h->partitioned = 0;
}

void starpu_data_unpartition(starpu_data_handle_t root, unsigned gathering_node)
{
    STARPU_ASSERT_MSG(root->partitioned, "handle is not partitioned");
    starpu_task_wait_for_all();
    int node = gathering_node == STARPU_MAIN_RAM ? RT_NODE_RAM : RT_NODE_GPU;
    int other_valid = gather(root, node);
    root->valid[node] = 1;
    root->valid[1 - node] = other_valid && root->allocated[1 - node];
    free_children(root);
}

void starpu_data_wont_use(starpu_data_handle_t handle) { (void)handle; }

void starpu_data_invalidate(starpu_data_handle_t h)
{
    starpu_task_wait_for_all();
    h->valid[RT_NODE_RAM] = h->valid[RT_NODE_GPU] = 0;
}

int starpu_data_acquire(starpu_data_handle_t h, enum starpu_data_access_mode mode)
{
    starpu_task_wait_for_all();
    if (mode & STARPU_R) gather(h, RT_NODE_RAM);
    if (mode & STARPU_W) rt_data_after_write(h, RT_NODE_RAM);
    return 0;
}

/* Asynchronous acquisition (datawizard/user_interactions.c): an internal
 * STARPU_NOWHERE task takes the access with the usual dependencies; its
 * prologue brings the data to RAM and calls `callback`, and an end
 * dependency keeps the access until starpu_data_release, so later tasks on
 * the handle wait for the release.  A graph-mode runtime (which records the
 * DAG before anything runs) acquires synchronously, then calls back. */
struct acquire_cb {
    starpu_data_handle_t h;
    enum starpu_data_access_mode mode;
    void (*callback)(void *);
    void *arg;
};

static void acquire_prologue(void *p)
{
    struct acquire_cb *a = p;
    rt_lock();
    if (a->mode & STARPU_R) gather(a->h, RT_NODE_RAM);
    if (a->mode & STARPU_W) rt_data_after_write(a->h, RT_NODE_RAM);
    rt_unlock();
    if (a->callback) a->callback(a->arg);
}

int starpu_data_acquire_cb(starpu_data_handle_t h, enum starpu_data_access_mode mode, void (*callback)(void *),
                           void *arg)
{
    if (rt.graph_mode) {
        starpu_data_acquire(h, mode);
        if (callback) callback(arg);
        return 0;
    }
    struct acquire_cb *a = malloc(sizeof *a);
    a->h = h;
    a->mode = mode;
    a->callback = callback;
    a->arg = arg;
    struct starpu_task *t = starpu_task_create();
    t->name = "acquire_cb";
    t->nbuffers = 1;
    t->handles[0] = h;
    t->modes[0] = mode;
    t->where = STARPU_NOWHERE;
    t->prologue_callback_func = acquire_prologue;
    t->prologue_callback_arg = a;
    t->prologue_callback_arg_free = 1;
    starpu_task_end_dep_add(t, 1);
    rt_lock();
    if (h->nacquired == h->capacquired) {
        h->capacquired = h->capacquired ? 2 * h->capacquired : 4;
        h->acquired = realloc(h->acquired, sizeof *h->acquired * h->capacquired);
    }
    h->acquired[h->nacquired++] = t;
    rt_unlock();
    return starpu_task_submit(t);
}

/* ends the oldest pending asynchronous acquisition of h; a synchronous one
 * holds nothing */
void starpu_data_release(starpu_data_handle_t h)
{
    struct starpu_task *t = NULL;
    rt_lock();
    if (h->nacquired) {
        t = h->acquired[0];
        memmove(h->acquired, h->acquired + 1, sizeof *h->acquired * --h->nacquired);
    }
    rt_unlock();
    if (t) starpu_task_end_dep_release(t);
}

static void unregister(starpu_data_handle_t h, int coherent)
{
    if (!h) return;
    starpu_task_wait_for_all();
    if (coherent && h->home_node == STARPU_MAIN_RAM) {
        if (h->partitioned) starpu_data_unpartition(h, STARPU_MAIN_RAM);
        gather(h, RT_NODE_RAM);
    } else if (h->partitioned) {
        free_children(h);
    }
    if (h->owned[RT_NODE_GPU]) rt_cuda_free(h->owned[RT_NODE_GPU]);
    if (h->owned[RT_NODE_RAM]) free(h->owned[RT_NODE_RAM]);
    free(h->readers);
    free(h->commuters);
    free(h->acquired);
    free(h);
}

void starpu_data_unregister(starpu_data_handle_t h) { unregister(h, 1); }
void starpu_data_unregister_no_coherency(starpu_data_handle_t h) { unregister(h, 0); }
