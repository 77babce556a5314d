/*
 * Runtime tests of libstarpu_gb300.so on CPU workers (no GPU needed), in the
 * style of the reference's tests/main/insert_task*.c,
 * tests/datawizard/data_implicit_deps.c, partition_*.c and tests/perfmodels/*.c.
 * Prints "ok <name>" per test; exit status 0 when every test passed.
 */
#include <math.h>
#include <starpu.h>
#include <unistd.h>

static int failures = 0;
#define CHECK(cond, name)                                                         \
    do {                                                                          \
        if (cond) printf("ok %s\n", name);                                        \
        else {                                                                    \
            printf("FAIL %s (%s:%d)\n", name, __FILE__, __LINE__);                \
            failures++;                                                           \
        }                                                                         \
    } while (0)

/* ---------------- codelets ---------------- */

/* v[0] = v[0] * 10 + digit (digit passed by value): order-sensitive */
static void append_digit(void *descr[], void *arg)
{
    int digit;
    starpu_codelet_unpack_args(arg, &digit, NULL);
    long *v = (long *)STARPU_VARIABLE_GET_PTR(descr[0]);
    usleep(1000 * (digit % 3));
    *v = *v * 10 + digit;
}
static struct starpu_codelet cl_append = {.cpu_funcs = {append_digit}, .nbuffers = 1, .modes = {STARPU_RW}};

/* dst = src (copy), slow so that a missing dependency would show */
static void copy_var(void *descr[], void *arg)
{
    (void)arg;
    usleep(2000);
    *(long *)STARPU_VARIABLE_GET_PTR(descr[1]) = *(long *)STARPU_VARIABLE_GET_PTR(descr[0]);
}
static struct starpu_codelet cl_copy = {.cpu_funcs = {copy_var}, .nbuffers = 2, .modes = {STARPU_R, STARPU_W}};

/* matrix tile += 1 */
static void tile_inc(void *descr[], void *arg)
{
    (void)arg;
    float *p = (float *)STARPU_MATRIX_GET_PTR(descr[0]);
    size_t nx = STARPU_MATRIX_GET_NX(descr[0]), ny = STARPU_MATRIX_GET_NY(descr[0]),
           ld = STARPU_MATRIX_GET_LD(descr[0]);
    for (size_t j = 0; j < ny; ++j)
        for (size_t i = 0; i < nx; ++i) p[i + j * ld] += 1.0f;
}
static struct starpu_perfmodel inc_model = {.type = STARPU_HISTORY_BASED, .symbol = "gb300_test_tile_inc"};
static struct starpu_codelet cl_inc = {
    .cpu_funcs = {tile_inc}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &inc_model, .name = "inc"};

static void noop(void *descr[], void *arg) { (void)descr; (void)arg; }
static void noop_cuda(void *descr[], void *arg) { (void)descr; (void)arg; }
static struct starpu_codelet cl_cuda_only = {.cuda_funcs = {noop_cuda}, .nbuffers = 0};
static struct starpu_codelet cl_noop = {.cpu_funcs = {noop}, .nbuffers = 0};

/* records the worker that ran task k */
static int ran_on[64];
static void where_k(void *descr[], void *arg)
{
    (void)descr;
    int k;
    starpu_codelet_unpack_args(arg, &k, NULL);
    ran_on[k] = starpu_worker_get_id();
}
static struct starpu_codelet cl_where = {.cpu_funcs = {where_k}, .nbuffers = 0};

/* b = a + 1, reported as failed on its first three runs */
static int ft_attempts = 0;
static void flaky_inc(void *descr[], void *arg)
{
    (void)arg;
    *(long *)STARPU_VARIABLE_GET_PTR(descr[1]) = *(long *)STARPU_VARIABLE_GET_PTR(descr[0]) + 1;
    if (++ft_attempts < 4) starpu_task_ft_failed(starpu_task_get_current());
}
static struct starpu_codelet cl_flaky = {.cpu_funcs = {flaky_inc}, .nbuffers = 2, .modes = {STARPU_R, STARPU_W}};

static void release_later(void *arg)
{
    usleep(20000);
    starpu_task_end_dep_release((struct starpu_task *)arg);
}

/* v += k, flagging any overlap with another commuting writer of v */
static int commute_active = 0, commute_overlap = 0;
static void commute_add(void *descr[], void *arg)
{
    int k;
    starpu_codelet_unpack_args(arg, &k, NULL);
    if (__sync_add_and_fetch(&commute_active, 1) != 1) __sync_fetch_and_add(&commute_overlap, 1);
    usleep(1000);
    *(long *)STARPU_VARIABLE_GET_PTR(descr[0]) += k;
    __sync_sub_and_fetch(&commute_active, 1);
}
static struct starpu_codelet cl_commute = {.cpu_funcs = {commute_add}, .nbuffers = 1, .modes = {STARPU_RW | STARPU_COMMUTE}};

/* every element of the vector block += its element size, read through the
 * vector interface */
static void vec_add_elemsize(void *descr[], void *arg)
{
    (void)arg;
    int *p = (int *)STARPU_VECTOR_GET_PTR(descr[0]);
    const size_t nx = STARPU_VECTOR_GET_NX(descr[0]), es = STARPU_VECTOR_GET_ELEMSIZE(descr[0]);
    for (size_t i = 0; i < nx; ++i) p[i] += (int)es;
}
static struct starpu_codelet cl_vec = {.cpu_funcs = {vec_add_elemsize}, .nbuffers = 1, .modes = {STARPU_RW}};

static int slow_done = 0;
static void slow_fn(void *descr[], void *arg)
{
    (void)descr;
    (void)arg;
    usleep(20000);
    __sync_fetch_and_add(&slow_done, 1);
}
static struct starpu_codelet cl_slow = {.cpu_funcs = {slow_fn}, .nbuffers = 0};

static int cb_count = 0;
static void cb(void *arg) { __sync_fetch_and_add(&cb_count, *(int *)arg); }

int main(void)
{
    setenv("STARPU_NCUDA", "0", 0);
    int ret = starpu_init(NULL);
    CHECK(ret == 0, "init");
    CHECK(starpu_cpu_worker_get_count() >= 1, "cpu_workers");

    /* 1. sequential consistency on one variable: RW tasks run in submission order */
    {
        long v = 0;
        starpu_data_handle_t h;
        starpu_variable_data_register(&h, STARPU_MAIN_RAM, (uintptr_t)&v, sizeof v);
        for (int d = 1; d <= 9; ++d)
            starpu_task_insert(&cl_append, STARPU_VALUE, &d, sizeof d, STARPU_RW, h, 0);
        starpu_task_wait_for_all();
        starpu_data_unregister(h);
        CHECK(v == 123456789, "rw_chain_order");
    }
    /* 2. RAW / WAR: b = a; a = 5 (the write must wait for the read); c = b */
    {
        long a = 7, b = 0, c = 0;
        starpu_data_handle_t ha, hb, hc;
        starpu_variable_data_register(&ha, STARPU_MAIN_RAM, (uintptr_t)&a, sizeof a);
        starpu_variable_data_register(&hb, STARPU_MAIN_RAM, (uintptr_t)&b, sizeof b);
        starpu_variable_data_register(&hc, STARPU_MAIN_RAM, (uintptr_t)&c, sizeof c);
        starpu_task_insert(&cl_copy, STARPU_R, ha, STARPU_W, hb, 0);
        int five = 5;
        long zero = 0;
        (void)zero;
        starpu_task_insert(&cl_append, STARPU_VALUE, &five, sizeof five, STARPU_RW, ha, 0); /* a = 75 */
        starpu_task_insert(&cl_copy, STARPU_R, hb, STARPU_W, hc, 0);
        starpu_task_wait_for_all();
        starpu_data_unregister(ha);
        starpu_data_unregister(hb);
        starpu_data_unregister(hc);
        CHECK(b == 7 && c == 7 && a == 75, "raw_war_edges");
    }
    /* 3. 2-level block filters with a ragged remainder, tasks on tiles, unpartition */
    {
        const unsigned n = 10, nb = 3;
        float *m = calloc(n * n, sizeof *m);
        starpu_data_handle_t h;
        starpu_matrix_data_register(&h, STARPU_MAIN_RAM, (uintptr_t)m, n, n, n, sizeof(float));
        struct starpu_data_filter f = {.filter_func = starpu_matrix_filter_block, .nchildren = nb};
        struct starpu_data_filter f2 = {.filter_func = starpu_matrix_filter_vertical_block, .nchildren = nb};
        starpu_data_map_filters(h, 2, &f, &f2);
        int shapes_ok = 1;
        for (unsigned i = 0; i < nb; ++i)
            for (unsigned j = 0; j < nb; ++j) {
                starpu_data_handle_t t = starpu_data_get_sub_data(h, 2, i, j);
                size_t ex_nx = n / nb + (i < n % nb), ex_ny = n / nb + (j < n % nb);
                shapes_ok &= starpu_matrix_get_nx(t) == ex_nx && starpu_matrix_get_ny(t) == ex_ny;
                for (unsigned r = 0; r <= i + j; ++r) starpu_task_insert(&cl_inc, STARPU_RW, t, 0);
            }
        starpu_task_wait_for_all();
        starpu_data_unpartition(h, STARPU_MAIN_RAM);
        starpu_data_unregister(h);
        int vals_ok = 1;
        for (unsigned jj = 0; jj < n; ++jj)
            for (unsigned ii = 0; ii < n; ++ii) {
                unsigned bi = ii < 4 ? 0 : ii < 7 ? 1 : 2, bj = jj < 4 ? 0 : jj < 7 ? 1 : 2;
                vals_ok &= m[ii + jj * n] == (float)(bi + bj + 1);
            }
        free(m);
        CHECK(shapes_ok, "filter_ragged_shapes");
        CHECK(vals_ok, "tile_tasks_and_unpartition");
    }
    /* 4. callbacks, priorities, task_build/destroy, -ENODEV */
    {
        int one = 1;
        for (int i = 0; i < 20; ++i)
            starpu_task_insert(&cl_noop, STARPU_CALLBACK_WITH_ARG, cb, &one, STARPU_PRIORITY, i, 0);
        starpu_task_wait_for_all();
        CHECK(cb_count == 20, "callbacks");
        struct starpu_task *t = starpu_task_build(&cl_noop, 0);
        CHECK(t && t->cl == &cl_noop, "task_build");
        t->destroy = 0;
        starpu_task_destroy(t);
        CHECK(starpu_task_insert(&cl_cuda_only, 0) == -ENODEV, "enodev_without_cuda_worker");
        CHECK(STARPU_MAX_PRIO == INT_MAX && STARPU_MIN_PRIO == INT_MIN, "unbounded_priorities");
    }
    /* 5. tags: C depends on A and B through declared tag dependencies */
    {
        long v = 0;
        starpu_data_handle_t h;
        starpu_variable_data_register(&h, STARPU_MAIN_RAM, (uintptr_t)&v, sizeof v);
        starpu_tag_declare_deps((starpu_tag_t)3, 2, (starpu_tag_t)1, (starpu_tag_t)2);
        int d1 = 1, d2 = 2, d3 = 3;
        starpu_task_insert(&cl_append, STARPU_VALUE, &d3, sizeof d3, STARPU_TAG, (starpu_tag_t)3, STARPU_RW, h,
                           STARPU_SEQUENTIAL_CONSISTENCY, 0, 0);
        starpu_task_insert(&cl_append, STARPU_VALUE, &d1, sizeof d1, STARPU_TAG, (starpu_tag_t)1, STARPU_RW, h,
                           STARPU_SEQUENTIAL_CONSISTENCY, 0, 0);
        starpu_task_insert(&cl_append, STARPU_VALUE, &d2, sizeof d2, STARPU_TAG, (starpu_tag_t)2, STARPU_RW, h,
                           STARPU_SEQUENTIAL_CONSISTENCY, 0, 0);
        starpu_tag_wait((starpu_tag_t)3);
        starpu_task_wait_for_all();
        starpu_data_unregister(h);
        /* 3 runs last; 1 and 2 may run in either order (no data ordering requested) */
        CHECK(v == 123 || v == 213, "tag_dependencies");
    }
    /* 6. history perfmodel: calibrated after enough runs, saved and reloaded */
    {
        float tile[64 * 64] = {0};
        starpu_data_handle_t h;
        starpu_matrix_data_register(&h, STARPU_MAIN_RAM, (uintptr_t)tile, 64, 64, 64, sizeof(float));
        for (int i = 0; i < 12; ++i) starpu_task_insert(&cl_inc, STARPU_RW, h, 0);
        starpu_task_wait_for_all();
        struct starpu_task *t = starpu_task_build(&cl_inc, STARPU_RW, h, 0);
        double len = starpu_task_expected_length(t, starpu_worker_get_perf_archtype(0, 0), 0);
        t->destroy = 0;
        starpu_task_destroy(t);
        starpu_data_unregister(h);
        CHECK(!isnan(len) && len >= 0, "perfmodel_calibrated");
        CHECK(starpu_save_history_based_model(&inc_model) == 0, "perfmodel_saved");
        char path[1024];
        starpu_perfmodel_get_model_path("gb300_test_tile_inc", path, sizeof path);
        FILE *f = fopen(path, "r");
        char line[256] = "";
        if (f) {
            fgets(line, sizeof line, f);
            fgets(line, sizeof line, f);
            fgets(line, sizeof line, f);
            fclose(f);
        }
        CHECK(f && atoi(line) == 45, "perfmodel_file_version_45");
        struct starpu_perfmodel loaded;
        CHECK(starpu_perfmodel_load_symbol("gb300_test_tile_inc", &loaded) == 0, "perfmodel_reload");
        starpu_perfmodel_unload_model(&loaded);
    }
    /* fault tolerance with the default retry policy (task.c:2522-2541): the
     * work runs until it stops failing; a task reading its output waits for
     * the meta task, which holds the data until then */
    {
        long a = 5, b = 0, c = 0;
        starpu_data_handle_t ha, hb, hc;
        starpu_variable_data_register(&ha, STARPU_MAIN_RAM, (uintptr_t)&a, sizeof a);
        starpu_variable_data_register(&hb, STARPU_MAIN_RAM, (uintptr_t)&b, sizeof b);
        starpu_variable_data_register(&hc, STARPU_MAIN_RAM, (uintptr_t)&c, sizeof c);
        int rc = starpu_task_insert(&cl_flaky, STARPU_PROLOGUE_CALLBACK, starpu_task_ft_prologue,
                                    STARPU_PROLOGUE_CALLBACK_ARG_NFREE, NULL, STARPU_R, ha, STARPU_W, hb, 0);
        rc |= starpu_task_insert(&cl_copy, STARPU_R, hb, STARPU_W, hc, 0);
        starpu_task_wait_for_all();
        starpu_data_unregister(ha);
        starpu_data_unregister(hb);
        starpu_data_unregister(hc);
        CHECK(rc == 0 && ft_attempts == 4 && b == 6 && c == 6 && a == 5, "ft_default_retry");
    }
    /* end dependencies (jobs.c:339-373): a STARPU_NOWHERE task holding its
     * data terminates only on the release, and its reader waits for that */
    {
        long v = 0, w = -1;
        starpu_data_handle_t hv, hw;
        starpu_variable_data_register(&hv, STARPU_MAIN_RAM, (uintptr_t)&v, sizeof v);
        starpu_variable_data_register(&hw, STARPU_MAIN_RAM, (uintptr_t)&w, sizeof w);
        struct starpu_task *hold = starpu_task_create();
        hold->cl = &cl_flaky;
        hold->handles[0] = hv;
        hold->handles[1] = hv;
        hold->modes[0] = STARPU_R;
        hold->modes[1] = STARPU_W;
        hold->where = STARPU_NOWHERE;
        starpu_task_end_dep_add(hold, 1); /* before submission */
        int rc = starpu_task_submit(hold);
        rc |= starpu_task_insert(&cl_copy, STARPU_R, hv, STARPU_W, hw, 0);
        usleep(5000);
        const long before = w; /* the copy cannot have run yet */
        v = 42;                /* the held data, written while the meta task owns it */
        pthread_t th;
        pthread_create(&th, NULL, (void *(*)(void *))release_later, hold);
        starpu_task_wait_for_all();
        pthread_join(th, NULL);
        starpu_data_unregister(hv);
        starpu_data_unregister(hw);
        CHECK(rc == 0 && before == -1 && w == 42, "end_dep_holds_termination");
    }
    /* end dependencies on tasks (starpu_task_dep.h): m is reported done only
     * once s1 (submitted) and s2 (submitted after the declaration) are */
    {
        struct starpu_task *m = starpu_task_create(), *s1 = starpu_task_create(), *s2 = starpu_task_create();
        m->cl = &cl_noop;
        m->detach = 0;
        m->destroy = 0;
        s1->cl = &cl_slow;
        s2->cl = &cl_slow;
        int rc = starpu_task_submit(s1);
        starpu_task_declare_end_deps(m, 2, s1, s2);
        rc |= starpu_task_submit(m);
        usleep(2000);
        rc |= starpu_task_submit(s2);
        rc |= starpu_task_wait(m);
        const int done_at_wait = slow_done;
        starpu_task_destroy(m);
        starpu_task_wait_for_all();
        CHECK(rc == 0 && done_at_wait == 2, "end_deps_on_tasks");
    }
    /* vectors: the codelet's view has the vector layout, and 3 blocks of 10
     * elements (4, 3, 3: vector_filters.c) cover every element once */
    {
        int vv[10] = {0};
        starpu_data_handle_t hv;
        starpu_vector_data_register(&hv, STARPU_MAIN_RAM, (uintptr_t)vv, 10, sizeof(int));
        struct starpu_data_filter f = {.filter_func = starpu_vector_filter_block, .nchildren = 3};
        starpu_data_partition(hv, &f);
        int rc = 0;
        for (unsigned c = 0; c < 3; ++c) rc |= starpu_task_insert(&cl_vec, STARPU_RW, starpu_data_get_sub_data(hv, 1, c), 0);
        starpu_task_wait_for_all();
        starpu_data_unpartition(hv, STARPU_MAIN_RAM);
        starpu_data_unregister(hv);
        int ok = rc == 0;
        for (int i = 0; i < 10; ++i) ok &= vv[i] == (int)sizeof(int);
        CHECK(ok, "vector_blocks_and_elemsize");
    }
    /* commuting writers (STARPU_RW | STARPU_COMMUTE): any order, never two at
     * once on one handle; a plain reader after them sees all of them */
    {
        long v = 0, w = -1;
        starpu_data_handle_t hv, hw;
        starpu_variable_data_register(&hv, STARPU_MAIN_RAM, (uintptr_t)&v, sizeof v);
        starpu_variable_data_register(&hw, STARPU_MAIN_RAM, (uintptr_t)&w, sizeof w);
        int rc = 0;
        for (int k = 1; k <= 16; ++k) rc |= starpu_task_insert(&cl_commute, STARPU_VALUE, &k, sizeof k, STARPU_RW | STARPU_COMMUTE, hv, 0);
        rc |= starpu_task_insert(&cl_copy, STARPU_R, hv, STARPU_W, hw, 0);
        starpu_task_wait_for_all();
        starpu_data_unregister(hv);
        starpu_data_unregister(hw);
        CHECK(rc == 0 && commute_overlap == 0 && v == 136 && w == 136, "commute_exclusive_then_reader");
    }
    /* scheduling contexts (src/core/sched_ctx.c): a context's tasks run on
     * its workers only; a context without a capable worker refuses tasks;
     * a deleted context hands its workers to its inheritor */
    {
        const int nw = (int)starpu_worker_get_count();
        const int half = nw >= 2 ? nw / 2 : 1;
        int wa[STARPU_NMAXWORKERS], wb[STARPU_NMAXWORKERS], na = 0, nb = 0;
        for (int w = 0; w < nw; ++w) {
            if (w < half) wa[na++] = w;
            if (w >= half || nw == 1) wb[nb++] = w;
        }
        unsigned ca = starpu_sched_ctx_create(wa, na, "ctx_a", STARPU_SCHED_CTX_POLICY_NAME, "dmda", 0);
        unsigned cb2 = starpu_sched_ctx_create(wb, nb, "ctx_b", 0);
        CHECK(ca != 0 && cb2 != 0 && ca != cb2, "ctx_create");
        CHECK(starpu_sched_ctx_get_context() == STARPU_NMAX_SCHED_CTXS, "ctx_none_current");
        CHECK(starpu_sched_ctx_get_nworkers(ca) == (unsigned)na && starpu_sched_ctx_get_nworkers(cb2) == (unsigned)nb,
              "ctx_nworkers");
        for (int k = 0; k < 64; ++k) ran_on[k] = -1;
        /* 32 tasks named to a context by STARPU_SCHED_CTX, 32 through the current one */
        int submitted = 1;
        for (int k = 0; k < 32; ++k)
            submitted &= starpu_task_insert(&cl_where, STARPU_VALUE, &k, sizeof k, STARPU_SCHED_CTX,
                                            (k & 1) ? ca : cb2, 0) == 0;
        starpu_sched_ctx_set_context(&ca);
        for (int k = 32; k < 64; ++k) submitted &= starpu_task_insert(&cl_where, STARPU_VALUE, &k, sizeof k, 0) == 0;
        CHECK(starpu_sched_ctx_get_context() == ca, "ctx_current");
        starpu_sched_ctx_set_context(NULL);
        starpu_task_wait_for_all();
        int placed = submitted;
        for (int k = 0; k < 64; ++k) {
            const unsigned c = k < 32 ? ((k & 1) ? ca : cb2) : ca;
            placed &= ran_on[k] >= 0 && starpu_sched_ctx_contains_worker(ran_on[k], c);
        }
        CHECK(placed, "ctx_tasks_on_their_workers");
        unsigned empty = starpu_sched_ctx_create(NULL, 0, "ctx_empty", 0);
        CHECK(starpu_task_insert(&cl_noop, STARPU_SCHED_CTX, empty, 0) == -ENODEV, "ctx_enodev_without_workers");
        starpu_sched_ctx_set_inheritor(ca, cb2);
        starpu_sched_ctx_delete(ca);
        CHECK(starpu_sched_ctx_get_nworkers(cb2) == (unsigned)nw, "ctx_delete_hands_workers_to_inheritor");
        starpu_sched_ctx_delete(cb2);
        starpu_sched_ctx_delete(empty);
        /* a task named to a deleted context runs in the initial one */
        CHECK(starpu_task_insert(&cl_noop, STARPU_SCHED_CTX, ca, 0) == 0, "ctx_deleted_falls_back_to_initial");
        starpu_task_wait_for_all();
    }
    starpu_shutdown();
    printf("%s\n", failures ? "FAILED" : "ALL OK");
    return failures ? 1 : 0;
}
