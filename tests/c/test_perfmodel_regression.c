/*
 * Regression-based and cost-function performance models through the StarPU
 * API of libstarpu_gb300.so on CPU workers (STARPU_NCPU=2):
 *   - a linear regression model (time = alpha size^beta) recorded over seven
 *     data sizes, its prediction inside and outside the measured size range,
 *     its file, and a runtime reload that keeps the fit but not the entries;
 *   - a non-linear model (time = a size^b + c): the entry's mean before the
 *     fit exists, the fit written when it is saved, the prediction from the
 *     reloaded fit and the fallback outside the size range;
 *   - common, per-arch and per-worker cost-function models, and the
 *     scheduler placing a task by its per-worker cost.
 * Prints "KEY value" lines that tests/test_perfmodel_tools.py replays through
 * the oracle, and "ALL OK" last when every check here passed.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <starpu.h>

static int failures;
#define CHECK(c, what)                                                                                       \
    do {                                                                                                     \
        if (!(c)) {                                                                                          \
            fprintf(stderr, "FAILED: %s\n", what);                                                           \
            ++failures;                                                                                      \
        }                                                                                                    \
    } while (0)

#define NSIZES 7
static const int dims[NSIZES] = {16, 24, 32, 48, 64, 96, 128}; /* float n x n tiles: 4 n^2 bytes */
static const double lin_us[NSIZES] = {26, 53, 89, 185, 310, 644, 1081};  /* ~0.05 size^0.9 */
static const double nl_us[NSIZES] = {14, 20, 29, 56, 96, 221, 407};      /* ~2e-3 size^1.1 + 10 */
static float tiles[128 * 256];

static int ran_on = -1;
static void noop(void *buffers[], void *arg)
{
    (void)buffers;
    (void)arg;
}
static void where(void *buffers[], void *arg)
{
    (void)buffers;
    (void)arg;
    ran_on = starpu_worker_get_id();
}

static double common_cost(struct starpu_task *t, unsigned nimpl)
{
    (void)t;
    (void)nimpl;
    return 1000.0;
}
static double arch_cost(struct starpu_task *t, struct starpu_perfmodel_arch *arch, unsigned nimpl)
{
    (void)t;
    (void)nimpl;
    return 3.0 + arch->ndevices;
}
static double worker_cost(struct starpu_task *t, unsigned workerid, unsigned nimpl)
{
    (void)t;
    (void)nimpl;
    return workerid == 1 ? 5.0 : 1e9;
}

static struct starpu_perfmodel lin = {.type = STARPU_REGRESSION_BASED, .symbol = "gb300_test_perfmodel_lreg"};
static struct starpu_perfmodel lin2 = {.type = STARPU_REGRESSION_BASED, .symbol = "gb300_test_perfmodel_lreg"};
static struct starpu_perfmodel nl = {.type = STARPU_NL_REGRESSION_BASED, .symbol = "gb300_test_perfmodel_nlreg"};
static struct starpu_perfmodel nl2 = {.type = STARPU_NL_REGRESSION_BASED, .symbol = "gb300_test_perfmodel_nlreg"};
static struct starpu_perfmodel common = {.type = STARPU_COMMON, .cost_function = common_cost};
static struct starpu_perfmodel per_arch = {.type = STARPU_PER_ARCH, .arch_cost_function = arch_cost};
static struct starpu_perfmodel per_worker = {.type = STARPU_PER_WORKER, .worker_cost_function = worker_cost};

static struct starpu_codelet cl_lin = {.cpu_funcs = {noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &lin};
static struct starpu_codelet cl_lin2 = {.cpu_funcs = {noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &lin2};
static struct starpu_codelet cl_nl = {.cpu_funcs = {noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &nl};
static struct starpu_codelet cl_nl2 = {.cpu_funcs = {noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &nl2};
static struct starpu_codelet cl_common = {.cpu_funcs = {noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &common};
static struct starpu_codelet cl_arch = {.cpu_funcs = {noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &per_arch};
static struct starpu_codelet cl_worker = {.cpu_funcs = {where}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &per_worker};

/* a task of codelet cl on an n x n float tile (not submitted) */
static struct starpu_task *tile_task(struct starpu_codelet *cl, int n, starpu_data_handle_t *h)
{
    starpu_matrix_data_register(h, STARPU_MAIN_RAM, (uintptr_t)tiles, n, n, n, sizeof(float));
    struct starpu_task *t = starpu_task_build(cl, STARPU_RW, *h, 0);
    t->destroy = 0;
    return t;
}

static void drop(struct starpu_task *t, starpu_data_handle_t h)
{
    starpu_task_destroy(t);
    starpu_data_unregister(h);
}

/* expected length of a task of cl on an n x n tile, printed as KEY */
static double expect(const char *key, struct starpu_codelet *cl, int n, struct starpu_perfmodel_arch *arch)
{
    starpu_data_handle_t h;
    struct starpu_task *t = tile_task(cl, n, &h);
    const double v = starpu_task_expected_length(t, arch, 0);
    printf("%s %.17g\n", key, v);
    drop(t, h);
    return v;
}

int main(void)
{
    if (starpu_init(NULL) != 0) return 77;
    struct starpu_perfmodel_arch *arch = starpu_worker_get_perf_archtype(0, 0);
    printf("CPU_CORES %d\n", arch->devices[0].ncores);

    /* linear regression: three calls per size */
    for (int k = 0; k < NSIZES; ++k) {
        starpu_data_handle_t h;
        struct starpu_task *t = tile_task(&cl_lin, dims[k], &h);
        for (int i = 0; i < 3; ++i) starpu_perfmodel_update_history(&lin, t, arch, 0, 0, lin_us[k]);
        drop(t, h);
    }
    expect("LIN_IN", &cl_lin, 64, arch);
    CHECK(isnan(expect("LIN_OUT", &cl_lin, 256, arch)), "no linear prediction outside [0.9 minx, 1.1 maxx]");
    CHECK(starpu_save_history_based_model(&lin) == 0, "save the linear model");
    {
        /* a runtime load of a linear model keeps the fit, not the entries */
        starpu_data_handle_t h;
        struct starpu_task *t = tile_task(&cl_lin2, 64, &h);
        printf("LIN_RELOAD %.17g\n", starpu_task_expected_length(t, arch, 0));
        const uint32_t fp = starpu_task_footprint(&lin2, t, arch, 0);
        CHECK(isnan(starpu_perfmodel_history_based_expected_perf(&lin2, arch, fp)), "reloaded linear model has no entries");
        drop(t, h);
    }

    /* non-linear regression: twelve equal calls per size (the first is kept:
     * this is not a history-based model), then the fit at save */
    for (int k = 0; k < NSIZES; ++k) {
        starpu_data_handle_t h;
        struct starpu_task *t = tile_task(&cl_nl, dims[k], &h);
        for (int i = 0; i < 12; ++i) starpu_perfmodel_update_history(&nl, t, arch, 0, 0, nl_us[k]);
        drop(t, h);
    }
    CHECK(expect("NL_BEFORE_FIT", &cl_nl, 64, arch) == nl_us[4], "entry mean before the fit exists");
    CHECK(starpu_save_history_based_model(&nl) == 0, "save the non-linear model");
    expect("NL_RELOAD", &cl_nl2, 64, arch);
    CHECK(isnan(expect("NL_OUT", &cl_nl2, 256, arch)), "outside the range and without an entry: no prediction");

    /* cost-function models */
    printf("SPEEDUP %.17g\n", starpu_worker_get_relative_speedup(arch));
    expect("COMMON", &cl_common, 32, arch);
    CHECK(expect("PER_ARCH", &cl_arch, 32, arch) == 4.0, "per-arch cost function");
    {
        starpu_data_handle_t h;
        struct starpu_task *t = tile_task(&cl_worker, 32, &h);
        CHECK(starpu_task_worker_expected_length(t, 0, 0, 0) == 1e9, "per-worker cost of worker 0");
        CHECK(starpu_task_worker_expected_length(t, 1, 0, 0) == 5.0, "per-worker cost of worker 1");
        CHECK(isnan(starpu_task_expected_length(t, arch, 0)), "a per-worker model has no per-arch prediction");
        drop(t, h);
        /* dmda places the task on the worker its cost function prefers */
        starpu_data_handle_t h2;
        starpu_matrix_data_register(&h2, STARPU_MAIN_RAM, (uintptr_t)tiles, 32, 32, 32, sizeof(float));
        CHECK(starpu_task_insert(&cl_worker, STARPU_RW, h2, 0) == 0, "submit");
        starpu_task_wait_for_all();
        printf("PER_WORKER_RAN_ON %d\n", ran_on);
        CHECK(ran_on == 1, "scheduled on the cheaper worker");
        starpu_data_unregister(h2);
    }

    char path[2048];
    starpu_perfmodel_get_model_path(lin.symbol, path, sizeof path);
    printf("LIN_PATH %s\n", path);
    starpu_perfmodel_get_model_path(nl.symbol, path, sizeof path);
    printf("NL_PATH %s\n", path);
    starpu_shutdown();
    printf("%s\n", failures ? "FAILED" : "ALL OK");
    return failures ? 1 : 0;
}
