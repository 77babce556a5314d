/*
 * History-model recording and the version-45 file, through the StarPU API of
 * libstarpu_gb300.so on CPU workers: samples for three data sizes on two
 * implementations (a new entry's single first sample is not kept; a batch of
 * several is), an outlier that the STARPU_HISTORY_MAX_ERROR rule drops,
 * then a save, a reload by symbol and the tooling printout of the reload.
 * Prints "ALL OK" last when every check passed.
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

static void noop(void *buffers[], void *arg)
{
    (void)buffers;
    (void)arg;
}

static struct starpu_perfmodel model = {.type = STARPU_HISTORY_BASED, .symbol = "gb300_test_perfmodel_io"};
static struct starpu_codelet cl = {.cpu_funcs = {noop, noop}, .nbuffers = 1, .modes = {STARPU_RW}, .model = &model};

int main(void)
{
    if (starpu_init(NULL) != 0) return 77;
    struct starpu_perfmodel_arch *arch = starpu_worker_get_perf_archtype(0, 0);
    static float tiles[3][128 * 128];
    const int sizes[3] = {32, 64, 128};
    for (int k = 0; k < 3; ++k) {
        starpu_data_handle_t h;
        starpu_matrix_data_register(&h, STARPU_MAIN_RAM, (uintptr_t)tiles[k], sizes[k], sizes[k], sizes[k],
                                    sizeof(float));
        struct starpu_task *t = starpu_task_build(&cl, STARPU_RW, h, 0);
        t->flops = 2.0 * sizes[k] * sizes[k] * sizes[k];
        for (int i = 0; i < 12; ++i) starpu_perfmodel_update_history(&model, t, arch, 0, 0, 100.0 * (k + 1) + (i & 1));
        /* 10x the mean: dropped as an error, not a sample */
        starpu_perfmodel_update_history(&model, t, arch, 0, 0, 1000.0 * (k + 1));
        starpu_perfmodel_update_history_n(&model, t, arch, 0, 1, 50.0 * (k + 1), 4);
        const uint32_t fp = starpu_task_footprint(&model, t, arch, 0);
        const double mean = starpu_perfmodel_history_based_expected_perf(&model, arch, fp);
        /* the first of the 12 (100 (k+1), i = 0) opens the entry and is not
         * kept (perfmodel_history.c:1926-1933); of the 11 kept, 6 are +1 */
        CHECK(fabs(mean - (100.0 * (k + 1) + 6.0 / 11.0)) < 1e-9, "mean of the kept samples");
        if (k == 0) {
            /* one mean per worker (all CPU workers share the CPU combination) */
            printf("ESTIMATIONS ");
            starpu_perfmodel_print_estimations(&model, fp, stdout);
            printf("\n");
        }
        CHECK(fabs(starpu_task_expected_length(t, arch, 0) - mean) < 1e-9, "expected length = history mean");
        t->destroy = 0;
        starpu_task_destroy(t);
        starpu_data_unregister(h);
    }
    CHECK(starpu_save_history_based_model(&model) == 0, "save");
    char path[2048];
    starpu_perfmodel_get_model_path(model.symbol, path, sizeof path);
    CHECK(path[0] != 0, "model path exists after the save");
    printf("PATH %s\n", path);

    struct starpu_perfmodel loaded;
    CHECK(starpu_perfmodel_load_symbol(model.symbol, &loaded) == 0, "reload");
    CHECK(loaded.type == STARPU_HISTORY_BASED, "reloaded type");
    printf("BEGIN_PRINT\n");
    starpu_perfmodel_print_all(&loaded, NULL, NULL, NULL, stdout);
    printf("END_PRINT\n");
    starpu_perfmodel_unload_model(&loaded);
    struct starpu_perfmodel missing;
    CHECK(starpu_perfmodel_load_symbol("gb300_no_such_model", &missing) == 1, "missing model loads with 1");
    starpu_shutdown();
    printf("%s\n", failures ? "FAILED" : "ALL OK");
    return failures ? 1 : 0;
}
