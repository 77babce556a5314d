/*
 * starpu_perfmodel_plot: write a gnuplot script (starpu_<symbol>.gp) and its
 * averages file (starpu_<symbol>_avg.data) drawing a history-based model, with
 * the options of StarPU's tools/starpu_perfmodel_plot.c:
 *   -s <symbol>           the model to draw
 *   -se <time> <energy>   power from a time model and an energy model
 *   -e                    the model holds energies (J), not times
 *   -f                    draw GFlop/s instead of time
 *   -lc                   list the model's architecture combinations
 *   -c <comb>             draw only that combination
 *   -o <dir>              output directory (default ".")
 *   -l / -d               list the model files / print the directories
 * FxT traces (-i) are not recorded by this runtime: the option is accepted and
 * its files ignored, as StarPU does when built without FxT.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <starpu.h>

#define PROGNAME "starpu_perfmodel_plot"

static void usage(void)
{
    fprintf(stderr,
            "Draw a graph corresponding to the execution time of a given perfmodel\n"
            "Usage: %s [ options ]\n\n"
            "One must specify a symbol with the -s option or use -l or -d\n"
            "Options:\n"
            "   -d\t\t\tdisplay the directory storing performance models\n"
            "   -l\t\t\tdisplay all available models\n"
            "   -s <symbol>\t\tspecify the symbol\n"
            "   -e\t\t\tdisplay perfmodel as energy instead of time\n"
            "   -se <time_symbol> <energy_symbol> \n"
            "\t\t\tspecify both a time symbol and an energy symbol\n"
            "   -f\t\t\tdraw GFlop/s instead of time\n"
            "   -i <Fxt files>\tinput FxT files generated by StarPU\n"
            "   -lc\t\t\tdisplay all combinations of a given model\n"
            "   -c <combination>\tspecify the combination (use the option -lc to list all combinations of a given "
            "model)\n"
            "   -o <directory>\tspecify directory in which to create output files (current directory by default)\n"
            "   -h, --help\t\tdisplay this help and exit\n"
            "   -v, --version\toutput version information and exit\n",
            PROGNAME);
}

int main(int argc, char **argv)
{
    const char *symbol = NULL, *energy_symbol = NULL, *dir = ".";
    int list = 0, directory = 0, list_combs = 0, gflops = 0, energy = 0, comb = -1, ok = 0, reading_inputs = 0;
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (!strcmp(a, "-s") || !strcmp(a, "-se") || !strcmp(a, "-c") || !strcmp(a, "-o") || !strcmp(a, "-i")) {
            const int need = !strcmp(a, "-se") ? 2 : 1;
            if (i + need >= argc) {
                fprintf(stderr, "%s requires %s\n", a, need == 2 ? "two arguments" : "an argument");
                usage();
                return 1;
            }
        }
        if (!strcmp(a, "-s")) {
            symbol = argv[++i];
            ok = 1;
        } else if (!strcmp(a, "-se")) {
            symbol = argv[++i];
            energy_symbol = argv[++i];
            ok = 1;
        } else if (!strcmp(a, "-o")) {
            dir = argv[++i];
        } else if (!strcmp(a, "-i")) {
            reading_inputs = 1;
            fprintf(stderr, "Warning: FxT traces are not recorded by this runtime: they will be ignored!\n");
        } else if (!strcmp(a, "-l")) {
            list = ok = 1;
        } else if (!strcmp(a, "-lc")) {
            list_combs = 1;
        } else if (!strcmp(a, "-f")) {
            gflops = 1;
        } else if (!strcmp(a, "-e")) {
            energy = 1;
        } else if (!strcmp(a, "-c")) {
            comb = atoi(argv[++i]);
        } else if (!strcmp(a, "-d")) {
            directory = ok = 1;
        } else if (!strcmp(a, "-h") || !strcmp(a, "--help")) {
            usage();
            return 0;
        } else if (!strcmp(a, "-v") || !strcmp(a, "--version")) {
            fputs(PROGNAME " (starpu_gb300)\n", stderr);
            return 0;
        } else if (!reading_inputs) {
            fprintf(stderr, "Unknown option %s\n", a);
        }
    }
    if (!ok) {
        fprintf(stderr, "Incorrect usage, aborting\n");
        usage();
        return 255;
    }
    starpu_drivers_preinit();
    starpu_perfmodel_initialize();
    int rc = 0;
    if (directory) {
        starpu_perfmodel_directory(stdout);
    } else if (list) {
        rc = starpu_perfmodel_list(stdout);
    } else {
        struct starpu_perfmodel model = {.type = STARPU_PERFMODEL_INVALID};
        struct starpu_perfmodel energy_model = {.type = STARPU_PERFMODEL_INVALID};
        rc = starpu_perfmodel_load_symbol(symbol, &model);
        if (energy_symbol && !rc) rc = starpu_perfmodel_load_symbol(energy_symbol, &energy_model);
        if (rc) {
            fprintf(stderr, "The performance model for the symbol <%s> could not be loaded\n",
                    energy_symbol ? energy_symbol : symbol);
        } else if (list_combs) {
            rc = starpu_perfmodel_list_combs(stdout, &model);
        } else {
            const char *kind = energy_symbol ? "power_" : gflops ? "gflops_" : "";
            char gp[4096], avg[4096];
            snprintf(gp, sizeof gp, "%s/starpu_%s%s.gp", dir, kind, symbol);
            snprintf(avg, sizeof avg, "%s/starpu_%s%s_avg.data", dir, kind, symbol);
            rc = starpu_gb300_perfmodel_plot(&model, energy_symbol ? &energy_model : NULL, symbol, energy_symbol, comb,
                                             gflops, energy, gp, avg);
            if (rc) {
                fprintf(stderr, "Cannot create <%s>\n", gp);
            } else {
                struct stat sb;
                if (stat(gp, &sb) == 0) chmod(gp, sb.st_mode | S_IXUSR | S_IXGRP | S_IXOTH);
                fprintf(stderr, "Gnuplot file <%s> generated\n", gp);
            }
        }
        starpu_perfmodel_unload_model(&model);
        if (energy_symbol) starpu_perfmodel_unload_model(&energy_model);
    }
    starpu_perfmodel_free_sampling();
    return rc ? 1 : 0;
}
