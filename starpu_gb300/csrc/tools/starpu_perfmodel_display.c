/*
 * starpu_perfmodel_display: show the history-based performance models this
 * runtime (or StarPU) wrote, with the options of StarPU's
 * tools/starpu_perfmodel_display.c:
 *   -l            list the model files of every model directory
 *   -d            print the model directories
 *   -s <symbol>   print the model of a symbol (symbol.hostname, or the file
 *                 named by a symbol holding a dot)
 *   -x            ... as XML
 *   -p <param>    ... only a, b, c, alpha, beta, mean or stddev
 *   -a <arch>     ... only cpu, cpu:<k>, cuda, cuda<d>
 *   -f <hash>     ... only the entry of that footprint
 * The directories come from STARPU_PERF_MODEL_DIR, STARPU_HOME / HOME and
 * STARPU_PERF_MODEL_PATH; the host name from STARPU_HOSTNAME.
 */
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>

#include <starpu.h>

#define PROGNAME "starpu_perfmodel_display"

static void usage(void)
{
    fprintf(stderr,
            "Display a given perfmodel\n\n"
            "Usage: %s [ options ]\n\n"
            "One must specify either -l or -s. -x can be used with -s\n"
            "Options:\n"
            "   -l\t\t\tdisplay all available models\n"
            "   -s <symbol>\t\tspecify the symbol\n"
            "   -x\t\t\tdisplay output in XML format\n"
            "   -p <parameter>\tspecify the parameter (e.g. a, b, c, mean, stddev)\n"
            "   -a <arch>\t\tspecify the architecture (e.g. cpu, cpu:k, cuda)\n"
            "   -f <footprint>\tdisplay the history-based model for the specified footprint\n"
            "   -d\t\t\tdisplay the directory storing performance models\n"
            "   -h, --help\t\tdisplay this help and exit\n"
            "   -v, --version\toutput version information and exit\n",
            PROGNAME);
}

int main(int argc, char **argv)
{
    int xml = 0, list = 0, directory = 0, with_footprint = 0;
    char *symbol = NULL, *parameter = NULL, *arch = NULL;
    uint32_t footprint = 0;
    static struct option longopts[] = {{"arch", required_argument, NULL, 'a'},
                                       {"footprint", required_argument, NULL, 'f'},
                                       {"help", no_argument, NULL, 'h'},
                                       {"list", no_argument, NULL, 'l'},
                                       {"dir", no_argument, NULL, 'd'},
                                       {"parameter", required_argument, NULL, 'p'},
                                       {"symbol", required_argument, NULL, 's'},
                                       {"version", no_argument, NULL, 'v'},
                                       {0, 0, 0, 0}};
    int c;
    while ((c = getopt_long(argc, argv, "dls:p:a:f:hxv", longopts, NULL)) != -1) {
        switch (c) {
        case 'l': list = 1; break;
        case 's': symbol = optarg; break;
        case 'p': parameter = optarg; break;
        case 'a': arch = optarg; break;
        case 'f':
            if (sscanf(optarg, "%x", &footprint) != 1) {
                fprintf(stderr, "Invalid footprint <%s>\n", optarg);
                return 1;
            }
            with_footprint = 1;
            break;
        case 'd': directory = 1; break;
        case 'x': xml = 1; break;
        case 'h': usage(); return 0;
        case 'v': fputs(PROGNAME " (starpu_gb300)\n", stderr); return 0;
        default: fprintf(stderr, "Unrecognized option: -%c\n", optopt);
        }
    }
    if (!symbol && !list && !directory) {
        fprintf(stderr, "Incorrect usage, aborting\n");
        usage();
        return 255;
    }
    starpu_drivers_preinit();
    starpu_perfmodel_initialize();
    int rc = 0;
    if (list) {
        starpu_perfmodel_list(stdout);
    } else if (directory) {
        starpu_perfmodel_directory(stdout);
    } else {
        struct starpu_perfmodel model = {.type = STARPU_PERFMODEL_INVALID};
        if (starpu_perfmodel_load_symbol(symbol, &model) != 0) {
            fprintf(stderr, "The performance model for the symbol <%s> could not be loaded\n", symbol);
            return 1;
        }
        if (xml) starpu_perfmodel_dump_xml(stdout, &model);
        else rc = starpu_perfmodel_print_all(&model, arch, parameter, with_footprint ? &footprint : NULL, stdout) ? 1 : 0;
        starpu_perfmodel_unload_model(&model);
    }
    starpu_perfmodel_free_sampling();
    return rc;
}
