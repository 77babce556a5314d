/*
 * History-based performance models, their version-45 files, and the
 * perfmodel tooling API (the calls tools/starpu_perfmodel_display.c and
 * tools/starpu_perfmodel_plot.c make).
 *
 * Models (src/core/perfmodel/perfmodel_history.c): per symbol, per
 * architecture combination (a set of devices: type, device id, cores) and per
 * implementation, a list of entries keyed by the footprint of the task's data
 * shapes, each with the running sum / sum of squares / count of measured
 * execution times in microseconds, their mean and standard deviation, the
 * data size and the task's flops.  Combinations are numbered process-wide in
 * the order they are first seen (perfmodel_history.c:187-230); a file
 * records, per combination, its devices and then its implementations.
 *
 * Files: <dir>/codelets/45/<symbol>.<hostname> (or <dir>/codelets/45/<symbol>
 * when the symbol already holds a dot), searched in
 * $STARPU_PERF_MODEL_DIR, $STARPU_HOME/.starpu/sampling (else
 * $HOME/.starpu/sampling), then each existing directory of
 * $STARPU_PERF_MODEL_PATH (src/core/perfmodel/perfmodel.c:663-683, 783-812);
 * written to the first of them.  The layout is the one
 * perfmodel_history.c:378-440, 571-574, 834-876, 912-968 write and 491-558,
 * 577-628, 629-812 read: '#' lines are comments, then the version, the number
 * of combinations, and per combination the device count, per device its type,
 * id and cores, the number of implementations, and per implementation the
 * entry count, the linear regression sums (alpha, beta as nan unless
 * computed), the non-linear a b c, the multiple-regression coefficient count
 * (and coefficients), then the entries
 *   footprint size flops mean deviation sum sum2 nsample
 * (older files omit flops).  Entries read from a file are put at the head of
 * their list, as perfmodel_history.c:655-657 does, so a load + save writes
 * them in reverse order.
 *
 * Recording (perfmodel_history.c:1900-1990): a measurement more than
 * STARPU_HISTORY_MAX_ERROR percent (default 50) away from the current mean
 * counts as an error and is dropped; when errors reach the sample count the
 * entry is reset.  A history model predicts once an entry holds
 * STARPU_CALIBRATE_MINIMUM (default 10) samples.  Regression-based models
 * (linear and non-linear) keep the same entries and, per call, the log-log
 * least-squares sums of time = alpha size^beta (perfmodel_history.c:1993-2023);
 * a non-linear model fits time = a size^b + c over its entries when it is
 * saved (regression.c) and predicts from the fit its file holds.
 *
 * Prediction (perfmodel.c:199-258): per-arch and per-worker models call the
 * codelet's cost function, a common model divides its cost by the
 * architecture's relative speed (CPU core 0.5, CUDA device 13.33), history
 * models take the entry's mean, regression models evaluate their fit inside
 * [0.9 minx, 1.1 maxx] of the sizes measured (a non-linear model falls back
 * to the entry's mean outside it).  Multiple-regression models (an offline
 * fit over codelet parameters) read, print and save their coefficients but
 * predict nothing here.
 *
 * Malformed files are reported and the load fails with 1, where the
 * reference asserts.
 */
#include <dirent.h>
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include "rt_internal.h"

#define PM_VERSION 45
#define PM_MAXIMPL STARPU_MAXIMPLEMENTATIONS
#define PM_MAXDIRS 20
#define PM_DIRLEN 1024

struct pm_entry {
    uint32_t footprint;
    size_t size;
    double flops, mean, deviation, sum, sum2;
    unsigned nsample, nerror;
    struct pm_entry *next;
};

struct pm_regression {
    double sumlnx, sumlnx2, sumlny, sumlnxlny, alpha, beta;
    unsigned nsample;
    unsigned long minx, maxx;
    double a, b, c;
    unsigned ncoeff;
    double *coeff;
    int valid, nl_valid;
};

struct pm_per_arch {
    struct pm_entry *list;
    struct pm_regression reg;
};

struct starpu_perfmodel_history_state {
    int ncombs;                    /* combinations this model holds, in file / first-use order */
    int *combs;                    /* their process-wide ids */
    int capcombs;
    int nslots;                    /* per_arch and nimpls are indexed by process-wide id */
    int *nimpls;
    struct pm_per_arch **per_arch; /* [comb][impl], PM_MAXIMPL per comb */
    int dirty;
};

/* ------------------------------------------------------ arch combinations */

static pthread_mutex_t comb_mu = PTHREAD_MUTEX_INITIALIZER;
static struct starpu_perfmodel_arch **arch_combs;
static int narch_combs, cap_arch_combs;
static char ignore_devid[STARPU_NARCH];
static int calibrate_minimum = 10;
static int history_max_error = 50;

static int comb_get_locked(int ndevices, const struct starpu_perfmodel_device *devices)
{
    for (int c = 0; c < narch_combs; ++c) {
        const struct starpu_perfmodel_arch *a = arch_combs[c];
        if (a->ndevices != ndevices) continue;
        int matched = 0;
        for (int d1 = 0; d1 < a->ndevices; ++d1)
            for (int d2 = 0; d2 < ndevices; ++d2) {
                const struct starpu_perfmodel_device *x = &a->devices[d1], *y = &devices[d2];
                int type = (int)y->type;
                int same_id = (type >= 0 && type < STARPU_NARCH && ignore_devid[type]) || x->devid == y->devid;
                if (x->type == y->type && same_id && x->ncores == y->ncores) ++matched;
            }
        if (matched == ndevices) return c;
    }
    return -1;
}

int starpu_perfmodel_arch_comb_get(int ndevices, struct starpu_perfmodel_device *devices)
{
    pthread_mutex_lock(&comb_mu);
    int c = comb_get_locked(ndevices, devices);
    pthread_mutex_unlock(&comb_mu);
    return c;
}

int starpu_perfmodel_arch_comb_add(int ndevices, struct starpu_perfmodel_device *devices)
{
    pthread_mutex_lock(&comb_mu);
    int c = comb_get_locked(ndevices, devices);
    if (c < 0) {
        if (narch_combs == cap_arch_combs) {
            cap_arch_combs = cap_arch_combs ? 2 * cap_arch_combs : 8;
            arch_combs = realloc(arch_combs, (size_t)cap_arch_combs * sizeof *arch_combs);
        }
        struct starpu_perfmodel_arch *a = malloc(sizeof *a);
        a->ndevices = ndevices;
        a->devices = malloc((size_t)(ndevices > 0 ? ndevices : 1) * sizeof *a->devices);
        memcpy(a->devices, devices, (size_t)ndevices * sizeof *devices);
        c = narch_combs++;
        arch_combs[c] = a;
    }
    pthread_mutex_unlock(&comb_mu);
    return c;
}

struct starpu_perfmodel_arch *starpu_perfmodel_arch_comb_fetch(int comb)
{
    pthread_mutex_lock(&comb_mu);
    struct starpu_perfmodel_arch *a = comb >= 0 && comb < narch_combs ? arch_combs[comb] : NULL;
    pthread_mutex_unlock(&comb_mu);
    return a;
}

int starpu_perfmodel_get_narch_combs(void)
{
    pthread_mutex_lock(&comb_mu);
    int n = narch_combs;
    pthread_mutex_unlock(&comb_mu);
    return n;
}

static int comb_of(struct starpu_perfmodel_arch *arch)
{
    return starpu_perfmodel_arch_comb_add(arch->ndevices, arch->devices);
}

const char *starpu_perfmodel_get_archtype_name(enum starpu_worker_archtype archtype)
{
    switch (archtype) {
    case STARPU_CPU_WORKER: return "cpu";
    case STARPU_CUDA_WORKER: return "cuda";
    case STARPU_OPENCL_WORKER: return "opencl";
    case STARPU_MAX_FPGA_WORKER: return "max_fpga";
    case STARPU_MPI_SC_WORKER: return "mpi_ms";
    case STARPU_TCPIP_SC_WORKER: return "tcpip_ms";
    case STARPU_HIP_WORKER: return "hip";
    case STARPU_SYCL_WORKER: return "sycl";
    default: return "unknown";
    }
}

static const char *archtype_upper(enum starpu_worker_archtype archtype)
{
    switch (archtype) {
    case STARPU_CPU_WORKER: return "CPU";
    case STARPU_CUDA_WORKER: return "CUDA";
    case STARPU_OPENCL_WORKER: return "OpenCL";
    case STARPU_MAX_FPGA_WORKER: return "MAX_FPGA";
    case STARPU_MPI_SC_WORKER: return "MPI_MS";
    case STARPU_TCPIP_SC_WORKER: return "TCPIP_MS";
    case STARPU_HIP_WORKER: return "HIP";
    case STARPU_SYCL_WORKER: return "SYCL";
    default: return "unknown";
    }
}

/* "<type><devid>_cores<ncores>[_...]_impl<impl> (Comb<id>)", perfmodel_history.c:1546-1560 */
void starpu_perfmodel_get_arch_name(struct starpu_perfmodel_arch *arch, char *archname, size_t maxlen, unsigned impl)
{
    int comb = comb_of(arch);
    char devices[512];
    size_t w = 0;
    devices[0] = 0;
    for (int i = 0; i < arch->ndevices && w < sizeof devices; ++i)
        w += (size_t)snprintf(devices + w, sizeof devices - w, "%s%d_cores%d%s",
                              starpu_perfmodel_get_archtype_name(arch->devices[i].type), arch->devices[i].devid,
                              arch->devices[i].ncores, i != arch->ndevices - 1 ? "_" : "");
    snprintf(archname, maxlen, "%s_impl%u (Comb%d)", devices, impl, comb);
}

/* ----------------------------------------------------------- directories */

static pthread_mutex_t dir_mu = PTHREAD_MUTEX_INITIALIZER;
static char *model_dirs[PM_MAXDIRS + 1];
static int nmodel_dirs;
static int model_dir_from_env;
static char dirs_signature[4 * PM_DIRLEN];

static void add_dir(const char *dir, int only_if_exists)
{
    if (!dir || !*dir || nmodel_dirs >= PM_MAXDIRS) return;
    if (only_if_exists) {
        DIR *d = opendir(dir);
        if (!d) {
            fprintf(stderr, "[starpu_gb300] perfmodel directory <%s> does not exist\n", dir);
            return;
        }
        closedir(d);
    }
    char *p = malloc(PM_DIRLEN);
    snprintf(p, PM_DIRLEN, "%s/", dir);
    model_dirs[nmodel_dirs++] = p;
    model_dirs[nmodel_dirs] = NULL;
}

/* The list is rebuilt whenever the variables it comes from change, so that a
 * process may point successive calls at other model directories. */

/* called with dir_mu held */
static void set_dirs_locked(void)
{
    char sig[sizeof dirs_signature];
    const char *v[4] = {getenv("STARPU_PERF_MODEL_DIR"), getenv("STARPU_HOME"), getenv("HOME"),
                        getenv("STARPU_PERF_MODEL_PATH")};
    snprintf(sig, sizeof sig, "%s\n%s\n%s\n%s", v[0] ? v[0] : "", v[1] ? v[1] : "", v[2] ? v[2] : "",
             v[3] ? v[3] : "");
    if (nmodel_dirs != 0 && strcmp(sig, dirs_signature) != 0) {
        for (int i = 0; i < nmodel_dirs; ++i) {
            free(model_dirs[i]);
            model_dirs[i] = NULL;
        }
        nmodel_dirs = 0;
    }
    if (nmodel_dirs == 0) {
        snprintf(dirs_signature, sizeof dirs_signature, "%s", sig);
        const char *env = getenv("STARPU_PERF_MODEL_DIR");
        model_dir_from_env = env && *env;
        if (model_dir_from_env) add_dir(env, 0);
        const char *home = getenv("STARPU_HOME");
        if (!home || !*home) home = getenv("HOME");
        if (!home || !*home) home = "/tmp";
        char buf[PM_DIRLEN];
        snprintf(buf, sizeof buf, "%s/.starpu/sampling", home);
        add_dir(buf, 0);
        const char *path = getenv("STARPU_PERF_MODEL_PATH");
        if (path && *path) {
            char *copy = strdup(path), *save = NULL;
            for (char *tok = strtok_r(copy, ":", &save); tok; tok = strtok_r(NULL, ":", &save)) add_dir(tok, 1);
            free(copy);
        }
    }
}

/* STARPU_HOSTNAME, else the host name up to its first dot (src/common/utils.c:539-590) */
static void host_name(char *host, size_t len)
{
    const char *h = getenv("STARPU_HOSTNAME");
    if (h && *h) {
        snprintf(host, len, "%s", h);
        return;
    }
    if (gethostname(host, len - 1) != 0) snprintf(host, len, "unknown");
    host[len - 1] = 0;
    char *dot = strchr(host, '.');
    if (dot) *dot = 0;
}

static void codelet_file(const char *dir, const char *symbol, char *path, size_t maxlen)
{
    char host[256];
    host_name(host, sizeof host);
    const int dotted = strrchr(symbol, '.') != NULL;
    snprintf(path, maxlen, "%scodelets/%d/%s%s%s", dir, PM_VERSION, symbol, dotted ? "" : ".", dotted ? "" : host);
}

static void mkdir_p(const char *path)
{
    char tmp[PM_DIRLEN + 256];
    snprintf(tmp, sizeof tmp, "%s", path);
    for (char *p = tmp + 1; *p; ++p)
        if (*p == '/') {
            *p = 0;
            mkdir(tmp, 0755);
            *p = '/';
        }
}

/* the first existing file among the directories, "" when none */
void starpu_perfmodel_get_model_path(const char *symbol, char *path, size_t maxlen)
{
    pthread_mutex_lock(&dir_mu);
    set_dirs_locked();
    for (int i = 0; i < nmodel_dirs; ++i) {
        codelet_file(model_dirs[i], symbol, path, maxlen);
        if (access(path, F_OK) == 0) {
            pthread_mutex_unlock(&dir_mu);
            return;
        }
    }
    pthread_mutex_unlock(&dir_mu);
    if (maxlen) path[0] = 0;
}

/* where a model is written: the first directory (its codelets/45/ is created) */
void starpu_perfmodel_get_model_path_default_location(const char *symbol, char *path, size_t maxlen)
{
    pthread_mutex_lock(&dir_mu);
    set_dirs_locked();
    codelet_file(model_dirs[0], symbol, path, maxlen);
    pthread_mutex_unlock(&dir_mu);
    mkdir_p(path);
}

void starpu_perfmodel_directory(FILE *output)
{
    pthread_mutex_lock(&dir_mu);
    set_dirs_locked();
    for (int i = 0; i < nmodel_dirs; ++i) fprintf(output, "directory: <%scodelets/%d/>\n", model_dirs[i], PM_VERSION);
    pthread_mutex_unlock(&dir_mu);
}

static int name_cmp(const struct dirent **a, const struct dirent **b) { return strcmp((*a)->d_name, (*b)->d_name); }

int starpu_perfmodel_list(FILE *output)
{
    pthread_mutex_lock(&dir_mu);
    set_dirs_locked();
    char dirs[PM_MAXDIRS][PM_DIRLEN + 32];
    const int ndirs = nmodel_dirs;
    for (int i = 0; i < ndirs; ++i) snprintf(dirs[i], sizeof dirs[i], "%scodelets/%d/", model_dirs[i], PM_VERSION);
    pthread_mutex_unlock(&dir_mu);
    for (int i = 0; i < ndirs; ++i) {
        const char *dir = dirs[i];
        struct dirent **list;
        int n = scandir(dir, &list, NULL, name_cmp);
        if (n < 0) {
            fprintf(stderr, "[starpu_gb300] could not open the perfmodel directory <%s>: %s\n", dir, strerror(errno));
            continue;
        }
        fprintf(output, "codelet directory: <%s>\n", dir);
        for (int j = 0; j < n; ++j) {
            if (strcmp(list[j]->d_name, ".") && strcmp(list[j]->d_name, ".."))
                fprintf(output, "file: <%s>\n", list[j]->d_name);
            free(list[j]);
        }
        free(list);
    }
    return 0;
}

/* ---------------------------------------------------------- model state */

static pthread_mutex_t model_mu = PTHREAD_MUTEX_INITIALIZER;
#define MAX_MODELS 256
static struct starpu_perfmodel *models[MAX_MODELS];
static int nmodels;

/* a fresh per-arch regression: all zero, as perfmodel.c's calloc leaves it
 * (a file written before the fit is valid holds alpha = beta = 0) */
static void reg_init(struct pm_regression *r)
{
    memset(r, 0, sizeof *r);
}

static struct pm_per_arch *per_arch(struct starpu_perfmodel_history_state *s, int comb, int impl)
{
    if (comb >= s->nslots) {
        int n = comb + 8;
        s->nimpls = realloc(s->nimpls, (size_t)n * sizeof *s->nimpls);
        s->per_arch = realloc(s->per_arch, (size_t)n * sizeof *s->per_arch);
        for (int i = s->nslots; i < n; ++i) {
            s->nimpls[i] = 0;
            s->per_arch[i] = NULL;
        }
        s->nslots = n;
    }
    if (!s->per_arch[comb]) {
        s->per_arch[comb] = calloc(PM_MAXIMPL, sizeof **s->per_arch);
        for (int i = 0; i < PM_MAXIMPL; ++i) reg_init(&s->per_arch[comb][i].reg);
        int known = 0;
        for (int i = 0; i < s->ncombs; ++i) known |= s->combs[i] == comb;
        if (!known) {
            if (s->ncombs == s->capcombs) {
                s->capcombs = s->capcombs ? 2 * s->capcombs : 8;
                s->combs = realloc(s->combs, (size_t)s->capcombs * sizeof *s->combs);
            }
            s->combs[s->ncombs++] = comb;
        }
    }
    if (impl >= s->nimpls[comb]) s->nimpls[comb] = impl + 1;
    return &s->per_arch[comb][impl];
}

static struct pm_per_arch *per_arch_if_any(struct starpu_perfmodel_history_state *s, int comb, int impl)
{
    if (!s || comb < 0 || comb >= s->nslots || !s->per_arch[comb] || impl >= s->nimpls[comb]) return NULL;
    return &s->per_arch[comb][impl];
}

static void free_state(struct starpu_perfmodel_history_state *s)
{
    if (!s) return;
    for (int c = 0; c < s->nslots; ++c) {
        if (!s->per_arch[c]) continue;
        for (int i = 0; i < PM_MAXIMPL; ++i) {
            struct pm_entry *e = s->per_arch[c][i].list;
            while (e) {
                struct pm_entry *n = e->next;
                free(e);
                e = n;
            }
            free(s->per_arch[c][i].reg.coeff);
        }
        free(s->per_arch[c]);
    }
    free(s->per_arch);
    free(s->nimpls);
    free(s->combs);
    free(s);
}

/* ------------------------------------------------------------ file parser */

struct pm_reader {
    char **lines; /* non-comment, non-blank lines */
    int nlines, line;
    char *pos;    /* next unread character of lines[line] */
    const char *path;
    int bad;
};

static int reader_open(struct pm_reader *r, const char *path)
{
    memset(r, 0, sizeof *r);
    r->path = path;
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    size_t cap = 0, len = 0;
    char *buf = NULL;
    for (;;) {
        if (len + 4096 + 1 > cap) {
            cap = cap ? 2 * cap : 65536;
            buf = realloc(buf, cap);
        }
        size_t got = fread(buf + len, 1, cap - len - 1, f);
        len += got;
        if (got == 0) break;
    }
    fclose(f);
    buf[len] = 0;
    int caplines = 0;
    for (char *save = NULL, *l = strtok_r(buf, "\n", &save); l; l = strtok_r(NULL, "\n", &save)) {
        char *p = l;
        while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
        if (!*p || *p == '#') continue;
        if (r->nlines == caplines) {
            caplines = caplines ? 2 * caplines : 256;
            r->lines = realloc(r->lines, (size_t)caplines * sizeof *r->lines);
        }
        r->lines[r->nlines++] = strdup(p);
    }
    free(buf);
    r->pos = r->nlines ? r->lines[0] : NULL;
    return 0;
}

static void reader_close(struct pm_reader *r)
{
    for (int i = 0; i < r->nlines; ++i) free(r->lines[i]);
    free(r->lines);
}

/* next whitespace-separated token, continuing on the next lines */
static char *next_token(struct pm_reader *r)
{
    while (r->line < r->nlines) {
        while (*r->pos == ' ' || *r->pos == '\t' || *r->pos == '\r') ++r->pos;
        if (*r->pos) {
            char *t = r->pos;
            while (*r->pos && *r->pos != ' ' && *r->pos != '\t' && *r->pos != '\r') ++r->pos;
            if (*r->pos) *r->pos++ = 0;
            return t;
        }
        if (++r->line < r->nlines) r->pos = r->lines[r->line];
    }
    r->bad = 1;
    return NULL;
}

/* the rest of the current line is dropped; the next read starts a new line */
static void end_line(struct pm_reader *r)
{
    if (r->line < r->nlines && ++r->line < r->nlines) r->pos = r->lines[r->line];
}

static long read_long(struct pm_reader *r)
{
    char *t = next_token(r), *end;
    if (!t) return 0;
    long v = strtol(t, &end, 10);
    if (*end) r->bad = 1;
    return v;
}

static double read_double(struct pm_reader *r)
{
    char *t = next_token(r), *end;
    if (!t) return NAN;
    double v = strtod(t, &end);
    if (*end) r->bad = 1;
    return v;
}

static int valid_regression(const struct pm_regression *g)
{
    return g->minx < (9 * g->maxx) / 10 && g->nsample >= (unsigned)calibrate_minimum;
}

static void parse_regression(struct pm_reader *r, struct pm_regression *g)
{
    g->sumlnx = read_double(r);
    g->sumlnx2 = read_double(r);
    g->sumlny = read_double(r);
    g->sumlnxlny = read_double(r);
    g->alpha = read_double(r);
    g->beta = read_double(r);
    g->nsample = (unsigned)read_long(r);
    g->minx = (unsigned long)read_long(r);
    g->maxx = (unsigned long)read_long(r);
    g->valid = !isnan(g->alpha) && !isnan(g->beta) && valid_regression(g);
    end_line(r);
    g->a = read_double(r);
    g->b = read_double(r);
    g->c = read_double(r);
    g->nl_valid = !isnan(g->a) && !isnan(g->b) && !isnan(g->c) && valid_regression(g);
    end_line(r);
    g->ncoeff = (unsigned)read_long(r);
    free(g->coeff);
    g->coeff = NULL;
    if (g->ncoeff > 0 && g->ncoeff < 4096) {
        g->coeff = malloc(g->ncoeff * sizeof *g->coeff);
        for (unsigned i = 0; i < g->ncoeff; ++i) g->coeff[i] = read_double(r);
    } else if (g->ncoeff) {
        r->bad = 1;
    }
    end_line(r);
}

static void parse_entry(struct pm_reader *r, struct pm_per_arch *pa)
{
    if (r->line >= r->nlines) {
        r->bad = 1;
        return;
    }
    unsigned fp, n;
    unsigned long size;
    double flops, mean, dev, sum, sum2;
    const char *l = r->pos;
    if (sscanf(l, "%x %lu %le %le %le %le %le %u", &fp, &size, &flops, &mean, &dev, &sum, &sum2, &n) != 8) {
        flops = 0;
        if (sscanf(l, "%x %lu %le %le %le %le %u", &fp, &size, &mean, &dev, &sum, &sum2, &n) != 7) {
            r->bad = 1;
            return;
        }
    }
    end_line(r);
    if (!pa) return;
    struct pm_entry *e = calloc(1, sizeof *e);
    e->footprint = fp;
    e->size = size;
    e->flops = flops;
    e->mean = mean;
    e->deviation = dev;
    e->sum = sum;
    e->sum2 = sum2;
    e->nsample = n;
    e->next = pa->list;
    pa->list = e;
}

/* parse a whole file into m->state (created if needed); 0 on success.
 * Without keep_entries the entries are read and dropped, as a runtime load
 * of a linear- or multiple-regression model does (perfmodel.c:177-183). */
static int parse_file(const char *path, struct starpu_perfmodel *m, int keep_entries)
{
    struct pm_reader r;
    if (reader_open(&r, path) != 0) return 1;
    if (r.nlines == 0) {
        fprintf(stderr, "[starpu_gb300] performance model file %s is empty, ignoring it\n", path);
        reader_close(&r);
        return 1;
    }
    long version = read_long(&r);
    end_line(&r);
    if (version != PM_VERSION) {
        fprintf(stderr, "[starpu_gb300] performance model file %s has version %ld, not %d\n", path, version,
                PM_VERSION);
        reader_close(&r);
        return 1;
    }
    long ncombs = read_long(&r);
    end_line(&r);
    for (long c = 0; c < ncombs && !r.bad; ++c) {
        long ndev = read_long(&r);
        end_line(&r);
        if (ndev <= 0 || ndev > 64) {
            r.bad = 1;
            break;
        }
        struct starpu_perfmodel_device devs[64];
        for (long d = 0; d < ndev; ++d) {
            devs[d].type = (enum starpu_worker_archtype)read_long(&r);
            end_line(&r);
            devs[d].devid = (int)read_long(&r);
            end_line(&r);
            devs[d].ncores = (int)read_long(&r);
            end_line(&r);
        }
        int id = starpu_perfmodel_arch_comb_add((int)ndev, devs);
        long nimpls = read_long(&r);
        end_line(&r);
        for (long i = 0; i < nimpls && !r.bad; ++i) {
            struct pm_per_arch *pa = i < PM_MAXIMPL ? per_arch(m->state, id, (int)i) : NULL;
            struct pm_regression dummy;
            reg_init(&dummy);
            long nentries = read_long(&r);
            end_line(&r);
            parse_regression(&r, pa ? &pa->reg : &dummy);
            free(dummy.coeff);
            for (long e = 0; e < nentries && !r.bad; ++e) parse_entry(&r, keep_entries ? pa : NULL);
            if (pa && m->type == STARPU_PERFMODEL_INVALID) {
                if (pa->reg.ncoeff) m->type = STARPU_MULTIPLE_REGRESSION_BASED;
                else if (!isnan(pa->reg.a) && !isnan(pa->reg.b) && !isnan(pa->reg.c))
                    m->type = STARPU_NL_REGRESSION_BASED;
                else if (!isnan(pa->reg.alpha) && !isnan(pa->reg.beta)) m->type = STARPU_REGRESSION_BASED;
                else if (nentries) m->type = STARPU_HISTORY_BASED;
            }
        }
    }
    int bad = r.bad;
    reader_close(&r);
    if (bad) fprintf(stderr, "[starpu_gb300] incorrect performance model file %s\n", path);
    return bad ? 1 : 0;
}

/* ------------------------------------------------------ regression models */

/* One measurement into the log-log least-squares sums of time = alpha
 * size^beta, and the fit once valid_regression() holds
 * (perfmodel_history.c:1993-2023): one sample per call, whatever the batch
 * size, outliers of the history entry included. */
static void regression_add(struct pm_regression *g, size_t size, double us)
{
    const double lx = log((double)size), ly = log(us);
    g->sumlnx += lx;
    g->sumlnx2 += lx * lx;
    g->sumlny += ly;
    g->sumlnxlny += lx * ly;
    if (g->minx == 0 || size < g->minx) g->minx = size;
    if (g->maxx == 0 || size > g->maxx) g->maxx = size;
    g->nsample++;
    if (valid_regression(g)) {
        const unsigned n = g->nsample;
        g->beta = (n * g->sumlnxlny - g->sumlnx * g->sumlny) / (n * g->sumlnx2 - g->sumlnx * g->sumlnx);
        g->alpha = exp((g->sumlny - g->beta * g->sumlnx) / n);
        g->valid = 1;
    }
}

/* Weight of an entry (its sample count `pop`, mean `y`) in the fit of
 * log(y - c) against log(size) (regression.c:25-45): entries whose time
 * does not exceed 2c are left out and those above 3c count fully, through
 * the reference's piecewise ramp of the relative distance (y - c) / c. */
static double nl_weight(unsigned pop, double c, double y)
{
    const double t = (y - c) / c - 1.0;
    double w;
    if (t <= 0.) w = 0.;
    else if (t >= 1.) w = 1.;
    else if (t < 0.5) w = -2 * t * t + 4 * t - 1;
    else w = 2 * t * t;
    return pop * w;
}

/* Weighted moments of X = log(size), Y = log(y - c) over the entries. */
struct nl_moments {
    double sxy, sx, sx2, sy, sy2, n;
};

static struct nl_moments nl_moments(double c, unsigned n, const size_t *x, const double *y, const unsigned *pop)
{
    struct nl_moments m = {0, 0, 0, 0, 0, 0};
    for (unsigned i = 0; i < n; ++i) {
        const double w = nl_weight(pop[i], c, y[i]);
        if (w <= 0) continue;
        const double X = log((double)x[i]), Y = log(y[i] - c);
        m.sxy += X * Y * w;
        m.sx += X * w;
        m.sx2 += X * X * w;
        m.sy += Y * w;
        m.sy2 += Y * Y * w;
        m.n += w;
    }
    return m;
}

static int cmp_double(const void *pa, const void *pb)
{
    const double a = *(const double *)pa, b = *(const double *)pb;
    return a < b ? -1 : a > b;
}

/* Fit time = a size^b + c over the entries that hold samples, in list order
 * (regression.c:218-300, after Augonnet's thesis, appendix B): c is searched
 * in [0, the n/3-th smallest mean] by repeatedly dropping the outer third on
 * the side of the worse correlation coefficient of the weighted log-log fit,
 * until that coefficient's distance to 1 changes by less than 1e-10 (at most
 * 1000 steps); b and a then come from the weighted least squares at the
 * middle of the last interval.  -1 when no entry holds samples. */
static int nl_fit(const struct pm_entry *list, double *pa, double *pb, double *pc)
{
    unsigned n = 0;
    for (const struct pm_entry *e = list; e; e = e->next) n += e->nsample != 0;
    if (!n) return -1;
    size_t *x = malloc(n * sizeof *x);
    double *y = malloc(n * sizeof *y), *sorted = malloc(n * sizeof *sorted);
    unsigned *pop = malloc(n * sizeof *pop);
    unsigned i = 0;
    for (const struct pm_entry *e = list; e; e = e->next)
        if (e->nsample) {
            x[i] = e->size;
            y[i] = e->mean;
            pop[i] = e->nsample;
            ++i;
        }
    memcpy(sorted, y, n * sizeof *y);
    qsort(sorted, n, sizeof *sorted, cmp_double);
    double lo = 0.0, hi = sorted[n / 3], err = 100000.0;
    for (int it = 0; it < 1000; ++it) {
        const double c1 = lo + 0.33 * (hi - lo), c2 = lo + 0.67 * (hi - lo);
        double r[2];
        for (int k = 0; k < 2; ++k) {
            const struct nl_moments m = nl_moments(k ? c2 : c1, n, x, y, pop);
            r[k] = (m.n * m.sxy - m.sx * m.sy) / sqrt((m.n * m.sx2 - m.sx * m.sx) * (m.n * m.sy2 - m.sy * m.sy));
        }
        const double e1 = fabs(1.0 - r[0]), e2 = fabs(1.0 - r[1]);
        if (e1 < e2) hi = c2;
        else lo = c1;
        const double best = e1 < e2 ? e1 : e2;
        if (fabs(err - best) < 1.0e-10) break;
        err = best;
    }
    const double c = (lo + hi) / 2;
    const struct nl_moments m = nl_moments(c, n, x, y, pop);
    const double b = (m.n * m.sxy - m.sx * m.sy) / (m.n * m.sx2 - m.sx * m.sx);
    *pa = exp((m.sy - b * m.sx) / m.n);
    *pb = b;
    *pc = c;
    free(x);
    free(y);
    free(sorted);
    free(pop);
    return 0;
}

/* ------------------------------------------------------------ file writer */

static void write_double(FILE *f, const char *fmt, double v)
{
    if (isnan(v)) fprintf(f, strchr(fmt, '-') ? "%-15s" : "%s", "nan");
    else fprintf(f, fmt, v);
}

static void write_file(FILE *f, struct starpu_perfmodel *m)
{
    struct starpu_perfmodel_history_state *s = m->state;
    fprintf(f, "##################\n# Performance Model Version\n%d\n\n", PM_VERSION);
    fprintf(f, "####################\n# COMBs\n# number of combinations\n%d\n", s->ncombs);
    for (int i = 0; i < s->ncombs; ++i) {
        int comb = s->combs[i];
        struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
        fprintf(f, "####################\n# COMB_%d\n# number of types devices\n%d\n", comb, a->ndevices);
        for (int d = 0; d < a->ndevices; ++d) {
            fprintf(f, "####################\n# DEV_%d\n# device type (CPU - 0, CUDA - 1)\n%u\n", d,
                    (unsigned)a->devices[d].type);
            fprintf(f, "####################\n# DEV_%d\n# device id \n%u\n", d, (unsigned)a->devices[d].devid);
            fprintf(f, "####################\n# DEV_%d\n# number of cores \n%u\n", d, (unsigned)a->devices[d].ncores);
        }
        int nimpls = s->nimpls[comb];
        fprintf(f, "##########\n# number of implementations\n%d\n", nimpls);
        for (int impl = 0; impl < nimpls; ++impl) {
            struct pm_per_arch *pa = &s->per_arch[comb][impl];
            unsigned nentries = 0;
            for (struct pm_entry *e = pa->list; e; e = e->next) ++nentries;
            char name[600];
            starpu_perfmodel_get_arch_name(a, name, sizeof name, (unsigned)impl);
            fprintf(f, "#####\n# Model for %s\n# number of entries\n%u\n", name, nentries);
            const struct pm_regression *g = &pa->reg;
            const int lin = (m->type == STARPU_REGRESSION_BASED || m->type == STARPU_NL_REGRESSION_BASED) &&
                            g->nsample > 1;
            fprintf(f, "# sumlnx\tsumlnx2\t\tsumlny\t\tsumlnxlny\talpha\t\tbeta\t\tn\tminx\t\tmaxx\n");
            fprintf(f, "%-15e\t%-15e\t%-15e\t%-15e\t", g->sumlnx, g->sumlnx2, g->sumlny, g->sumlnxlny);
            write_double(f, "%-15e", lin ? g->alpha : NAN);
            fprintf(f, "\t");
            write_double(f, "%-15e", lin ? g->beta : NAN);
            fprintf(f, "\t%u\t%-15lu\t%-15lu\n", g->nsample, g->minx, g->maxx);
            /* a non-linear model's fit is made from its entries as it is
             * written (perfmodel_history.c:410-425) */
            double a = NAN, b = NAN, c = NAN;
            if (m->type == STARPU_NL_REGRESSION_BASED && nl_fit(pa->list, &a, &b, &c) != 0)
                fprintf(stderr, "[starpu_gb300] could not compute a non-linear regression for model %s\n",
                        m->symbol ? m->symbol : "?");
            fprintf(f, "# a\t\tb\t\tc\n");
            write_double(f, "%-15e", a);
            fprintf(f, "\t");
            write_double(f, "%-15e", b);
            fprintf(f, "\t");
            write_double(f, "%-15e", c);
            fprintf(f, "\n");
            if (g->ncoeff) {
                fprintf(f, "# n\tintercept\t\n%u", g->ncoeff);
                for (unsigned k = 0; k < g->ncoeff; ++k) {
                    fprintf(f, "\t");
                    write_double(f, "%-15e", g->coeff[k]);
                }
                fprintf(f, "\n");
            } else {
                fprintf(f, "# not multiple-regression-base\n0\n");
            }
            fprintf(f, "# hash\t\tsize\t\tflops\t\tmean (us or J)\tdev (us or J)\tsum\t\tsum2\t\tn\n");
            for (struct pm_entry *e = pa->list; e; e = e->next)
                fprintf(f, "%08x\t%-15lu\t%-15e\t%-15e\t%-15e\t%-15e\t%-15e\t%u\n", e->footprint,
                        (unsigned long)e->size, e->flops, e->mean, e->deviation, e->sum, e->sum2, e->nsample);
            fprintf(f, "\n");
        }
    }
}

static int save_model(struct starpu_perfmodel *m)
{
    if (!m->symbol || !m->state) return -EINVAL;
    char path[PM_DIRLEN + 512];
    starpu_perfmodel_get_model_path(m->symbol, path, sizeof path);
    if (path[0] == 0 || model_dir_from_env) starpu_perfmodel_get_model_path_default_location(m->symbol, path, sizeof path);
    char tmp[sizeof path + 32];
    snprintf(tmp, sizeof tmp, "%s.%d.tmp", path, (int)getpid());
    FILE *f = fopen(tmp, "w");
    if (!f) return -errno;
    write_file(f, m);
    if (fclose(f) != 0 || rename(tmp, path) != 0) {
        int err = errno;
        unlink(tmp);
        return -err;
    }
    m->state->dirty = 0;
    return 0;
}

/* --------------------------------------------------- runtime model access */

/* Double-checked initialisation: the fast path's acquire load pairs with the
 * release store below, so a thread that sees is_init also sees m->state. */
static void ensure_model(struct starpu_perfmodel *m)
{
    if (__atomic_load_n(&m->is_init, __ATOMIC_ACQUIRE)) return;
    pthread_mutex_lock(&model_mu);
    if (!m->is_init) {
        m->state = calloc(1, sizeof *m->state);
        if (m->symbol) {
            char path[PM_DIRLEN + 512];
            starpu_perfmodel_get_model_path(m->symbol, path, sizeof path);
            const int keep = m->type != STARPU_REGRESSION_BASED && m->type != STARPU_MULTIPLE_REGRESSION_BASED;
            if (path[0] && parse_file(path, m, keep) != 0) {
                /* a damaged file is ignored: the model calibrates again */
                free_state(m->state);
                m->state = calloc(1, sizeof *m->state);
            }
        }
        if (nmodels < MAX_MODELS) models[nmodels++] = m;
        m->is_loaded = 1;
        __atomic_store_n(&m->is_init, 1, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&model_mu);
}

static uint32_t task_footprint(struct starpu_task *t)
{
    if (t->cl && t->cl->model && t->cl->model->footprint) return t->cl->model->footprint(t);
    uint32_t x = 0;
    for (int i = 0; i < t->nbuffers; ++i) {
        if (!t->handles[i] || (t->modes[i] & STARPU_NOFOOTPRINT) || (t->modes[i] & STARPU_SCRATCH)) continue;
        uint32_t f = rt_data_footprint(t->handles[i]);
        x = (x * 0x9E3779B1u) ^ f;
    }
    return x;
}

static size_t task_size(struct starpu_task *t, unsigned nimpl)
{
    struct starpu_perfmodel *m = t->cl ? t->cl->model : NULL;
    if (m && m->size_base) return m->size_base(t, nimpl);
    size_t s = 0;
    for (int i = 0; i < t->nbuffers; ++i)
        if (t->handles[i]) s += rt_data_size(t->handles[i]);
    return s;
}

static struct pm_entry *find_entry(struct pm_per_arch *pa, uint32_t fp)
{
    for (struct pm_entry *e = pa ? pa->list : NULL; e; e = e->next)
        if (e->footprint == fp) return e;
    return NULL;
}

/* Relative speed of an architecture: the sum over its devices of the
 * driver's speed factor times the device's cores (perfmodel.c:133-144; the
 * factors of drivers/cpu/driver_cpu.c:84-88 and drivers/cuda/driver_cuda_init.c:26-30). */
double starpu_worker_get_relative_speedup(struct starpu_perfmodel_arch *perf_arch)
{
    double speedup = 0;
    for (int d = 0; d < perf_arch->ndevices; ++d) {
        const double coef = perf_arch->devices[d].type == STARPU_CUDA_WORKER ? 13.33f
                            : perf_arch->devices[d].type == STARPU_CPU_WORKER ? 0.5f
                                                                              : 1.0f;
        speedup += coef * perf_arch->devices[d].ncores;
    }
    return speedup;
}

/* The calibrated mean of the task's entry, NAN below STARPU_CALIBRATE_MINIMUM
 * samples; called with model_mu held. */
static double entry_mean(struct pm_per_arch *pa, struct starpu_task *t)
{
    struct pm_entry *e = find_entry(pa, task_footprint(t));
    return (e && e->nsample >= (unsigned)calibrate_minimum) ? e->mean : NAN;
}

/* Expected duration (us) of task t on architecture arch for one model type
 * (perfmodel.c:199-244, perfmodel_history.c:1575-1680, 1740-1826); NAN when
 * the model cannot tell yet. */
static double model_expected(struct starpu_perfmodel *m, struct starpu_task *t, struct starpu_perfmodel_arch *arch,
                             unsigned nimpl)
{
    switch (m->type) {
    case STARPU_PER_ARCH:
        STARPU_ASSERT_MSG(m->arch_cost_function, "STARPU_PER_ARCH needs arch_cost_function to be defined");
        return m->arch_cost_function(t, arch, nimpl);
    case STARPU_COMMON: {
        STARPU_ASSERT_MSG(m->cost_function, "STARPU_COMMON requires common cost_function to be defined");
        const double alpha = starpu_worker_get_relative_speedup(arch);
        STARPU_ASSERT(alpha != 0.);
        return m->cost_function(t, nimpl) / alpha;
    }
    case STARPU_HISTORY_BASED:
    case STARPU_REGRESSION_BASED:
    case STARPU_NL_REGRESSION_BASED:
        break;
    default:
        return NAN;
    }
    if (nimpl >= PM_MAXIMPL) return NAN;
    ensure_model(m);
    const int comb = comb_of(arch);
    const size_t size = task_size(t, nimpl);
    pthread_mutex_lock(&model_mu);
    struct pm_per_arch *pa = per_arch_if_any(m->state, comb, (int)nimpl);
    double v = NAN;
    if (pa) {
        const struct pm_regression *g = &pa->reg;
        const int in_range = size >= g->minx * 0.9 && size <= g->maxx * 1.1;
        if (m->type == STARPU_HISTORY_BASED) v = entry_mean(pa, t);
        else if (m->type == STARPU_REGRESSION_BASED) v = g->valid && in_range ? g->alpha * pow((double)size, g->beta) : NAN;
        else v = g->nl_valid && in_range ? g->a * pow((double)size, g->b) + g->c : entry_mean(pa, t);
    }
    pthread_mutex_unlock(&model_mu);
    return v;
}

double starpu_task_expected_length(struct starpu_task *task, struct starpu_perfmodel_arch *arch, unsigned nimpl)
{
    struct starpu_perfmodel *m = task->cl ? task->cl->model : NULL;
    if (!m || !arch || arch->ndevices < 1) return NAN;
    return model_expected(m, task, arch, nimpl);
}

/* A per-worker model calls the codelet's worker cost function; the others
 * predict for the worker's architecture (perfmodel.c:246-258). */
double starpu_task_worker_expected_length(struct starpu_task *task, unsigned workerid, unsigned sched_ctx_id,
                                          unsigned nimpl)
{
    struct starpu_perfmodel *m = task->cl ? task->cl->model : NULL;
    if (!m) return NAN;
    if (m->type == STARPU_PER_WORKER) {
        STARPU_ASSERT_MSG(m->worker_cost_function, "STARPU_PER_WORKER needs worker_cost_function to be defined");
        return m->worker_cost_function(task, workerid, nimpl);
    }
    struct starpu_perfmodel_arch *arch = starpu_worker_get_perf_archtype((int)workerid, sched_ctx_id);
    return arch ? model_expected(m, task, arch, nimpl) : NAN;
}

uint32_t starpu_task_footprint(struct starpu_perfmodel *model, struct starpu_task *task,
                               struct starpu_perfmodel_arch *arch, unsigned nimpl)
{
    (void)model;
    (void)arch;
    (void)nimpl;
    return task_footprint(task);
}

/* A further measurement of an existing entry (perfmodel_history.c:1941-1989);
 * called with model_mu held. */
static void update_entry(struct pm_entry *e, struct starpu_task *t, double us, unsigned number,
                         struct starpu_perfmodel *m)
{
    const double ratio = e->mean > 0 ? us / e->mean : 1.0;
    if (e->nsample && (100 * ratio > 100 + history_max_error || 100 / ratio > 100 + history_max_error)) {
        e->nerror += number;
        if (e->nerror >= e->nsample) {
            fprintf(stderr,
                    "[starpu_gb300] too big deviation for model %s: %f us vs average %f us, flushing the entry "
                    "(STARPU_HISTORY_MAX_ERROR=%d%%)\n",
                    m->symbol ? m->symbol : "?", us, e->mean, history_max_error);
            e->sum = e->sum2 = e->mean = e->deviation = 0;
            e->nsample = e->nerror = 0;
        }
    } else {
        e->sum += us * number;
        e->sum2 += us * us * number;
        e->nsample += number;
        const unsigned n = e->nsample;
        e->mean = e->sum / n;
        e->deviation = sqrt(fabs(e->sum2 - e->sum * e->sum / n) / n);
    }
    if (t->flops != 0. && !isnan(e->flops)) {
        if (e->flops == 0.) e->flops = t->flops;
        else if (fabs(e->flops - t->flops) / e->flops > 0.00001) e->flops = NAN;
    }
}

/* the model types that keep measurements (perfmodel_history.c:1898) */
static int records_history(const struct starpu_perfmodel *m)
{
    return m->type == STARPU_HISTORY_BASED || m->type == STARPU_REGRESSION_BASED ||
           m->type == STARPU_NL_REGRESSION_BASED;
}

static void record(struct starpu_perfmodel *m, struct starpu_task *t, struct starpu_perfmodel_arch *arch,
                   unsigned nimpl, double us, unsigned number)
{
    ensure_model(m);
    if (nimpl >= PM_MAXIMPL || !records_history(m)) return;
    const int comb = comb_of(arch);
    const uint32_t fp = task_footprint(t);
    const size_t size = task_size(t, nimpl);
    pthread_mutex_lock(&model_mu);
    struct pm_per_arch *pa = per_arch(m->state, comb, (int)nimpl);
    struct pm_entry *e = find_entry(pa, fp);
    if (!e) {
        /* a new footprint (perfmodel_history.c:1915-1940): a history-based
         * model does not keep a single first measurement, which is very often
         * bogus (cold caches, lazy initialisation), and starts counting from
         * the second; other models, and batches of several, keep it */
        e = calloc(1, sizeof *e);
        e->footprint = fp;
        e->size = size;
        e->flops = t->flops;
        if (number != 1 || m->type != STARPU_HISTORY_BASED) {
            e->sum = us * number;
            e->sum2 = us * us * number;
            e->nsample = number;
            e->mean = us;
        }
        e->next = pa->list;
        pa->list = e;
    } else {
        update_entry(e, t, us, number, m);
    }
    if (m->type == STARPU_REGRESSION_BASED || m->type == STARPU_NL_REGRESSION_BASED) regression_add(&pa->reg, size, us);
    m->state->dirty = 1;
    pthread_mutex_unlock(&model_mu);
}

void rt_perfmodel_feedback(struct starpu_task *t, struct starpu_perfmodel_arch *arch, double us)
{
    struct starpu_perfmodel *m = t->cl->model;
    if (!m || !records_history(m) || !arch) return;
    record(m, t, arch, 0, us, 1);
}

void starpu_perfmodel_update_history(struct starpu_perfmodel *model, struct starpu_task *task,
                                     struct starpu_perfmodel_arch *arch, unsigned cpuid, unsigned nimpl,
                                     double measured)
{
    (void)cpuid;
    if (!model || !arch || arch->ndevices < 1) return;
    record(model, task, arch, nimpl, measured, 1);
}

/* `number` measurements averaging `average_measured` at once */
void starpu_perfmodel_update_history_n(struct starpu_perfmodel *model, struct starpu_task *task,
                                       struct starpu_perfmodel_arch *arch, unsigned cpuid, unsigned nimpl,
                                       double average_measured, unsigned number)
{
    (void)cpuid;
    if (!model || !arch || arch->ndevices < 1 || number == 0) return;
    record(model, task, arch, nimpl, average_measured, number);
}

/* the calibrated mean for a footprint on an architecture (implementation 0), NAN otherwise */
double starpu_perfmodel_history_based_expected_perf(struct starpu_perfmodel *model, struct starpu_perfmodel_arch *arch,
                                                    uint32_t footprint)
{
    ensure_model(model);
    const int comb = comb_of(arch);
    pthread_mutex_lock(&model_mu);
    struct pm_entry *e = find_entry(per_arch_if_any(model->state, comb, 0), footprint);
    double v = (e && e->nsample >= (unsigned)calibrate_minimum) ? e->mean : NAN;
    pthread_mutex_unlock(&model_mu);
    return v;
}

int starpu_save_history_based_model(struct starpu_perfmodel *model)
{
    ensure_model(model);
    pthread_mutex_lock(&model_mu);
    int rc = save_model(model);
    pthread_mutex_unlock(&model_mu);
    return rc;
}

/* starpu_init: worker architecture defaults (perfmodel_history.c:92-130) */
void rt_perfmodel_init(void)
{
    const char *v = getenv("STARPU_CALIBRATE_MINIMUM");
    calibrate_minimum = v && *v ? atoi(v) : 10;
    v = getenv("STARPU_HISTORY_MAX_ERROR");
    history_max_error = v && *v ? atoi(v) : 50;
    pthread_mutex_lock(&comb_mu);
    for (int a = 0; a < STARPU_NARCH; ++a) {
        char name[64];
        snprintf(name, sizeof name, "STARPU_PERF_MODEL_HOMOGENEOUS_%s", archtype_upper((enum starpu_worker_archtype)a));
        const char *e = getenv(name);
        ignore_devid[a] = e && *e ? (char)(atoi(e) != 0) : (char)(a == STARPU_CPU_WORKER);
    }
    pthread_mutex_unlock(&comb_mu);
}

void rt_perfmodel_save_all(void)
{
    pthread_mutex_lock(&model_mu);
    for (int i = 0; i < nmodels; ++i)
        if (models[i]->state && models[i]->state->dirty) save_model(models[i]);
    pthread_mutex_unlock(&model_mu);
}

/* ------------------------------------------------------- tooling: loading */

void starpu_perfmodel_initialize(void)
{
    pthread_mutex_lock(&dir_mu);
    set_dirs_locked();
    pthread_mutex_unlock(&dir_mu);
}

void starpu_perfmodel_init(struct starpu_perfmodel *model) { ensure_model(model); }

int starpu_perfmodel_deinit(struct starpu_perfmodel *model) { return starpu_perfmodel_unload_model(model); }

/* 0 on success, 1 when the file is empty or malformed (perfmodel_history.c:1475-1499) */
int starpu_perfmodel_load_file(const char *filename, struct starpu_perfmodel *model)
{
    if (!model->state) model->state = calloc(1, sizeof *model->state);
    int rc = parse_file(filename, model, 1);
    if (rc) {
        starpu_perfmodel_unload_model(model);
        return 1;
    }
    model->is_loaded = 1;
    model->is_init = 1;
    return 0;
}

/* 0 on success, 1 when no file exists for the symbol (perfmodel_history.c:1442-1473) */
int starpu_perfmodel_load_symbol(const char *symbol, struct starpu_perfmodel *model)
{
    memset(model, 0, sizeof *model);
    model->symbol = strdup(symbol);
    char path[PM_DIRLEN + 512];
    starpu_perfmodel_get_model_path(symbol, path, sizeof path);
    if (path[0]) return starpu_perfmodel_load_file(path, model);
    const char *dot = strrchr(symbol, '.');
    if (dot) {
        char *base = strdup(symbol);
        base[dot - symbol] = 0;
        fprintf(stderr, "[starpu_gb300] note: loading history from %s instead of %s\n", base, symbol);
        int rc = starpu_perfmodel_load_symbol(base, model);
        free(base);
        return rc;
    }
    fprintf(stderr, "[starpu_gb300] there is no performance model for symbol %s\n", symbol);
    return 1;
}

int starpu_perfmodel_unload_model(struct starpu_perfmodel *model)
{
    pthread_mutex_lock(&model_mu);
    for (int i = 0; i < nmodels; ++i)
        if (models[i] == model) {
            models[i] = models[--nmodels];
            break;
        }
    pthread_mutex_unlock(&model_mu);
    free_state(model->state);
    model->state = NULL;
    model->is_init = 0;
    model->is_loaded = 0;
    return 0;
}

/* the search directories and the process-wide combination table are dropped */
void starpu_perfmodel_free_sampling(void)
{
    pthread_mutex_lock(&dir_mu);
    for (int i = 0; i < nmodel_dirs; ++i) {
        free(model_dirs[i]);
        model_dirs[i] = NULL;
    }
    nmodel_dirs = 0;
    pthread_mutex_unlock(&dir_mu);
    pthread_mutex_lock(&comb_mu);
    for (int c = 0; c < narch_combs; ++c) {
        free(arch_combs[c]->devices);
        free(arch_combs[c]);
    }
    free(arch_combs);
    arch_combs = NULL;
    narch_combs = cap_arch_combs = 0;
    pthread_mutex_unlock(&comb_mu);
}

/* ------------------------------------------------------ tooling: printing */

static void print_history(struct pm_per_arch *pa, const char *parameter, uint32_t *footprint, FILE *out)
{
    if (!parameter && pa->list) fprintf(out, "# hash\t\tsize\t\tflops\t\tmean (us or J)\tstddev (us or J)\t\tn\n");
    for (struct pm_entry *e = pa->list; e; e = e->next) {
        if (footprint && e->footprint != *footprint) continue;
        if (!parameter) {
            fprintf(out, "%08x\t%-15lu\t%-15e\t%-15e\t%-15e\t%u\n", e->footprint, (unsigned long)e->size, e->flops,
                    e->mean, e->deviation, e->nsample);
        } else if (!strcmp(parameter, "mean")) {
            fprintf(out, "%-15e\n", e->mean);
        } else if (!strcmp(parameter, "stddev")) {
            fprintf(out, "%-15e\n", e->deviation);
            return;
        }
    }
}

/* perfmodel_print.c:59-163 */
static int print_one(struct starpu_perfmodel *model, struct starpu_perfmodel_arch *arch, unsigned nimpl,
                           char *parameter, uint32_t *footprint, FILE *output)
{
    const int comb = starpu_perfmodel_arch_comb_get(arch->ndevices, arch->devices);
    struct pm_per_arch *pa = per_arch_if_any(model->state, comb, (int)nimpl);
    if (!pa) return -1;
    const struct pm_regression *g = &pa->reg;
    if (g->nsample || g->valid || g->nl_valid || pa->list) {
        char name[600];
        starpu_perfmodel_get_arch_name(arch, name, sizeof name, nimpl);
        fprintf(output, "# performance model for %s\n", name);
    }
    if (!parameter) {
        if (g->nsample) fprintf(output, "\tRegression : #sample = %u\n", g->nsample);
        if (g->valid) {
            fprintf(output, "\tLinear: y = alpha size ^ beta\n");
            fprintf(output, "\t\talpha = %e\n", g->alpha);
            fprintf(output, "\t\tbeta = %e\n", g->beta);
        }
        if (g->nl_valid) {
            fprintf(output, "\tNon-Linear: y = a size ^b + c\n");
            fprintf(output, "\t\ta = %e\n", g->a);
            fprintf(output, "\t\tb = %e\n", g->b);
            fprintf(output, "\t\tc = %e\n", g->c);
        }
        print_history(pa, NULL, footprint, output);
        return 0;
    }
    if (!strcmp(parameter, "a")) fprintf(output, "%e\n", g->a);
    else if (!strcmp(parameter, "b")) fprintf(output, "%e\n", g->b);
    else if (!strcmp(parameter, "c")) fprintf(output, "%e\n", g->c);
    else if (!strcmp(parameter, "alpha")) fprintf(output, "%e\n", g->alpha);
    else if (!strcmp(parameter, "beta")) fprintf(output, "%e\n", g->beta);
    else if (!strcmp(parameter, "mean") || !strcmp(parameter, "stddev")) print_history(pa, parameter, footprint, output);
    else {
        fprintf(stderr, "[starpu_gb300] unknown parameter requested: %s\n", parameter);
        return -1;
    }
    return 0;
}

void starpu_perfmodel_print(struct starpu_perfmodel *model, struct starpu_perfmodel_arch *arch, unsigned nimpl,
                            char *parameter, uint32_t *footprint, FILE *output)
{
    pthread_mutex_lock(&model_mu);
    print_one(model, arch, nimpl, parameter, footprint, output);
    pthread_mutex_unlock(&model_mu);
}

static void print_single(struct starpu_perfmodel *model, enum starpu_worker_archtype type, int devid, int ncores,
                         char *parameter, uint32_t *footprint, FILE *output)
{
    struct starpu_perfmodel_device dev = {type, devid, ncores};
    struct starpu_perfmodel_arch arch = {1, &dev};
    const int comb = starpu_perfmodel_arch_comb_get(1, &dev);
    const int nimpls = model->state && comb >= 0 && comb < model->state->nslots ? model->state->nimpls[comb] : 0;
    for (int impl = 0; impl < nimpls; ++impl) print_one(model, &arch, (unsigned)impl, parameter, footprint, output);
}

/* arch: NULL (every combination), "cpu", "cpu:<k>", "cuda", "cuda<d>" / "cuda_<d>" (perfmodel_print.c:166-285) */
static int print_all_locked(struct starpu_perfmodel *model, char *arch, char *parameter, uint32_t *footprint,
                            FILE *output);

/* the model's lists are read under the model lock: workers may be recording */
int starpu_perfmodel_print_all(struct starpu_perfmodel *model, char *arch, char *parameter, uint32_t *footprint,
                               FILE *output)
{
    ensure_model(model);
    pthread_mutex_lock(&model_mu);
    const int rc = print_all_locked(model, arch, parameter, footprint, output);
    pthread_mutex_unlock(&model_mu);
    return rc;
}

static int print_all_locked(struct starpu_perfmodel *model, char *arch, char *parameter, uint32_t *footprint,
                            FILE *output)
{
    if (!arch) {
        const int n = starpu_perfmodel_get_narch_combs();
        for (int comb = 0; comb < n; ++comb) {
            struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
            const int nimpls = model->state && comb < model->state->nslots ? model->state->nimpls[comb] : 0;
            for (int impl = 0; impl < nimpls; ++impl) print_one(model, a, (unsigned)impl, parameter, footprint, output);
        }
        return 0;
    }
    int k;
    if (!strcmp(arch, "cpu")) {
        print_single(model, STARPU_CPU_WORKER, 0, 1, parameter, footprint, output);
        return 0;
    }
    if (sscanf(arch, "cpu:%d", &k) == 1) {
        if (k < 1 || k > STARPU_NMAXWORKERS) {
            fprintf(stderr, "[starpu_gb300] invalid CPU size %d\n", k);
            return -1;
        }
        print_single(model, STARPU_CPU_WORKER, 0, k, parameter, footprint, output);
        return 0;
    }
    if (!strcmp(arch, "cuda")) {
        const int n = starpu_perfmodel_get_narch_combs();
        for (int comb = 0; comb < n; ++comb) {
            struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
            if (a->ndevices == 1 && a->devices[0].type == STARPU_CUDA_WORKER)
                print_single(model, STARPU_CUDA_WORKER, a->devices[0].devid, 1, parameter, footprint, output);
        }
        return 0;
    }
    if (sscanf(arch, "cuda_%d", &k) == 1 || sscanf(arch, "cuda%d", &k) == 1) {
        print_single(model, STARPU_CUDA_WORKER, k, 1, parameter, footprint, output);
        return 0;
    }
    fprintf(stderr, "[starpu_gb300] unknown architecture requested\n");
    return -1;
}

/* per worker, the mean for `footprint` on its architecture, "inf" when none (perfmodel_print.c:288-324) */
int starpu_perfmodel_print_estimations(struct starpu_perfmodel *model, uint32_t footprint, FILE *output)
{
    ensure_model(model);
    for (unsigned w = 0; w < starpu_worker_get_count(); ++w) {
        struct starpu_perfmodel_arch *a = starpu_worker_get_perf_archtype((int)w, 0);
        const int comb = a ? starpu_perfmodel_arch_comb_get(a->ndevices, a->devices) : -1;
        pthread_mutex_lock(&model_mu);
        struct pm_entry *e = find_entry(per_arch_if_any(model->state, comb, 0), footprint);
        const double mean = e ? e->mean : 0.0;
        pthread_mutex_unlock(&model_mu);
        if (e) fprintf(output, "%s%e", w ? " " : "", mean);
        else fprintf(output, "%sinf", w ? " " : "");
    }
    return 0;
}

/* "Model <symbol>" and one line per combination and device (perfmodel_history.c:2107-2126) */
int starpu_perfmodel_list_combs(FILE *output, struct starpu_perfmodel *model)
{
    fprintf(output, "Model <%s>\n", model->symbol);
    for (int i = 0; model->state && i < model->state->ncombs; ++i) {
        const int comb = model->state->combs[i];
        struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
        fprintf(output, "\tComb %d: %d device%s\n", comb, a->ndevices, a->ndevices > 1 ? "s" : "");
        for (int d = 0; d < a->ndevices; ++d)
            fprintf(output, "\t\tDevice %d: type: %s - devid: %d - ncores: %d\n", d,
                    starpu_perfmodel_get_archtype_name(a->devices[d].type), a->devices[d].devid,
                    a->devices[d].ncores);
    }
    return 0;
}

/* perfmodel_history.c:970-1122 */
void starpu_perfmodel_dump_xml(FILE *f, struct starpu_perfmodel *model)
{
    ensure_model(model);
    fprintf(f, "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n");
    fprintf(f, "<!DOCTYPE StarPUPerfmodel SYSTEM \"starpu-perfmodel.dtd\">\n");
    fprintf(f, "<!-- symbol %s -->\n", model->symbol);
    fprintf(f, "<!-- All times in us -->\n");
    fprintf(f, "<perfmodel version=\"%u\">\n", PM_VERSION);
    pthread_mutex_lock(&model_mu);
    struct starpu_perfmodel_history_state *s = model->state;
    for (int i = 0; s && i < s->ncombs; ++i) {
        const int comb = s->combs[i];
        struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
        fprintf(f, "  <combination>\n");
        for (int d = 0; d < a->ndevices; ++d) {
            fprintf(f, "    <device type=\"%s\" id=\"%d\"", archtype_upper(a->devices[d].type), a->devices[d].devid);
            if (a->devices[d].type == STARPU_CPU_WORKER) fprintf(f, " ncores=\"%d\"", a->devices[d].ncores);
            fprintf(f, "/>\n");
        }
        for (int impl = 0; impl < s->nimpls[comb]; ++impl) {
            struct pm_per_arch *pa = &s->per_arch[comb][impl];
            const struct pm_regression *g = &pa->reg;
            char name[600];
            starpu_perfmodel_get_arch_name(a, name, sizeof name, (unsigned)impl);
            fprintf(f, "    <implementation id=\"%d\">\n", impl);
            fprintf(f, "      <!-- %s -->\n", name);
            if (model->type == STARPU_REGRESSION_BASED) {
                fprintf(f, "      <!-- time = alpha size ^ beta -->\n");
                fprintf(f, "      <l_regression sumlnx=\"%e\" sumlnx2=\"%e\" sumlny=\"%e\" sumlnxlny=\"%e\"", g->sumlnx,
                        g->sumlnx2, g->sumlny, g->sumlnxlny);
                fprintf(f, " alpha=\"");
                write_double(f, "%e", g->alpha);
                fprintf(f, "\" beta=\"");
                write_double(f, "%e", g->beta);
                fprintf(f, "\" nsample=\"%u\" minx=\"%lu\" maxx=\"%lu\"/>\n", g->nsample, g->minx, g->maxx);
            } else if (model->type == STARPU_NL_REGRESSION_BASED) {
                fprintf(f, "      <!-- time = a size ^b + c -->\n");
                fprintf(f, "      <nl_regression a=\"");
                write_double(f, "%e", g->a);
                fprintf(f, "\" b=\"");
                write_double(f, "%e", g->b);
                fprintf(f, "\" c=\"");
                write_double(f, "%e", g->c);
                fprintf(f, "\"/>\n");
            } else if (model->type == STARPU_MULTIPLE_REGRESSION_BASED) {
                /* a model loaded from its file has no parameter combinations */
                fprintf(f, "      <ml_regression constant=\"nan\"/>\n");
            }
            for (struct pm_entry *e = pa->list; e; e = e->next)
                fprintf(f,
                        "      <entry footprint=\"%08x\" size=\"%zu\" flops=\"%e\" mean=\"%e\" deviation=\"%e\" "
                        "sum=\"%e\" sum2=\"%e\" nsample=\"%u\"/>\n",
                        e->footprint, e->size, e->flops, e->mean, e->deviation, e->sum, e->sum2, e->nsample);
            fprintf(f, "    </implementation>\n");
        }
        fprintf(f, "  </combination>\n");
    }
    pthread_mutex_unlock(&model_mu);
    fprintf(f, "</perfmodel>\n");
}

/* ------------------------------------------------- tooling: gnuplot files */

static char *dashes(const char *str)
{
    char *p = strdup(str);
    for (char *q = p; *q; ++q)
        if (*q == '_') *q = '-';
    return p;
}

static void plot_sep(FILE *f, int *first)
{
    if (*first) *first = 0;
    else fprintf(f, ",\\\n\t");
}

static int plot_selected(int comb, int only_comb) { return only_comb < 0 || only_comb == comb; }

/*
 * The gnuplot script and averages file of tools/starpu_perfmodel_plot.c
 * (its display_perf_model, display_history_based_perf_models and
 * display_selected_models, lines 281-575): regression curves per combination
 * and implementation, then one errorline per history list, reading the
 * averages file whose rows are the distinct data sizes in increasing order
 * with (value, error) pairs per list ("" "" where a list has no entry of that
 * size).  Times are in ms, energies in J, rates in GFlop/s (per W with -e);
 * with an energy model the value is power (W) from the two models' means.
 */
int starpu_gb300_perfmodel_plot(struct starpu_perfmodel *model, struct starpu_perfmodel *energy_model,
                                const char *symbol, const char *energy_symbol, int only_comb, int gflops, int energy,
                                const char *gp_path, const char *avg_path)
{
    struct starpu_perfmodel_history_state *s = model->state;
    if (!s) return -EINVAL;
    FILE *gp = fopen(gp_path, "w+");
    if (!gp) return -errno;
    FILE *data = fopen(avg_path, "w");
    if (!data) {
        int err = errno;
        fclose(gp);
        return -err;
    }
    char host[256];
    host_name(host, sizeof host);
    char *dsym = dashes(symbol);
    const char *prefix = energy_symbol ? "power_" : gflops ? "gflops_" : "";
    fprintf(gp, "#!/usr/bin/gnuplot -persist\n\n");
    fprintf(gp, "set term postscript eps enhanced color\n");
    fprintf(gp, "set output \"starpu_%s%s.eps\"\n", prefix, symbol);
    fprintf(gp, "set title \"Model for codelet %s on %s\"\n", dsym, host);
    fprintf(gp, "set xlabel \"Total data size\"\n");
    if (energy_symbol) fprintf(gp, "set ylabel \"Power (W)\"\n");
    else if (gflops) fprintf(gp, energy ? "set ylabel \"GFlop/s/W\"\n" : "set ylabel \"GFlop/s\"\n");
    else fprintf(gp, energy ? "set ylabel \"Energy (J)\"\n" : "set ylabel \"Time (ms)\"\n");
    fprintf(gp, "\nset key top left\nset logscale x\nset logscale y\n\n");
    fprintf(gp, "set xrange [1 < * < 10**9 : 1 < * < 10**9]\n\n");
    fprintf(gp, "plot\t");
    int first = 1;
    const char *factor = energy ? "" : "0.001 * ";
    if (!energy_symbol && !gflops)
        for (int i = 0; i < s->ncombs; ++i) {
            const int comb = s->combs[i];
            if (!plot_selected(comb, only_comb)) continue;
            struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
            for (int impl = 0; impl < s->nimpls[comb]; ++impl) {
                const struct pm_regression *g = &s->per_arch[comb][impl].reg;
                char name[256];
                starpu_perfmodel_get_arch_name(a, name, sizeof name, (unsigned)impl);
                if (g->valid && !g->nl_valid) {
                    plot_sep(gp, &first);
                    fprintf(gp, "%s%g * x ** %g title \"Linear Regression %s\"", factor, g->alpha, g->beta, name);
                }
                if (g->nl_valid) {
                    plot_sep(gp, &first);
                    fprintf(gp, "%s%g * x ** %g + %s%g title \"Non-Linear Regression %s\"", factor, g->a, g->b,
                            factor, g->c, name);
                }
            }
        }
    int col = 2;
    for (int i = 0; i < s->ncombs; ++i) {
        const int comb = s->combs[i];
        if (!plot_selected(comb, only_comb)) continue;
        struct starpu_perfmodel_arch *a = starpu_perfmodel_arch_comb_fetch(comb);
        for (int impl = 0; impl < s->nimpls[comb]; ++impl) {
            if (!s->per_arch[comb][impl].list) continue;
            char name[32]; /* the tool's own buffer size: longer names are cut */
            starpu_perfmodel_get_arch_name(a, name, sizeof name, (unsigned)impl);
            char *dname = dashes(name);
            plot_sep(gp, &first);
            fprintf(gp, "\"%s\" using 1:%d:%d with errorlines title \"Average %s\"", avg_path, col, col + 1, dname);
            col += 2;
            free(dname);
        }
    }
    unsigned long last = 0;
    for (;;) {
        unsigned long next = ~0UL;
        for (int i = 0; i < s->ncombs; ++i) {
            const int comb = s->combs[i];
            if (!plot_selected(comb, only_comb)) continue;
            for (int impl = 0; impl < s->nimpls[comb]; ++impl)
                for (struct pm_entry *e = s->per_arch[comb][impl].list; e; e = e->next)
                    if (e->size > last && e->size < next) next = e->size;
        }
        if (next == ~0UL) break;
        last = next;
        fprintf(data, "%-15lu ", next);
        for (int i = 0; i < s->ncombs; ++i) {
            const int comb = s->combs[i];
            if (!plot_selected(comb, only_comb)) continue;
            for (int impl = 0; impl < s->nimpls[comb]; ++impl) {
                struct pm_per_arch *pa = &s->per_arch[comb][impl];
                int found = 0;
                for (struct pm_entry *e = pa->list; e; e = e->next) {
                    if (e->size != next) continue;
                    if (energy_symbol) {
                        struct pm_per_arch *pb = per_arch_if_any(energy_model->state, comb, impl);
                        for (struct pm_entry *q = pb ? pb->list : NULL; q; q = q->next)
                            if (q->size == next) {
                                const double rel = sqrt((q->deviation * q->deviation) / (q->mean * q->mean) +
                                                        (e->deviation * e->deviation) / (e->mean * e->mean));
                                const double watts = q->mean / (e->mean / 1000000);
                                fprintf(data, "\t%-15le\t%-15le", watts, watts * rel);
                                found = 1;
                                break;
                            }
                    } else if (gflops) {
                        if (energy)
                            fprintf(data, "\t%-15le\t%-15le", e->flops / e->mean / 1e9,
                                    e->flops * e->deviation / (e->mean * e->mean) / 1e9);
                        else
                            fprintf(data, "\t%-15le\t%-15le", e->flops / (e->mean * 1000),
                                    e->flops * e->deviation / (e->mean * e->mean * 1000));
                        found = 1;
                    } else {
                        if (energy) fprintf(data, "\t%-15le\t%-15le", e->mean, e->deviation);
                        else fprintf(data, "\t%-15le\t%-15le", 0.001 * e->mean, 0.001 * e->deviation);
                        found = 1;
                    }
                    break;
                }
                if (!found && pa->list) fprintf(data, "\t\"\"\t\"\"");
            }
        }
        fprintf(data, "\n");
    }
    fclose(data);
    fprintf(gp, "\nset term png\n");
    fprintf(gp, "set output \"starpu_%s%s.png\"\n", prefix, symbol);
    fprintf(gp, "replot\n\n");
    fclose(gp);
    free(dsym);
    return 0;
}
