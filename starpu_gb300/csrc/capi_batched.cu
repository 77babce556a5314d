// Batched SPD solve (many independent systems of uneven sizes in one
// persistent launch) and its block-size autotuner.
//
// The tuning table is stored next to StarPU's history perfmodels, as
//   <perfmodel dir>/codelets/45/gb300_chol_tuning.<hostname>
// (the path starpu_perfmodel_get_model_path() gives for that symbol):
//   "bucket max_n nb time_us"   the batched solver's block size NB per size bucket;
//   "dense nb lookahead_sms t_diag_us update_tflops panel_rate n step_ms"
//                               the mixed solve's schedule for tile nb (written
//                               by starpu_gb300_dense_autotune, capi_tc.cu).
// Each autotuner rewrites its own lines and keeps the other's.
#include <algorithm>
#include <math.h>
#include <mutex>
#include <numeric>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "gb300_internal.h"
#include "kernels/batched_chol.cuh"
#include "starpu.h"
#include "starpu_gb300_solver.h"

namespace gb300 {

static const int kBuckets = 6;                      // n <= 32, 64, 128, 256, 512, 1024
static signed char g_nb_table[kBuckets] = {16, 32, 32, 64, 64, 64};
static double g_nb_us[kBuckets] = {0, 0, 0, 0, 0, 0};
static bool g_nb_tuned = false;
static const int kDense = 8;
static DenseTuning g_dense[kDense];
static int g_ndense = 0;
static bool g_table_loaded = false;
static std::mutex g_table_mu;

static size_t smem_bytes() { return (size_t)(64 * 65 + 2 * 64 * BAT_TP) * sizeof(float); }

// the existing table file, else where a new one is written
static void tuning_path(char *path, size_t len)
{
    starpu_perfmodel_get_model_path("gb300_chol_tuning", path, len);
    if (!path[0]) starpu_perfmodel_get_model_path_default_location("gb300_chol_tuning", path, len);
}

static void load_table_locked()
{
    if (g_table_loaded) return;
    g_table_loaded = true;
    char path[1200];
    tuning_path(path, sizeof path);
    FILE *f = fopen(path, "r");
    if (!f) return;
    char line[256];
    while (fgets(line, sizeof line, f)) {
        int b, maxn, nb;
        double us;
        if (line[0] == '#') continue;
        DenseTuning d;
        if (sscanf(line, "dense %d %d %lf %lf %lf %d %lf", &d.nb, &d.lookahead_sms, &d.t_diag_us, &d.update_tflops,
                   &d.panel_rate, &d.n, &d.step_ms) == 7) {
            if (d.nb > 0 && d.t_diag_us > 0 && d.update_tflops > 0 && d.panel_rate > 0 && g_ndense < kDense)
                g_dense[g_ndense++] = d;
            continue;
        }
        if (sscanf(line, "%d %d %d %lf", &b, &maxn, &nb, &us) == 4 && b >= 0 && b < kBuckets &&
            (nb == 16 || nb == 32 || nb == 64)) {
            g_nb_table[b] = (signed char)nb;
            g_nb_us[b] = us;
            g_nb_tuned = true;
        }
    }
    fclose(f);
}

// the whole table (both autotuners' lines), written through a temporary file
static int write_table_locked()
{
    char path[1200];
    tuning_path(path, sizeof path);
    // create the directory chain like the perfmodel writer does
    for (char *p = path + 1; *p; ++p)
        if (*p == '/') {
            *p = 0;
            mkdir(path, 0755);
            *p = '/';
        }
    char tmp[1300];
    snprintf(tmp, sizeof tmp, "%s.tmp", path);
    FILE *f = fopen(tmp, "w");
    if (!f) return GB300_EINVAL;
    static const int maxn_of[kBuckets] = {32, 64, 128, 256, 512, 1024};
    if (g_nb_tuned) {
        fprintf(f, "# GB300 batched Cholesky tuning: diagonal/panel block size per size bucket\n");
        fprintf(f, "# bucket max_n nb time_us\n");
        for (int b = 0; b < kBuckets; ++b) fprintf(f, "%d %d %d %.3f\n", b, maxn_of[b], (int)g_nb_table[b], g_nb_us[b]);
    }
    if (g_ndense) {
        fprintf(f, "# GB300 mixed-solve schedule per tile size (lookahead_sms -1: chosen per step by the model)\n");
        fprintf(f, "# dense nb lookahead_sms t_diag_us update_tflops panel_rate n step_ms\n");
        for (int i = 0; i < g_ndense; ++i)
            fprintf(f, "dense %d %d %.3f %.3f %.4f %d %.4f\n", g_dense[i].nb, g_dense[i].lookahead_sms,
                    g_dense[i].t_diag_us, g_dense[i].update_tflops, g_dense[i].panel_rate, g_dense[i].n,
                    g_dense[i].step_ms);
    }
    const bool ok = fclose(f) == 0 && rename(tmp, path) == 0;
    if (!ok) unlink(tmp);
    return ok ? GB300_OK : GB300_EINVAL;
}

bool dense_tuning(int nb, DenseTuning *out)
{
    std::lock_guard<std::mutex> g(g_table_mu);
    load_table_locked();
    for (int i = 0; i < g_ndense; ++i)
        if (g_dense[i].nb == nb) {
            if (out) *out = g_dense[i];
            return true;
        }
    return false;
}

int dense_tuning_store(const DenseTuning &d)
{
    std::lock_guard<std::mutex> g(g_table_mu);
    load_table_locked();
    int i = 0;
    while (i < g_ndense && g_dense[i].nb != d.nb) ++i;
    if (i == g_ndense) {
        if (g_ndense == kDense) return GB300_ENOMEM;
        ++g_ndense;
    }
    g_dense[i] = d;
    return write_table_locked();
}

// Persistent grid of the batched kernel on the current device: the SMs times
// the CTAs resident per SM (the shared memory limit is set per device first).
static int batched_grid()
{
    if (gb300_func_dyn_smem((const void *)batched_dposv_kernel, (int)smem_bytes())) return 0;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batched_dposv_kernel, BAT_THREADS, smem_bytes()) !=
        cudaSuccess) {
        cudaGetLastError();
        per = 1;
    }
    return gb300_device_sms() * std::max(1, per);
}

struct BatWs {
    int *n, *order, *status;
    long long *a_off, *b_off;
    double *berr, *R;
    float *W, *Y;
    unsigned *ticket;
    signed char *nb;
};

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t bat_layout(int nsys, long long wtotal, long long btotal, void *base, BatWs *ws)
{
    size_t off = 0;
    auto take = [&](size_t b) {
        size_t o = off;
        off = al(off + b);
        return o;
    };
    size_t on = take(sizeof(int) * nsys), oo = take(sizeof(int) * nsys), os = take(sizeof(int) * nsys);
    size_t oa = take(sizeof(long long) * nsys), ob = take(sizeof(long long) * nsys);
    size_t oe = take(sizeof(double) * nsys), oR = take(sizeof(double) * btotal);
    size_t oW = take(sizeof(float) * wtotal), oY = take(sizeof(float) * btotal);
    size_t ot = take(sizeof(unsigned)), onb = take(kBuckets);
    if (base && ws) {
        char *b = (char *)base;
        ws->n = (int *)(b + on);
        ws->order = (int *)(b + oo);
        ws->status = (int *)(b + os);
        ws->a_off = (long long *)(b + oa);
        ws->b_off = (long long *)(b + ob);
        ws->berr = (double *)(b + oe);
        ws->R = (double *)(b + oR);
        ws->W = (float *)(b + oW);
        ws->Y = (float *)(b + oY);
        ws->ticket = (unsigned *)(b + ot);
        ws->nb = (signed char *)(b + onb);
    }
    return off;
}

static void totals(int nsys, const int *n, int nrhs, long long *wt, long long *bt)
{
    long long w = 0, b = 0;
    for (int i = 0; i < nsys; ++i) {
        w += (long long)n[i] * n[i];
        b += (long long)n[i] * nrhs;
    }
    *wt = w;
    *bt = b;
}

// Launch over systems whose metadata is in host arrays; synchronous.
static int run_batched(cudaStream_t s, int nsys, const int *n, const double *A, const long long *a_off,
                       const double *B, const long long *b_off, double *X, int nrhs, double tol, int max_iter,
                       void *work, size_t lwork, const signed char *nb_table, int *status, double *berr,
                       float *kernel_ms)
{
    long long wt, bt;
    totals(nsys, n, nrhs, &wt, &bt);
    if (lwork < bat_layout(nsys, wt, bt, nullptr, nullptr)) return GB300_EINVAL;
    BatWs ws;
    bat_layout(nsys, wt, bt, work, &ws);
    // W / Y / R reuse the caller's offsets, which index A / B (elements)
    std::vector<int> order(nsys);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
    std::vector<long long> aoff(a_off, a_off + nsys), boff(b_off, b_off + nsys);
    int rc;
    if ((rc = gb300_record_cuda_error(cudaMemcpyAsync(ws.n, n, sizeof(int) * nsys, cudaMemcpyHostToDevice, s)))) return rc;
    cudaMemcpyAsync(ws.order, order.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.a_off, aoff.data(), sizeof(long long) * nsys, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.b_off, boff.data(), sizeof(long long) * nsys, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.nb, nb_table, kBuckets, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(ws.ticket, 0, sizeof(unsigned), s);
    BatchedArgs a;
    a.nsys = nsys;
    a.n = ws.n;
    a.a_off = ws.a_off;
    a.b_off = ws.b_off;
    a.order = ws.order;
    a.smem_bytes = smem_bytes();
    a.A = A;
    a.B = B;
    a.X = X;
    a.W = ws.W;
    a.Y = ws.Y;
    a.R = ws.R;
    a.nrhs = nrhs;
    a.tol = tol;
    a.max_iter = max_iter;
    a.status = ws.status;
    a.berr = ws.berr;
    a.ticket = ws.ticket;
    a.nb_of_bucket = ws.nb;
    const int bgrid = batched_grid();
    if (bgrid <= 0) return GB300_ECUDA;  // the attribute set-up failed; its message is recorded
    const int grid = std::min(nsys, bgrid);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (kernel_ms) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
    }
    int slot = gb300_prof_begin(s, GB300_PROF_BATCHED);
    gb300_count_launch(), batched_dposv_kernel<<<grid, BAT_THREADS, smem_bytes(), s>>>(a);
    double fl = 0;
    for (int i = 0; i < nsys; ++i) fl += (double)n[i] * n[i] * n[i] / 3.0 + 2.0 * (double)n[i] * n[i] * nrhs;
    gb300_prof_end(s, slot, fl, 8.0 * (double)wt);
    if (kernel_ms) cudaEventRecord(e1, s);
    if ((rc = gb300_last_launch_status())) return rc;
    if (status) cudaMemcpyAsync(status, ws.status, sizeof(int) * nsys, cudaMemcpyDeviceToHost, s);
    if (berr) cudaMemcpyAsync(berr, ws.berr, sizeof(double) * nsys, cudaMemcpyDeviceToHost, s);
    rc = gb300_record_cuda_error(cudaStreamSynchronize(s));
    if (kernel_ms) {
        cudaEventElapsedTime(kernel_ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return rc;
}

// A_ij = 1/(1+i+j) + n delta_ij for a batch of identical sizes (tuning input)
__global__ void fill_tuning_kernel(int n, int nsys, double *A, double *B, int nrhs)
{
    const long total = (long)n * n * nsys;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const long e = idx % ((long)n * n);
        const int i = (int)(e % n), j = (int)(e / n);
        A[idx] = 1.0 / (1.0 + i + j) + (i == j ? (double)n : 0.0);
    }
    const long tb = (long)n * nrhs * nsys;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < tb; idx += (long)gridDim.x * blockDim.x)
        B[idx] = 1.0 - 2.0 * (double)((idx * 2654435761u) % 1000) / 1000.0;
}

} // namespace gb300

using namespace gb300;

extern "C" {

size_t starpu_gb300_dposv_batched_workspace(int nsys, const int *n, int nrhs)
{
    if (nsys <= 0 || !n || nrhs <= 0) return 0;
    long long wt, bt;
    totals(nsys, n, nrhs, &wt, &bt);
    return bat_layout(nsys, wt, bt, nullptr, nullptr);
}

int starpu_gb300_dposv_batched(void *stream, int nsys, const int *n, const double *A, const long long *a_off,
                               const double *B, const long long *b_off, double *X, int nrhs, double tol,
                               int max_iter, void *work, size_t lwork, int *status, double *berr)
{
    if (nsys < 0 || nrhs < 1 || nrhs > BAT_MAXRHS || max_iter < 0 || !(tol >= 0)) return GB300_EINVAL;
    if (!nsys) return GB300_OK;
    if (!n || !a_off || !b_off || !A || !B || !X || !work) return GB300_EINVAL;
    for (int i = 0; i < nsys; ++i)
        if (n[i] < 1 || n[i] > BAT_MAXN || a_off[i] < 0 || b_off[i] < 0) return GB300_EINVAL;
    signed char table[kBuckets];
    {
        std::lock_guard<std::mutex> g(g_table_mu);
        load_table_locked();
        memcpy(table, g_nb_table, sizeof table);
    }
    return run_batched((cudaStream_t)stream, nsys, n, A, a_off, B, b_off, X, nrhs, tol, max_iter, work, lwork,
                       table, status, berr, nullptr);
}

int starpu_gb300_batched_get_tuning(signed char *nb_per_bucket, int nbuckets)
{
    if (!nb_per_bucket || nbuckets < kBuckets) return GB300_EINVAL;
    std::lock_guard<std::mutex> g(g_table_mu);
    load_table_locked();
    memcpy(nb_per_bucket, g_nb_table, kBuckets);
    return kBuckets;
}

int starpu_gb300_batched_autotune(int systems_per_bucket, int reps)
{
    if (systems_per_bucket <= 0) systems_per_bucket = 2 * std::max(1, batched_grid());
    if (reps <= 0) reps = 2;
    cudaStream_t s = nullptr;
    const int nrhs = 4;
    const int maxn_of[kBuckets] = {32, 64, 128, 256, 512, 1024};
    const int cands[3] = {16, 32, 64};
    signed char best_nb[kBuckets];
    double best_us[kBuckets];
    for (int b = 0; b < kBuckets; ++b) {
        const int n = maxn_of[b] * 3 / 4;  // a size inside the bucket
        const int nsys = b >= 4 ? std::max(1, systems_per_bucket / (b == 5 ? 4 : 2)) : systems_per_bucket;
        std::vector<int> ns(nsys, n);
        std::vector<long long> ao(nsys), bo(nsys);
        for (int i = 0; i < nsys; ++i) {
            ao[i] = (long long)i * n * n;
            bo[i] = (long long)i * n * nrhs;
        }
        double *A = nullptr, *B = nullptr, *X = nullptr;
        void *work = nullptr;
        size_t lw = starpu_gb300_dposv_batched_workspace(nsys, ns.data(), nrhs);
        if (cudaMalloc(&A, sizeof(double) * (size_t)nsys * n * n) || cudaMalloc(&B, sizeof(double) * (size_t)nsys * n * nrhs) ||
            cudaMalloc(&X, sizeof(double) * (size_t)nsys * n * nrhs) || cudaMalloc(&work, lw)) {
            cudaFree(A);
            cudaFree(B);
            cudaFree(X);
            cudaFree(work);
            return gb300_record_cuda_error(cudaGetLastError());
        }
        gb300_count_launch(), fill_tuning_kernel<<<1024, 256, 0, s>>>(n, nsys, A, B, nrhs);
        best_us[b] = INFINITY;
        best_nb[b] = g_nb_table[b];
        for (int c = 0; c < 3; ++c) {
            if (cands[c] > 2 * maxn_of[b]) continue;
            signed char table[kBuckets];
            memcpy(table, g_nb_table, kBuckets);
            table[b] = (signed char)cands[c];
            double tot = 0;
            int ok = 1;
            for (int r = 0; r <= reps; ++r) {
                float ms = 0;
                int rc = run_batched(s, nsys, ns.data(), A, ao.data(), B, bo.data(), X, nrhs, 1e-12, 10, work, lw,
                                     table, nullptr, nullptr, &ms);
                if (rc) {
                    ok = 0;
                    break;
                }
                if (r > 0) tot += ms;  // first run is a warm-up
            }
            const double us = tot / reps * 1e3;
            if (ok && us < best_us[b]) {
                best_us[b] = us;
                best_nb[b] = (signed char)cands[c];
            }
        }
        cudaFree(A);
        cudaFree(B);
        cudaFree(X);
        cudaFree(work);
    }
    std::lock_guard<std::mutex> g(g_table_mu);
    load_table_locked();
    memcpy(g_nb_table, best_nb, kBuckets);
    for (int b = 0; b < kBuckets; ++b) g_nb_us[b] = best_us[b];
    g_nb_tuned = true;
    return write_table_locked();
}

} // extern "C"
