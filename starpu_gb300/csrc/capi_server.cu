// Serving: a request loop with continuous batching, a device-resident factor
// cache and an HBM budget (see starpu_gb300_solver.h for the contract).
//
// Executors are host threads, each bound to one CUDA stream and to buffers
// sized for the largest admitted system; executors pull from one admission
// queue.  A free executor takes every queued small request (n <= 1024,
// nrhs <= 8; up to 512 of them within its batch buffers) as one persistent
// batched launch, or else the oldest large request, which it solves with the
// tensor-core factorisation + FP64 refinement -- reusing the device-resident
// factor when the request's matrix_id is cached.  Requests therefore join the
// device as soon as an executor frees, and executors overlap on the GPU.
// Every request is computed by a fixed kernel sequence chosen by its own size
// alone (batched systems are independent CTAs), so its result is the same
// whether it runs alone or in the mix.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string.h>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gb300_internal.h"
#include "starpu.h"
#include "starpu_gb300_kernels.h"
#include "starpu_gb300_solver.h"

namespace {

constexpr int SMALL_MAX_N = 1024;
constexpr int SMALL_MAX_RHS = 8;
constexpr int BATCH_MAX = 512;
constexpr long long BATCH_A_ELEMS = 16ll << 20;   // 128 MiB of FP64 matrices per batched launch
constexpr int NB = 1024;

struct CacheEntry {
    uint64_t id = 0;
    int n = 0;
    double *A = nullptr;
    void *ws = nullptr;
    size_t bytes = 0;
    int in_use = 0;
    bool ready = false;
    unsigned long long last = 0;
};

struct Exec {
    std::thread th;
    cudaStream_t s = nullptr;
    double *A = nullptr, *B = nullptr, *X = nullptr;
    void *ws = nullptr;
    size_t lws = 0;
    double *pA = nullptr, *pB = nullptr, *pX = nullptr;  // batch pools
    void *bws = nullptr;
    size_t lbws = 0;
};

} // namespace

struct starpu_gb300_server {
    size_t budget = 0, used = 0;
    int mode = 0, max_n = 0, max_nrhs = 0, nexec = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<starpu_gb300_request *> queue;
    std::unordered_map<uint64_t, CacheEntry *> cache;
    std::vector<Exec> ex;
    bool stop = false;
    long inflight = 0;
    unsigned long long tick = 0, served = 0, batches = 0, hits = 0, evictions = 0;
};

static bool is_small(const starpu_gb300_server *sv, const starpu_gb300_request *r)
{
    return sv->mode == 0 && r->n <= SMALL_MAX_N && r->nrhs <= SMALL_MAX_RHS;
}

static void finish(starpu_gb300_server *sv, starpu_gb300_request *r)
{
    r->end_us = starpu_timing_now();
    std::lock_guard<std::mutex> g(sv->mu);
    r->done = 1;
    sv->served++;
    sv->inflight--;
    sv->cv_done.notify_all();
}

static int copy_in(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    return gb300_record_cuda_error(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
}

// evict least-recently used entries that are not in use until `need` bytes fit (lock held)
static bool make_room(starpu_gb300_server *sv, size_t need, cudaStream_t s)
{
    while (sv->used + need > sv->budget) {
        CacheEntry *victim = nullptr;
        for (auto &kv : sv->cache)
            if (kv.second->in_use == 0 && kv.second->ready && (!victim || kv.second->last < victim->last))
                victim = kv.second;
        if (!victim) return false;
        cudaFreeAsync(victim->A, s);
        cudaFreeAsync(victim->ws, s);
        sv->used -= victim->bytes;
        sv->cache.erase(victim->id);
        delete victim;
        sv->evictions++;
    }
    return true;
}

static void serve_large(starpu_gb300_server *sv, Exec &e, starpu_gb300_request *r)
{
    cudaStream_t s = e.s;
    const int n = r->n, nrhs = r->nrhs;
    const double tol = r->tol > 0 ? r->tol : 1e-12;
    const int max_iter = r->max_iter > 0 ? r->max_iter : 30;
    starpu_gb300_ir_info info;
    memset(&info, 0, sizeof info);
    int rc = 0;
    if (sv->mode == 1) {  // plain baseline: FP64 dposv, alone
        rc = copy_in(e.A, r->A, sizeof(double) * (size_t)n * n, s);
        if (!rc) rc = copy_in(e.X, r->B, sizeof(double) * (size_t)n * nrhs, s);
        if (!rc) rc = starpu_gb300_dposv(s, n, nrhs, e.A, n, e.X, n, 512, nullptr);
        if (!rc) rc = copy_in(r->X, e.X, sizeof(double) * (size_t)n * nrhs, s);
        if (!rc) rc = gb300_record_cuda_error(cudaStreamSynchronize(s));
        r->status = rc;
        finish(sv, r);
        return;
    }
    CacheEntry *entry = nullptr;
    bool fresh = false;
    const size_t ws_bytes = starpu_gb300_dsposv_workspace(n, sv->max_nrhs, NB);
    {
        std::lock_guard<std::mutex> g(sv->mu);
        if (r->matrix_id && sv->mode == 0) {  // mode 2 keeps no factors
            auto it = sv->cache.find(r->matrix_id);
            if (it != sv->cache.end() && it->second->ready && it->second->n == n) {
                entry = it->second;
                entry->in_use++;
                entry->last = ++sv->tick;
                sv->hits++;
            } else if (it == sv->cache.end()) {
                const size_t need = sizeof(double) * (size_t)n * n + ws_bytes;
                if (make_room(sv, need, s)) {
                    entry = new CacheEntry();
                    entry->id = r->matrix_id;
                    entry->n = n;
                    entry->bytes = need;
                    entry->in_use = 1;
                    entry->last = ++sv->tick;
                    sv->used += need;
                    sv->cache[r->matrix_id] = entry;
                    fresh = true;
                }
            }
        }
    }
    double *Adev = e.A;
    void *ws = e.ws;
    if (entry && fresh) {
        rc = gb300_record_cuda_error(cudaMallocAsync((void **)&entry->A, sizeof(double) * (size_t)n * n, s));
        if (!rc) rc = gb300_record_cuda_error(cudaMallocAsync(&entry->ws, ws_bytes, s));
    }
    if (!rc && entry) {
        Adev = entry->A;
        ws = entry->ws;
    }
    if (!rc) rc = copy_in(e.B, r->B, sizeof(double) * (size_t)n * nrhs, s);
    if (!rc && !(entry && !fresh)) {
        if (!r->A) rc = GB300_EINVAL;  // no cached factor for this id and no matrix given
        if (!rc) rc = copy_in(Adev, r->A, sizeof(double) * (size_t)n * n, s);
        if (!rc) rc = gb300::dsposv_factor(s, n, nrhs, Adev, n, NB, 3, ws, &info);
    } else if (!rc) {
        r->cache_hit = 1;
    }
    if (!rc) rc = gb300::dsposv_refine(s, n, nrhs, Adev, n, e.B, n, e.X, n, NB, tol, max_iter, ws, &info);
    if (rc == GB300_OK || rc == GB300_ETIMEDOUT) {
        int rc2 = copy_in(r->X, e.X, sizeof(double) * (size_t)n * nrhs, s);
        if (!rc2) rc2 = gb300_record_cuda_error(cudaStreamSynchronize(s));
        if (rc2) rc = rc2;
    } else {
        cudaStreamSynchronize(s);
    }
    {
        std::lock_guard<std::mutex> g(sv->mu);
        if (entry) {
            entry->in_use--;
            if (fresh) {
                if (rc == GB300_OK || rc == GB300_ETIMEDOUT) {
                    entry->ready = true;
                } else {  // factor failed: do not keep it
                    cudaFreeAsync(entry->A, s);
                    cudaFreeAsync(entry->ws, s);
                    sv->used -= entry->bytes;
                    sv->cache.erase(entry->id);
                    delete entry;
                }
            }
        }
    }
    r->status = rc;
    r->iterations = info.iterations;
    r->backward_error = info.backward_error;
    finish(sv, r);
}

static void serve_batch(starpu_gb300_server *sv, Exec &e, std::vector<starpu_gb300_request *> &rs)
{
    cudaStream_t s = e.s;
    const int nsys = (int)rs.size();
    std::vector<int> ns(nsys), status(nsys);
    std::vector<long long> ao(nsys), bo(nsys);
    std::vector<double> berr(nsys);
    int nrhs = 1;
    for (auto *r : rs) nrhs = std::max(nrhs, r->nrhs);
    long long a = 0, b = 0;
    int rc = 0;
    for (int i = 0; i < nsys && !rc; ++i) {
        starpu_gb300_request *r = rs[i];
        ns[i] = r->n;
        ao[i] = a;
        bo[i] = b;
        rc = copy_in(e.pA + a, r->A, sizeof(double) * (size_t)r->n * r->n, s);
        if (!rc) rc = copy_in(e.pB + b, r->B, sizeof(double) * (size_t)r->n * r->nrhs, s);
        if (!rc && r->nrhs < nrhs)  // padded right-hand sides are zero
            rc = gb300_record_cuda_error(
                cudaMemsetAsync(e.pB + b + (long long)r->n * r->nrhs, 0, sizeof(double) * (size_t)r->n * (nrhs - r->nrhs), s));
        a += (long long)r->n * r->n;
        b += (long long)r->n * nrhs;
    }
    double tol = 1e-12;
    int max_iter = 30;
    for (auto *r : rs) {
        if (r->tol > 0) tol = std::min(tol, r->tol);
        if (r->max_iter > 0) max_iter = std::max(max_iter, r->max_iter);
    }
    if (!rc)
        rc = starpu_gb300_dposv_batched(s, nsys, ns.data(), e.pA, ao.data(), e.pB, bo.data(), e.pX, nrhs, tol, max_iter,
                                        e.bws, e.lbws, status.data(), berr.data());
    for (int i = 0; i < nsys && !rc; ++i) rc = copy_in(rs[i]->X, e.pX + bo[i], sizeof(double) * (size_t)ns[i] * rs[i]->nrhs, s);
    if (!rc) rc = gb300_record_cuda_error(cudaStreamSynchronize(s));
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->batches++;
    }
    for (int i = 0; i < nsys; ++i) {
        starpu_gb300_request *r = rs[i];
        r->batched = 1;
        r->iterations = status[i] >= 0 ? status[i] : 0;
        r->backward_error = berr[i];
        r->status = rc ? rc : (status[i] >= 0 ? GB300_OK : (status[i] == -1000 ? GB300_ETIMEDOUT : GB300_EDOM));
        finish(sv, r);
    }
}

static void executor_main(starpu_gb300_server *sv, int idx)
{
    Exec &e = sv->ex[idx];
    for (;;) {
        std::vector<starpu_gb300_request *> batch;
        starpu_gb300_request *large = nullptr;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv_work.wait(lk, [&] { return sv->stop || !sv->queue.empty(); });
            if (sv->queue.empty()) return;
            if (is_small(sv, sv->queue.front())) {
                long long elems = 0;
                for (auto it = sv->queue.begin(); it != sv->queue.end() && (int)batch.size() < BATCH_MAX;) {
                    starpu_gb300_request *r = *it;
                    const long long need = (long long)r->n * r->n;
                    if (is_small(sv, r) && elems + need <= BATCH_A_ELEMS) {
                        elems += need;
                        batch.push_back(r);
                        it = sv->queue.erase(it);
                    } else {
                        ++it;
                    }
                }
            } else {
                large = sv->queue.front();
                sv->queue.pop_front();
            }
        }
        const double now = starpu_timing_now();
        if (large) {
            large->start_us = now;
            serve_large(sv, e, large);
        } else {
            for (auto *r : batch) r->start_us = now;
            serve_batch(sv, e, batch);
        }
    }
}

static void free_exec(Exec &e)
{
    cudaFree(e.A);
    cudaFree(e.B);
    cudaFree(e.X);
    cudaFree(e.ws);
    cudaFree(e.pA);
    cudaFree(e.pB);
    cudaFree(e.pX);
    cudaFree(e.bws);
    if (e.s) cudaStreamDestroy(e.s);
}

extern "C" {

starpu_gb300_server *starpu_gb300_server_create(size_t hbm_budget_bytes, int executors, int max_n, int max_nrhs,
                                                int mode)
{
    if (executors < 1 || max_n < 1 || max_nrhs < 1 || mode < 0 || mode > 2) return nullptr;
    starpu_gb300_server *sv = new starpu_gb300_server();
    sv->budget = hbm_budget_bytes;
    sv->mode = mode;
    sv->max_n = max_n;
    sv->max_nrhs = max_nrhs;
    sv->nexec = executors;
    sv->ex.resize(executors);
    bool ok = true;
    for (auto &e : sv->ex) {
        ok &= !gb300_record_cuda_error(cudaStreamCreateWithFlags(&e.s, cudaStreamNonBlocking));
        ok &= !gb300_record_cuda_error(cudaMalloc(&e.A, sizeof(double) * (size_t)max_n * max_n));
        ok &= !gb300_record_cuda_error(cudaMalloc(&e.B, sizeof(double) * (size_t)max_n * max_nrhs));
        ok &= !gb300_record_cuda_error(cudaMalloc(&e.X, sizeof(double) * (size_t)max_n * max_nrhs));
        size_t bytes = sizeof(double) * ((size_t)max_n * max_n + 2 * (size_t)max_n * max_nrhs);
        if (mode == 2) {  // per-request mixed solves: one solver workspace, no batch pools
            e.lws = starpu_gb300_dsposv_workspace(max_n, max_nrhs, NB);
            ok &= !gb300_record_cuda_error(cudaMalloc(&e.ws, e.lws));
            bytes += e.lws;
        }
        if (mode == 0) {
            e.lws = starpu_gb300_dsposv_workspace(max_n, max_nrhs, NB);
            ok &= !gb300_record_cuda_error(cudaMalloc(&e.ws, e.lws));
            const long long bmax = BATCH_A_ELEMS / 32 * SMALL_MAX_RHS + (long long)SMALL_MAX_N * SMALL_MAX_RHS * BATCH_MAX;
            ok &= !gb300_record_cuda_error(cudaMalloc(&e.pA, sizeof(double) * BATCH_A_ELEMS));
            ok &= !gb300_record_cuda_error(cudaMalloc(&e.pB, sizeof(double) * bmax));
            ok &= !gb300_record_cuda_error(cudaMalloc(&e.pX, sizeof(double) * bmax));
            // worst case of the batched workspace: every element of the pools used
            std::vector<int> worst(BATCH_MAX, 32);
            e.lbws = starpu_gb300_dposv_batched_workspace(BATCH_MAX, worst.data(), SMALL_MAX_RHS) +
                     sizeof(float) * (BATCH_A_ELEMS + bmax) + sizeof(double) * bmax + (1 << 20);
            ok &= !gb300_record_cuda_error(cudaMalloc(&e.bws, e.lbws));
            bytes += e.lws + sizeof(double) * (BATCH_A_ELEMS + 2 * bmax) + e.lbws;
        }
        sv->used += bytes;
    }
    if (!ok || sv->used > sv->budget) {
        if (ok) gb300_set_error("starpu_gb300_server_create: executor buffers exceed the HBM budget");
        for (auto &e : sv->ex) free_exec(e);
        delete sv;
        return nullptr;
    }
    for (int i = 0; i < executors; ++i) sv->ex[i].th = std::thread(executor_main, sv, i);
    return sv;
}

int starpu_gb300_server_submit(starpu_gb300_server *sv, starpu_gb300_request *r)
{
    if (!sv || !r || r->n < 1 || r->nrhs < 1 || r->n > sv->max_n || r->nrhs > sv->max_nrhs || !r->B || !r->X ||
        (!r->A && !r->matrix_id))
        return GB300_EINVAL;
    r->done = 0;
    r->status = 0;
    r->cache_hit = 0;
    r->batched = 0;
    r->iterations = 0;
    r->backward_error = 0;
    r->submit_us = starpu_timing_now();
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->queue.push_back(r);
        sv->inflight++;
    }
    sv->cv_work.notify_one();
    return GB300_OK;
}

int starpu_gb300_server_wait(starpu_gb300_server *sv, starpu_gb300_request *r)
{
    if (!sv || !r) return GB300_EINVAL;
    // a request that was never queued is not waited for: with nothing in
    // flight and r not done, submit refused it (or it was never submitted)
    std::unique_lock<std::mutex> lk(sv->mu);
    sv->cv_done.wait(lk, [&] { return r->done != 0 || sv->inflight == 0; });
    return r->done ? r->status : GB300_EINVAL;
}

int starpu_gb300_server_drain(starpu_gb300_server *sv)
{
    if (!sv) return GB300_EINVAL;
    std::unique_lock<std::mutex> lk(sv->mu);
    sv->cv_done.wait(lk, [&] { return sv->inflight == 0; });
    return GB300_OK;
}

int starpu_gb300_server_stats(starpu_gb300_server *sv, unsigned long long *served, unsigned long long *batches,
                              unsigned long long *cache_hits, unsigned long long *evictions, size_t *bytes_in_use)
{
    if (!sv) return GB300_EINVAL;
    std::lock_guard<std::mutex> g(sv->mu);
    if (served) *served = sv->served;
    if (batches) *batches = sv->batches;
    if (cache_hits) *cache_hits = sv->hits;
    if (evictions) *evictions = sv->evictions;
    if (bytes_in_use) *bytes_in_use = sv->used;
    return GB300_OK;
}

int starpu_gb300_server_destroy(starpu_gb300_server *sv)
{
    if (!sv) return GB300_OK;
    starpu_gb300_server_drain(sv);
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto &e : sv->ex)
        if (e.th.joinable()) e.th.join();
    for (auto &kv : sv->cache) {
        cudaFree(kv.second->A);
        cudaFree(kv.second->ws);
        delete kv.second;
    }
    for (auto &e : sv->ex) free_exec(e);
    delete sv;
    return GB300_OK;
}

} // extern "C"
