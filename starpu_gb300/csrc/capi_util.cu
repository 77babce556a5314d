// Error reporting and device-memory helpers of the C-ABI.
#include "gb300_internal.h"
#include <algorithm>
#include <atomic>
#include <mutex>
#include <stdio.h>
#include <string.h>
#include <vector>

static thread_local char g_last_error[256] = "";
static std::atomic<unsigned long long> g_launches{0};

extern "C" void gb300_count_launch(void) { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ---- profiling: CUDA-event pairs per launch, resolved lazily -------------
namespace {
struct ProfRec {
    cudaEvent_t e0, e1;
    int kind;
    double flops, bytes;
    double sm_share;  // fraction of the SMs the launch's grid was limited to
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<ProfRec> g_prof_pending;
std::vector<cudaEvent_t> g_event_pool;
struct ProfAgg {
    unsigned long long launches = 0;
    double ms = 0, flops = 0, bytes = 0;
    double share_ms = 0;  // sum of time x SM share
} g_prof_agg[GB300_PROF_KINDS];

cudaEvent_t pool_get()
{
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// per-launch timeline (start / end relative to the first launch after a
// reset), kept for the last kMaxTimeline launches
struct ProfSpan {
    int kind;
    double start_ms, end_ms;
};
constexpr size_t kMaxTimeline = 1 << 16;
std::vector<ProfSpan> g_prof_timeline;
cudaEvent_t g_prof_origin = nullptr;  // e0 of the first launch after a reset (kept out of the pool)

void resolve_locked()
{
    for (auto &r : g_prof_pending) {
        cudaEventSynchronize(r.e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, r.e0, r.e1);
        if (!g_prof_origin) {
            g_prof_origin = r.e0;
            r.e0 = pool_get();  // the pool gets a fresh event in place of the kept one
        }
        if (g_prof_timeline.size() < kMaxTimeline) {
            float t0 = 0;
            if (r.e0 != nullptr) cudaEventElapsedTime(&t0, g_prof_origin, r.e1);
            g_prof_timeline.push_back({r.kind, (double)t0 - ms, (double)t0});
        }
        auto &a = g_prof_agg[r.kind];
        a.launches++;
        a.ms += ms;
        a.flops += r.flops;
        a.bytes += r.bytes;
        a.share_ms += ms * r.sm_share;
        g_event_pool.push_back(r.e0);
        g_event_pool.push_back(r.e1);
    }
    g_prof_pending.clear();
}
} // namespace

extern "C" int gb300_prof_begin(cudaStream_t s, int kind)
{
    std::lock_guard<std::mutex> g(g_prof_mu);
    if (!g_prof_on) return -1;
    ProfRec r;
    r.e0 = pool_get();
    r.e1 = pool_get();
    r.kind = kind;
    r.flops = r.bytes = 0;
    r.sm_share = 1.0;
    cudaEventRecord(r.e0, s);
    g_prof_pending.push_back(r);
    return (int)g_prof_pending.size() - 1;
}

extern "C" void gb300_prof_end(cudaStream_t s, int slot, double flops, double bytes)
{
    std::lock_guard<std::mutex> g(g_prof_mu);
    if (slot < 0 || slot >= (int)g_prof_pending.size()) return;
    ProfRec &r = g_prof_pending[slot];
    r.flops = flops;
    r.bytes = bytes;
    cudaEventRecord(r.e1, s);
}

extern "C" void gb300_prof_set_share(int slot, double sm_share)
{
    std::lock_guard<std::mutex> g(g_prof_mu);
    if (slot < 0 || slot >= (int)g_prof_pending.size()) return;
    g_prof_pending[slot].sm_share = sm_share;
}

extern "C" int gb300_record_cuda_error(cudaError_t e)
{
    if (e == cudaSuccess) return GB300_OK;
    snprintf(g_last_error, sizeof g_last_error, "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return GB300_ECUDA;
}

extern "C" void gb300_set_error(const char *msg) { snprintf(g_last_error, sizeof g_last_error, "%s", msg); }

// ---- per-device launch set-up ----------------------------------------------
// A kernel's dynamic shared memory limit is a property of the function on one
// device: the first launch on every device needs its own cudaFuncSetAttribute.
// The book keeps (function, device, bytes) triples under a mutex, so host
// threads racing on a first call set the attribute once and never read a
// half-written entry.
namespace {
std::mutex g_attr_mu;
struct AttrRec {
    const void *fn;
    int dev, bytes;
};
std::vector<AttrRec> g_attr;

// setter(fn, bytes) is called for (fn, dev) unless an entry with at least
// `bytes` exists; the entry is recorded only when the setter succeeds.
template <typename F> int attr_book_ensure(std::vector<AttrRec> &book, const void *fn, int dev, int bytes, F setter)
{
    for (const auto &r : book)
        if (r.fn == fn && r.dev == dev && r.bytes >= bytes) return GB300_OK;
    const int rc = setter(fn, bytes);
    if (rc == GB300_OK) {
        for (auto &r : book)
            if (r.fn == fn && r.dev == dev) {
                r.bytes = bytes;
                return rc;
            }
        book.push_back({fn, dev, bytes});
    }
    return rc;
}

constexpr unsigned long long kDefaultWaitBudgetNs = 2000000000ull;  // 2 s: far above any legitimate stall
std::atomic<unsigned long long> g_wait_budget_ns{kDefaultWaitBudgetNs};

constexpr int kMaxDevices = 64;
std::atomic<int> g_sms[kMaxDevices];
} // namespace

extern "C" int gb300_func_dyn_smem(const void *fn, int bytes)
{
    int dev = 0;
    int rc = gb300_record_cuda_error(cudaGetDevice(&dev));
    if (rc) return rc;
    std::lock_guard<std::mutex> g(g_attr_mu);
    return attr_book_ensure(g_attr, fn, dev, bytes, [](const void *f, int b) {
        return gb300_record_cuda_error(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    });
}

extern "C" int gb300_device_sms(void)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    if (dev < 0 || dev >= kMaxDevices) dev = 0;
    int n = g_sms[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 1;
        }
        g_sms[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

extern "C" unsigned long long gb300_wait_budget_ns(void) { return g_wait_budget_ns.load(std::memory_order_relaxed); }

extern "C" int gb300_last_launch_status(void)
{
    return gb300_record_cuda_error(cudaGetLastError());
}

extern "C" {

const char *starpu_gb300_last_error(void) { return g_last_error; }

unsigned long long starpu_gb300_set_wait_budget_ns(unsigned long long ns)
{
    return g_wait_budget_ns.exchange(ns ? ns : kDefaultWaitBudgetNs);
}

int starpu_gb300_selftest_attr_book(void)
{
    std::vector<AttrRec> book;
    int calls = 0, fail = 0;
    auto setter = [&](const void *, int) {
        ++calls;
        return fail ? GB300_ECUDA : GB300_OK;
    };
    static const char f1 = 0, f2 = 0, f3 = 0;
    struct Step {
        const void *fn;
        int dev, bytes, fail, calls_after, rc;
    } steps[] = {
        {&f1, 0, 54272, 0, 1, GB300_OK},     // first launch on device 0
        {&f1, 0, 54272, 0, 1, GB300_OK},     // again on device 0: nothing to do
        {&f1, 1, 54272, 0, 2, GB300_OK},     // first launch on device 1 sets it there too
        {&f1, 0, 40000, 0, 2, GB300_OK},     // a smaller request is covered
        {&f1, 0, 100000, 0, 3, GB300_OK},    // a larger one raises the limit
        {&f1, 0, 100000, 0, 3, GB300_OK},
        {&f1, 1, 100000, 0, 4, GB300_OK},    // ... separately per device
        {&f2, 0, 54272, 0, 5, GB300_OK},     // another function
        {&f3, 0, 1024, 1, 6, GB300_ECUDA},   // a failed set-up is not recorded
        {&f3, 0, 1024, 0, 7, GB300_OK},      // and is retried on the next call
        {&f3, 0, 1024, 0, 7, GB300_OK},
    };
    int i = 0;
    for (const Step &st : steps) {
        ++i;
        fail = st.fail;
        const int rc = attr_book_ensure(book, st.fn, st.dev, st.bytes, setter);
        if (rc != st.rc || calls != st.calls_after) return i;
    }
    return book.size() == 4 ? 0 : i + 1;
}

void *starpu_gb300_device_malloc(size_t bytes)
{
    void *p = nullptr;
    if (gb300_record_cuda_error(cudaMalloc(&p, bytes ? bytes : 1)) != GB300_OK) return nullptr;
    return p;
}

int starpu_gb300_device_free(void *p) { return gb300_record_cuda_error(cudaFree(p)); }

void *starpu_gb300_host_malloc_pinned(size_t bytes)
{
    void *p = nullptr;
    if (gb300_record_cuda_error(cudaMallocHost(&p, bytes ? bytes : 1)) != GB300_OK) return nullptr;
    return p;
}

int starpu_gb300_host_free_pinned(void *p) { return gb300_record_cuda_error(cudaFreeHost(p)); }

int starpu_gb300_memcpy_h2d(void *stream, void *dst, const void *src, size_t bytes)
{
    return gb300_record_cuda_error(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
}

int starpu_gb300_memcpy_d2h(void *stream, void *dst, const void *src, size_t bytes)
{
    return gb300_record_cuda_error(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
}

int starpu_gb300_memset(void *stream, void *dst, int value, size_t bytes)
{
    return gb300_record_cuda_error(cudaMemsetAsync(dst, value, bytes, (cudaStream_t)stream));
}

int starpu_gb300_stream_sync(void *stream) { return gb300_record_cuda_error(cudaStreamSynchronize((cudaStream_t)stream)); }

void *starpu_gb300_stream_create(void)
{
    cudaStream_t s = nullptr;
    if (gb300_record_cuda_error(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != GB300_OK) return nullptr;
    return (void *)s;
}

int starpu_gb300_stream_destroy(void *stream) { return gb300_record_cuda_error(cudaStreamDestroy((cudaStream_t)stream)); }

unsigned long long starpu_gb300_launch_count(void) { return g_launches.load(); }

void starpu_gb300_profiling_enable(int on)
{
    std::lock_guard<std::mutex> g(g_prof_mu);
    if (!on) resolve_locked();
    g_prof_on = on != 0;
}

void starpu_gb300_profiling_reset(void)
{
    std::lock_guard<std::mutex> g(g_prof_mu);
    resolve_locked();
    for (auto &a : g_prof_agg) a = ProfAgg();
    g_prof_timeline.clear();
    if (g_prof_origin) {
        g_event_pool.push_back(g_prof_origin);
        g_prof_origin = nullptr;
    }
}

int starpu_gb300_profiling_timeline(int max, int *kinds, double *start_ms, double *end_ms)
{
    if (max < 0) return GB300_EINVAL;
    std::lock_guard<std::mutex> g(g_prof_mu);
    resolve_locked();
    const int n = (int)std::min((size_t)max, g_prof_timeline.size());
    for (int i = 0; i < n; ++i) {
        if (kinds) kinds[i] = g_prof_timeline[i].kind;
        if (start_ms) start_ms[i] = g_prof_timeline[i].start_ms;
        if (end_ms) end_ms[i] = g_prof_timeline[i].end_ms;
    }
    return (int)g_prof_timeline.size();
}

int starpu_gb300_profiling_get(int kind, unsigned long long *launches, double *total_ms, double *flops, double *bytes)
{
    if (kind < 0 || kind >= GB300_PROF_KINDS) return GB300_EINVAL;
    std::lock_guard<std::mutex> g(g_prof_mu);
    resolve_locked();
    if (launches) *launches = g_prof_agg[kind].launches;
    if (total_ms) *total_ms = g_prof_agg[kind].ms;
    if (flops) *flops = g_prof_agg[kind].flops;
    if (bytes) *bytes = g_prof_agg[kind].bytes;
    return GB300_OK;
}

int starpu_gb300_profiling_sm_share(int kind, double *share)
{
    if (kind < 0 || kind >= GB300_PROF_KINDS || !share) return GB300_EINVAL;
    std::lock_guard<std::mutex> g(g_prof_mu);
    resolve_locked();
    const ProfAgg &a = g_prof_agg[kind];
    *share = a.ms > 0 ? a.share_ms / a.ms : 1.0;
    return GB300_OK;
}

void *starpu_gb300_event_create(void)
{
    cudaEvent_t e = nullptr;
    if (gb300_record_cuda_error(cudaEventCreate(&e)) != GB300_OK) return nullptr;
    return (void *)e;
}

int starpu_gb300_event_record(void *event, void *stream)
{
    return gb300_record_cuda_error(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream));
}

double starpu_gb300_event_elapsed_ms(void *start, void *end)
{
    float ms = -1.0f;
    if (cudaEventSynchronize((cudaEvent_t)end) != cudaSuccess ||
        cudaEventElapsedTime(&ms, (cudaEvent_t)start, (cudaEvent_t)end) != cudaSuccess) {
        gb300_record_cuda_error(cudaGetLastError());
        return -1.0;
    }
    return ms;
}

int starpu_gb300_event_destroy(void *event) { return gb300_record_cuda_error(cudaEventDestroy((cudaEvent_t)event)); }

int starpu_gb300_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

} // extern "C"
