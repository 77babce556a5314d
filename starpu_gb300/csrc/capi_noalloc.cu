// Allocation-free FP32 POTRS for callers that cannot allocate device memory.
//
// Some callers of this library must not allocate: a StarPU codelet body runs
// on the worker's stream inside a runtime that owns every device buffer and
// hands the codelet only its data (a cudaMalloc there would synchronise the
// device and break the worker's asynchronous pipeline), and serving loops and
// real-time hosts forbid allocation on their request path.  This entry point
// gives them the same solve as starpu_gb300_spotrs_sweep without a workspace
// argument: its scratch (the inverted 64 x 64 diagonal blocks, the sweeps'
// completion flags and an error word) lives in one file-scope device array of
// fixed size, which every GPU that loads the library keeps until the process
// exits.  The caller still passes the factor and the right-hand sides.
//
// Set-up: the first call on each device (with that device current) looks the
// array's device address up with cudaGetSymbolAddress and caches it; make that
// first call before any stream capture.  All calls share the one array and it
// keeps the last call's contents: calls whose work overlaps on the GPU (for
// instance on two streams) race on it and must be serialised by the caller.
// Without a caller status word (d_err NULL) the call waits for its stream and
// returns GB300_ETIMEDOUT if a sweep wait ran out.
#include <mutex>
#include <stdio.h>

#include "gb300_internal.h"
#include "starpu_gb300_kernels.h"

namespace {

// Largest order n supported: 16384 / 64 = 256 inverted blocks of 16 KiB (4 MiB),
// plus the flags and the error word.
constexpr int NOALLOC_MAX_N = STARPU_GB300_NOALLOC_MAX_N;
constexpr size_t NOALLOC_SWEEP_BYTES = (size_t)(NOALLOC_MAX_N / 64) * 64 * 64 * sizeof(float) + 2048;
constexpr size_t NOALLOC_ERR_OFFSET = NOALLOC_SWEEP_BYTES;
constexpr size_t NOALLOC_BYTES = NOALLOC_SWEEP_BYTES + 256;

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
void *g_scratch_dev[MAX_DEVICES];  // device address of the array, per device

} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of the scratch array on the current device (looked up once per device).
static int noalloc_scratch(void **out)
{
    int dev = 0;
    int rc = gb300_record_cuda_error(cudaGetDevice(&dev));
    if (rc) return rc;
    if (dev < 0 || dev >= MAX_DEVICES) return GB300_ENOTSUP;
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_dev[dev]) {
        void *p = nullptr;
        rc = gb300_record_cuda_error(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (rc) return rc;
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return GB300_OK;
}

extern "C" int starpu_gb300_spotrs_noalloc(void *stream, int n, int nrhs, const float *L, int ldl, float *B, int ldb,
                                           int *d_err)
{
    if (n < 0 || nrhs < 0 || ldl < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (n > NOALLOC_MAX_N) {
        gb300_set_error("starpu_gb300_spotrs_noalloc: n exceeds STARPU_GB300_NOALLOC_MAX_N (16384); "
                        "use starpu_gb300_spotrs_sweep with a caller-provided workspace");
        return GB300_EINVAL;
    }
    if (!n || !nrhs) return GB300_OK;
    void *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    if (gb300::potrs_sweep_workspace<float>(n) > NOALLOC_SWEEP_BYTES) return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    // A caller's d_err is used as starpu_gb300_spotrs_sweep uses it: set on a
    // timeout, never cleared here.  Without one the array's own error word is
    // cleared (it keeps the previous call's value), and read back once the
    // solve has run, so that a timeout still reaches the caller.
    int *err = d_err ? d_err : (int *)((char *)scratch + NOALLOC_ERR_OFFSET);
    if (!d_err && (rc = gb300_record_cuda_error(cudaMemsetAsync(err, 0, sizeof(int), s)))) return rc;
    gb300::potrs_sweep_prepare<float>(s, n, L, ldl, scratch);
    gb300::potrs_sweep<float>(s, n, nrhs, L, ldl, scratch, B, ldb, err);
    if ((rc = gb300_last_launch_status()) || d_err) return rc;
    int h_err = 0;
    if ((rc = gb300_record_cuda_error(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s))) ||
        (rc = gb300_record_cuda_error(cudaStreamSynchronize(s))))
        return rc;
    if (h_err) {
        gb300_set_error("starpu_gb300_spotrs_noalloc: a sweep wait timed out; B is invalid");
        return GB300_ETIMEDOUT;
    }
    return GB300_OK;
}
