// Error reporting and device-memory helpers of the C-ABI.
#include "gb300_internal.h"
#include <stdio.h>
#include <string.h>

static thread_local char g_last_error[256] = "";

extern "C" int gb300_record_cuda_error(cudaError_t e)
{
    if (e == cudaSuccess) return GB300_OK;
    snprintf(g_last_error, sizeof g_last_error, "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return GB300_ECUDA;
}

extern "C" int gb300_last_launch_status(void)
{
    return gb300_record_cuda_error(cudaGetLastError());
}

extern "C" {

const char *starpu_gb300_last_error(void) { return g_last_error; }

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
