// Synthetic SPD inputs generated on the device, with the same streams as the
// CPU generators used by the tests: row i of the N(0,1) matrix B comes from
// PCG64 (XSL-RR 128/64) stream i+1, Box-Muller pairs fill (even, odd)
// columns; right-hand side column j is U[-1,1] from stream 2^40 + j.  The
// device log/sin/cos may differ from the host libm in the last ulp, so device
// and host inputs agree to ~1e-15 relative, not bit for bit.
#include "gb300_internal.h"
#include "starpu_gb300_kernels.h"
#include "starpu_gb300_solver.h"

namespace gb300 {

struct pcg64 {
    unsigned __int128 state, inc;
};

__device__ __forceinline__ uint64_t pcg_next(pcg64 &r)
{
    const unsigned __int128 mult = ((unsigned __int128)0x2360ED051FC65DA4ULL << 64) | 0x4385DF649FCCF645ULL;
    r.state = r.state * mult + r.inc;
    uint64_t hi = (uint64_t)(r.state >> 64), lo = (uint64_t)r.state;
    uint64_t x = hi ^ lo;
    unsigned rot = (unsigned)(hi >> 58);
    return (x >> rot) | (x << ((64 - rot) & 63));
}

__device__ __forceinline__ void pcg_seed(pcg64 &r, uint64_t seed, uint64_t stream)
{
    r.inc = ((unsigned __int128)stream << 1) | 1u;
    r.state = 0;
    pcg_next(r);
    r.state += ((unsigned __int128)seed << 64) | (unsigned __int128)(seed ^ 0x9E3779B97F4A7C15ULL);
    pcg_next(r);
}

__global__ void gen_normal_kernel(int rows, int cols, uint64_t seed, double *__restrict__ B, long ldb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    pcg64 r;
    pcg_seed(r, seed, (uint64_t)i + 1);
    const double two_pi = 6.283185307179586476925286766559;
    for (int j = 0; j < cols; j += 2) {
        double u1 = ((double)(pcg_next(r) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
        double u2 = (double)(pcg_next(r) >> 11) * (1.0 / 9007199254740992.0);
        double rad = sqrt(-2.0 * log(u1));
        double s, c;
        sincos(two_pi * u2, &s, &c);
        B[i + (long)j * ldb] = rad * c;
        if (j + 1 < cols) B[i + (long)(j + 1) * ldb] = rad * s;
    }
}

__global__ void gen_uniform_rhs_kernel(int n, int nrhs, uint64_t seed, double *__restrict__ B, long ldb)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs) return;
    pcg64 r;
    pcg_seed(r, seed, ((uint64_t)1 << 40) + (uint64_t)j);
    for (int i = 0; i < n; i++) B[i + (long)j * ldb] = 2.0 * ((double)(pcg_next(r) >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

// Mirror the lower triangle into the upper one and add alpha on the diagonal.
__global__ void symmetrize_shift_kernel(int n, double alpha, double *__restrict__ A, long lda)
{
    const int tj = blockIdx.y * 32, ti = blockIdx.x * 32;
    if (ti < tj) return;  // tile (ti, tj) of the lower part
    __shared__ double t[32][33];
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        int i = ti + threadIdx.x, j = tj + c;
        if (i < n && j < n) {
            double v = A[i + (long)j * lda];
            if (i == j) {
                v += alpha;
                A[i + (long)j * lda] = v;
            }
            t[c][threadIdx.x] = v;
        }
    }
    __syncthreads();
    // write (j, i) = (i, j) for i > j
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        int j = tj + threadIdx.x, i = ti + c;  // element (i, j) of lower, stored at t[j - tj][i - ti]
        if (i < n && j < n && i > j) A[j + (long)i * lda] = t[threadIdx.x][c];
    }
}

__global__ void shift_diagonal_kernel(int n, double delta, double *__restrict__ A, long lda)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        A[i + i * lda] += delta;
}

} // namespace gb300

using namespace gb300;

extern "C" {

int starpu_gb300_gen_normal(void *stream, int rows, int cols, uint64_t seed, double *B, int ldb)
{
    if (rows < 0 || cols < 0 || ldb < (rows > 1 ? rows : 1)) return GB300_EINVAL;
    if (!rows || !cols) return GB300_OK;
    gb300_count_launch(), gen_normal_kernel<<<(rows + 127) / 128, 128, 0, (cudaStream_t)stream>>>(rows, cols, seed, B, ldb);
    return gb300_last_launch_status();
}

int starpu_gb300_gen_uniform_rhs(void *stream, int n, int nrhs, uint64_t seed, double *B, int ldb)
{
    if (n < 0 || nrhs < 0 || ldb < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (!n || !nrhs) return GB300_OK;
    gb300_count_launch(), gen_uniform_rhs_kernel<<<(nrhs + 63) / 64, 64, 0, (cudaStream_t)stream>>>(n, nrhs, seed, B, ldb);
    return gb300_last_launch_status();
}

int starpu_gb300_gen_spd_gram(void *stream, int n, uint64_t seed, double alpha, double *A, int lda, double *work)
{
    if (n < 0 || lda < (n > 1 ? n : 1) || !work) return GB300_EINVAL;
    if (!n) return GB300_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = starpu_gb300_gen_normal(stream, n, n, seed, work, n);
    if (rc) return rc;
    gemm<double>(s, false, true, true, n, n, n, 1.0 / (double)n, work, n, work, n, 0.0, A, lda);
    dim3 g((n + 31) / 32, (n + 31) / 32);
    gb300_count_launch(), symmetrize_shift_kernel<<<g, dim3(32, 8), 0, s>>>(n, alpha, A, lda);
    return gb300_last_launch_status();
}

int starpu_gb300_shift_diagonal(void *stream, int n, double *A, int lda, double delta)
{
    if (n < 0 || lda < (n > 1 ? n : 1)) return GB300_EINVAL;
    if (!n) return GB300_OK;
    gb300_count_launch(), shift_diagonal_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, delta, A, lda);
    return gb300_last_launch_status();
}

int starpu_gb300_set_device(int device) { return gb300_record_cuda_error(cudaSetDevice(device)); }

int starpu_gb300_memcpy_d2d(void *stream, void *dst, const void *src, size_t bytes)
{
    return gb300_record_cuda_error(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
}

} // extern "C"
