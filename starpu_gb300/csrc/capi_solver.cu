// Mixed-precision SPD solve with FP64 iterative refinement (LAPACK dsposv
// semantics with uplo = L: only the lower triangle of A is read; no reference
// counterpart: the reference Cholesky is FP32 factorisation only,
// examples/cholesky/cholesky_kernels.c:53-55).
//
//   W = fp32(A)                       (lower triangle, fused with ||A||_inf)
//   W = L L^T                         tensor-core tiled Cholesky (scaled-FP16 split)
//   x = fp64(L^-T L^-1 fp32(b))
//   repeat: r = b - A x   (FP64)      backward error ||r||/(||A|| ||x|| + ||b||)
//           x += fp64(L^-T L^-1 fp32(r))
// until every right-hand side meets `tol` or `max_iter` corrections ran.
// FP64 is used only for A, the residual and the solution accumulation.
#include <algorithm>
#include <atomic>
#include <functional>
#include <vector>
#include <stdlib.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "gb300_internal.h"
#include "kernels/tile_sweep.cuh"
#include "kernels/residual_df.cuh"
#include "kernels/simt_blas.cuh"
#include "starpu_gb300_kernels.h"
#include "starpu_gb300_solver.h"

namespace gb300 {


// W(c, r) = W(r, c) for the rows r in [r0, n) below the column block
// [c0, c0 + w): the strictly upper part of W then holds L^T outside the
// diagonal tiles, which the backward sweeps read column by column like the
// forward ones.  32 x 32 tiles transposed through shared memory.
__global__ void mirror_block_kernel(int n, int c0, int w, int r0, float *W, long ldw)
{
    __shared__ float t[32][33];
    const int rb = r0 + blockIdx.x * 32, cb = c0 + blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = rb + threadIdx.x, c = cb + y;
        if (r < n && c < c0 + w) t[y][threadIdx.x] = W[r + (long)c * ldw];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = rb + y, c = cb + threadIdx.x;
        if (r < n && c < c0 + w) W[c + (long)r * ldw] = t[threadIdx.x][y];
    }
}

// One CTA per column j of A: writes the lower part of column j to W in FP32
// and folds sum_i |A_ij| (= row sum of the symmetric A) into *anorm.
__global__ void convert_lower_norm_kernel(int n, const double *__restrict__ A, long lda, float *__restrict__ W,
                                          long ldw, unsigned long long *anorm_bits)
{
    const long j = blockIdx.x;
    const double *a = A + j * lda;
    float *w = W ? W + j * ldw : nullptr;
    double s = 0.0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = a[i];
        s += fabs(v);
        if (w && i >= j) w[i] = (float)v;
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicMax(anorm_bits, (unsigned long long)__double_as_longlong(s));
    }
}

// W = fp32(A) on and below the diagonal (W optional), one CTA per column j
// (rows j .. n-1), and max |A_ij| over the lower triangle into *amax_bits as
// FP64 bits (an integer max of the magnitudes' bit patterns: exact and
// order-independent).  The scale of the residual's digit slices and of the
// infinity norm below.
__global__ void __launch_bounds__(256) convert_lower_max_kernel(int n, const double *__restrict__ A, long lda,
                                                                float *__restrict__ W, long ldw,
                                                                unsigned long long *amax_bits, int j0 = 0)
{
    const long j = j0 + (long)blockIdx.x;
    const double *a = A + j * lda;
    float *w = W ? W + j * ldw : nullptr;
    unsigned long long m = 0;
    auto take = [&](long i, double v) {
        m = max(m, (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull);
        if (w) w[i] = (float)v;
    };
    long i0 = j;
    // one element first when the column's lower part starts off a 16-byte boundary
    if (i0 < n && ((uintptr_t)(a + i0) & 15)) {
        if (threadIdx.x == 0) take(i0, a[i0]);
        ++i0;
    }
    const bool vec = !((uintptr_t)(a + i0) & 15) && (!w || !((uintptr_t)(w + i0) & 7));
    if (vec) {
        // 16-byte loads, four in flight per thread: the conversion streams A at
        // the HBM rate instead of waiting on one load at a time
        const double2 *a2 = (const double2 *)(a + i0);
        float2 *w2 = w ? (float2 *)(w + i0) : nullptr;
        const long n2 = (n - i0) / 2;
        for (long p = threadIdx.x; p < n2; p += 4 * 256) {
            double2 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (p + u * 256 < n2) v[u] = __ldcs(a2 + p + u * 256);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (p + u * 256 >= n2) break;
                m = max(m, (unsigned long long)__double_as_longlong(v[u].x) & 0x7FFFFFFFFFFFFFFFull);
                m = max(m, (unsigned long long)__double_as_longlong(v[u].y) & 0x7FFFFFFFFFFFFFFFull);
                if (w2) w2[p + u * 256] = make_float2((float)v[u].x, (float)v[u].y);
            }
        }
        if (((n - i0) & 1) && threadIdx.x == 0) take(n - 1, a[n - 1]);
    } else {
        for (long i = i0 + threadIdx.x; i < n; i += 256) take(i, a[i]);
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)m, o));
    __shared__ unsigned long long red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < 8; ++q) m = max(m, red[q]);
        atomicMax(amax_bits, m);
    }
}

// ||A||_inf of the symmetric A from the per-tile row sums of |A| 2^-alpha
// (rowsum[bk n + i], written while A is cut into its digit slices): each row
// summed in a fixed order in FP64, the maximum folded into *anorm_bits.
__global__ void norm_from_rowsums_kernel(int n, int nbk, const float *__restrict__ rowsum,
                                         const unsigned long long *__restrict__ amax_bits,
                                         unsigned long long *anorm_bits)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double sum = 0.0;
    if (i < n)
        for (int bk = 0; bk < nbk; ++bk) sum += (double)rowsum[(long)bk * n + i];
    const double amax = __longlong_as_double((long long)*amax_bits);
    const int alpha = (amax > 0.0 && isfinite(amax)) ? ilogb(amax) + 1 : 1;
    unsigned long long m = (unsigned long long)__double_as_longlong(ldexp(sum, alpha));
    for (int o = 16; o > 0; o >>= 1) m = max(m, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(anorm_bits, m);
}

// y (FP32, n x nrhs) = fp32(x_j * 2^-e_j); used for b and r.  The power-of-two
// column scale (e_j = exponent of max |x_j|) keeps the FP32 solve away from
// overflow and from underflow once the residual has become small.
__global__ void to_f32_kernel(int n, int nrhs, const double *__restrict__ x, long ldx, float *__restrict__ y, long ldy,
                              const int *__restrict__ exps)
{
    const long j = blockIdx.y;
    const int e = exps[j];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i + j * ldy] = (float)scalbn(x[i + j * ldx], -e);
}

// x (FP64) = (accumulate ? x : 0) + fp64(y_j) * 2^e_j, skipping converged columns
__global__ void accumulate_kernel(int n, int nrhs, const float *__restrict__ y, long ldy, double *__restrict__ x,
                                  long ldx, int accumulate, const int *__restrict__ done, const int *__restrict__ exps)
{
    const long j = blockIdx.y;
    if (done && done[j]) return;
    const int e = exps[j];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        x[i + j * ldx] = (accumulate ? x[i + j * ldx] : 0.0) + scalbn((double)y[i + j * ldy], e);
}

// exponent of the largest magnitude of v (0 for zero or non-finite), as FP32 column scales use
__device__ __forceinline__ int column_exp(double v) { return (v > 0.0 && isfinite(v)) ? ilogb(v) : 0; }

// e_j = exponent of max_i |M_ij| (one CTA per column)
__global__ void colmax_exp_kernel(int n, const double *__restrict__ M, long ldm, int *__restrict__ exps)
{
    const long j = blockIdx.x;
    double m = 0.0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(M[i + j * ldm]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
        exps[j] = column_exp(m);
    }
}

// R = B (copy) before the GEMM R -= A X
__global__ void copy_f64_kernel(int n, const double *__restrict__ B, long ldb, double *__restrict__ R, long ldr)
{
    const long j = blockIdx.y;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        R[i + j * ldr] = B[i + j * ldb];
}

// R = B + sum_z P_z, the K-split partials of -A X, added in a fixed order
// (B null: R = -A X, the product the conjugate-gradient steps need)
__global__ void residual_reduce_kernel(int n, int nrhs, int nk, const double *__restrict__ B, long ldb,
                                       const double *__restrict__ P, double *__restrict__ R, long ldr)
{
    const long j = blockIdx.y;
    const long stride = (long)n * nrhs;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double v = B ? B[i + j * ldb] : 0.0;
        for (int z = 0; z < nk; ++z) v += P[z * stride + i + j * (long)n];
        R[i + j * ldr] = v;
    }
}

// K chunks of the residual so that the grid holds enough equal CTAs for the
// hardware scheduler to balance 152 SMs (a few hundred CTAs of equal size
// leave some SMs one CTA behind the others).
static int residual_nk(int n, int nrhs)
{
    const long tiles = (long)((n + 63) / 64) * ((nrhs + 15) / 16);
    long nk = (8192 + tiles - 1) / tiles;
    if (nk > 32) nk = 32;
    if (nk < 1) nk = 1;
    while (nk > 1 && (long)n / nk < 64) --nk;
    return (int)nk;
}

// R = B - A X in FP64 (A n x n, X / B / R n x nrhs), deterministic split-K
static void residual_f64(cudaStream_t s, int n, int nrhs, const double *A, long lda, const double *X, long ldx,
                         const double *B, long ldb, double *R, long ldr, double *partials)
{
    const int nk = residual_nk(n, nrhs);
    const int kchunk = ((n + nk - 1) / nk + 7) / 8 * 8;
    dim3 grid((n + 63) / 64, (nrhs + 15) / 16, nk);
    gb300_count_launch(), gemm_simt_kernel<double, false, false, 64, 16, 8, 4, 2, false>
        <<<grid, 128, 0, s>>>(n, nrhs, n, -1.0, A, lda, X, ldx, 0.0, partials, n, kchunk, (long)n * nrhs);
    const unsigned gx = (unsigned)std::min<long>(((long)n + 255) / 256, 1024);
    gb300_count_launch(), residual_reduce_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, nk, B, ldb, partials, R, ldr);
}

// K chunk of the double-float residual: a multiple of the flush length, with
// enough chunks for ~16 CTAs per SM over the row blocks
static int residual_df_kchunk(int n, int nrhs)
{
    const long tiles = (long)((n + RDF_BM - 1) / RDF_BM) * ((nrhs + 15) / 16);
    long nk = (16 * 152 + tiles - 1) / tiles;
    nk = std::max(1L, std::min(32L, nk));
    const long step = (long)RDF_BK * RDF_FLUSH;
    long kc = ((n + nk - 1) / nk + step - 1) / step * step;
    return (int)std::max(kc, step);
}

// FP64 partials the residual needs, either form
static size_t residual_partials(int n, int nrhs)
{
    const int kc = residual_df_kchunk(n, nrhs);
    const long nz = std::max(1, (n + kc - 1) / kc);
    return (size_t)std::max<long>(residual_nk(n, nrhs), nz) * n * nrhs;
}

// R = B - A X with the double-float product on the FP32 pipe (~2^-47 relative
// per 128-term block, partials reduced in FP64 in a fixed order).  anorm_bits:
// an upper bound of max |A_ij| (||A||_inf) as FP64 bits.  xs: n x 16 * groups
// float2, sx: nrhs ints.
static void residual_df(cudaStream_t s, int n, int nrhs, const double *A, long lda, const double *X, long ldx,
                        const double *B, long ldb, double *R, long ldr, double *partials, float2 *xs, int *sx,
                        const unsigned long long *anorm_bits)
{
    const int kc = residual_df_kchunk(n, nrhs);
    const int nz = (n + kc - 1) / kc;
    gb300_count_launch(), df_split_x_kernel<<<nrhs, 256, 0, s>>>(n, X, ldx, xs, sx);
    dim3 grid((n + RDF_BM - 1) / RDF_BM, (nrhs + 15) / 16, nz);
    gb300_count_launch(), residual_df_kernel<<<grid, 256, 0, s>>>(n, nrhs, A, lda, xs, sx, anorm_bits, kc, partials);
    const unsigned gx = (unsigned)std::min<long>(((long)n + 255) / 256, 1024);
    gb300_count_launch(), residual_reduce_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, nz, B, ldb, partials, R, ldr);
}

// The refinement's residual R = B - A X: the products on the tensor cores in
// exact fixed-point slices (residual_tc), or, with STARPU_GB300_RESIDUAL=df,
// in double-float on the FP32 pipe (residual_df).  The partials are reduced
// in FP64 in a fixed order either way.
// anorm_bits: [0] ||A||_inf, [2] max |A_ij| (the slices' scale), as FP64 bits.
static int residual_mixed(cudaStream_t s, int n, int nrhs, const double *A, long lda, const double *X, long ldx,
                          const double *B, long ldb, double *R, long ldr, double *partials, float2 *xs, int *sx,
                          const void *rtc_a, void *rtc_xs, const unsigned long long *anorm_bits, int *d_err)
{
    static const bool use_df = [] {
        const char *e = getenv("STARPU_GB300_RESIDUAL");
        return e && !strcmp(e, "df");
    }();
    if (use_df) {
        residual_df(s, n, nrhs, A, lda, X, ldx, B, ldb, R, ldr, partials, xs, sx, anorm_bits);
        return gb300_last_launch_status();
    }
    const long cap = (long)(residual_partials(n, nrhs) / ((size_t)n * nrhs));
    const int kc = residual_tc_kchunk(n, nrhs, (int)cap);
    gb300_count_launch(), df_split_x_kernel<<<nrhs, 256, 0, s>>>(n, X, ldx, xs, sx);
    int rc = residual_tc(s, n, nrhs, rtc_a, X, ldx, sx, anorm_bits + 2, kc, rtc_xs, partials, d_err);
    if (rc) return rc;
    const unsigned gx = (unsigned)std::min<long>(((long)n + 255) / 256, 1024);
    gb300_count_launch(), residual_reduce_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, (n + kc - 1) / kc, B, ldb,
                                                                                partials, R, ldr);
    return gb300_last_launch_status();
}

// Per right-hand side j (one CTA): berr_j = ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf);
// done_j = berr_j <= tol.
__global__ void backward_error_kernel(int n, const double *__restrict__ R, long ldr, const double *__restrict__ X,
                                      long ldx, const double *__restrict__ B, long ldb,
                                      const unsigned long long *anorm_bits, double tol, double *berr, int *done,
                                      int *rexp)
{
    const long j = blockIdx.x;
    double rm = 0, xm = 0, bm = 0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        rm = fmax(rm, fabs(R[i + j * ldr]));
        xm = fmax(xm, fabs(X[i + j * ldx]));
        bm = fmax(bm, fabs(B[i + j * ldb]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        rm = fmax(rm, __shfl_down_sync(0xffffffffu, rm, o));
        xm = fmax(xm, __shfl_down_sync(0xffffffffu, xm, o));
        bm = fmax(bm, __shfl_down_sync(0xffffffffu, bm, o));
    }
    __shared__ double s[3][32];
    if ((threadIdx.x & 31) == 0) {
        s[0][threadIdx.x >> 5] = rm;
        s[1][threadIdx.x >> 5] = xm;
        s[2][threadIdx.x >> 5] = bm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            rm = fmax(rm, s[0][w]);
            xm = fmax(xm, s[1][w]);
            bm = fmax(bm, s[2][w]);
        }
        const double an = __longlong_as_double((long long)*anorm_bits);
        const double den = an * xm + bm;
        const double e = den > 0 ? rm / den : (rm > 0 ? INFINITY : 0.0);
        berr[j] = e;
        done[j] = (e <= tol) ? 1 : 0;
        if (rexp) rexp[j] = column_exp(rm);  // scale of the next FP32 correction solve
    }
}

// Sum of v over the CTA in a fixed order (warp trees, then the warps in
// order): deterministic, the same value in every thread.  red: 32 doubles.
__device__ __forceinline__ double block_sum_fixed(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    return s;
}

__device__ __forceinline__ double block_max(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    return m;
}

// Flexible preconditioned conjugate gradients, the refinement used once a
// classic correction has contracted the error slowly (ill-conditioned A).
// One CTA per right-hand side j not yet done.  After the preconditioner
// solve Y = L^-T L^-1 fp32(r 2^-e) with the mixed factor:
//   z = fp64(Y) 2^e,  rz = r.z,  beta = (rz - r.z_prev) / rho   (0 on a restart:
//   Polak-Ribiere, which tolerates the FP32 preconditioner not being exactly
//   the same linear map every time),  p = z + beta p,  z_prev = z,  rho = rz.
__global__ void __launch_bounds__(512) pcg_direction_kernel(int n, const float *__restrict__ Y, long ldy,
                                                            const int *__restrict__ exps, const double *__restrict__ R,
                                                            long ldr, double *__restrict__ Zp, double *__restrict__ P,
                                                            double *__restrict__ rho, const int *__restrict__ done,
                                                            int restart)
{
    const long j = blockIdx.x;
    if (done[j]) return;
    __shared__ double red[32];
    const int e = exps[j];
    const float *y = Y + j * ldy;
    const double *r = R + j * ldr;
    double *zp = Zp + j * (long)n, *p = P + j * (long)n;
    double rz = 0.0, rzp = 0.0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        const double z = scalbn((double)y[i], e);
        rz += r[i] * z;
        if (!restart) rzp += r[i] * zp[i];
    }
    rz = block_sum_fixed(rz, red);
    rzp = block_sum_fixed(rzp, red);
    const double old = rho[j];
    double beta = restart ? 0.0 : (rz - rzp) / old;
    if (!(old > 0.0) || !isfinite(beta)) beta = 0.0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        const double z = scalbn((double)y[i], e);
        p[i] = restart ? z : z + beta * p[i];
        zp[i] = z;
    }
    __syncthreads();
    if (threadIdx.x == 0) rho[j] = rz;
}

// The step along p (Qn = -A p from the residual kernel with no right-hand
// side): alpha = rho / (p^T A p), x += alpha p, r -= alpha A p (the
// recurrence residual), then the backward error of that residual as
// backward_error_kernel computes it.  A direction with p^T A p <= 0 (the
// preconditioned operator lost definiteness in rounding) is not taken and
// *breakdown is set: the host restarts from the true residual.
__global__ void __launch_bounds__(512) pcg_step_kernel(int n, const double *__restrict__ P, const double *__restrict__ Qn,
                                                       const double *__restrict__ rho, double *__restrict__ X, long ldx,
                                                       double *__restrict__ R, long ldr, const double *__restrict__ B,
                                                       long ldb, const unsigned long long *anorm_bits, double tol,
                                                       double *berr, int *done, int *rexp, int *breakdown)
{
    const long j = blockIdx.x;
    if (done[j]) return;
    __shared__ double red[32];
    const double *p = P + j * (long)n, *q = Qn + j * (long)n;
    double *x = X + j * ldx, *r = R + j * ldr;
    const double *b = B + j * ldb;
    double pap = 0.0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) pap -= p[i] * q[i];
    pap = block_sum_fixed(pap, red);
    double alpha = rho[j] / pap;
    if (!(pap > 0.0) || !isfinite(alpha)) {
        alpha = 0.0;
        if (threadIdx.x == 0) *breakdown = 1;
    }
    double rm = 0.0, xm = 0.0, bm = 0.0;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        const double xi = x[i] + alpha * p[i], ri = r[i] + alpha * q[i];
        x[i] = xi;
        r[i] = ri;
        rm = fmax(rm, fabs(ri));
        xm = fmax(xm, fabs(xi));
        bm = fmax(bm, fabs(b[i]));
    }
    rm = block_max(rm, red);
    xm = block_max(xm, red);
    bm = block_max(bm, red);
    if (threadIdx.x == 0) {
        const double an = __longlong_as_double((long long)*anorm_bits);
        const double den = an * xm + bm;
        const double e = den > 0 ? rm / den : (rm > 0 ? INFINITY : 0.0);
        berr[j] = e;
        done[j] = (e <= tol) ? 1 : 0;
        rexp[j] = column_exp(rm);
    }
}

// max_i L_ii^2 / min_i L_ii^2 of the FP32 factor (one CTA): the ratio of the
// largest to the smallest Cholesky pivot, a lower bound of kappa_2(A) (every
// pivot lies between the extreme eigenvalues).
__global__ void pivot_ratio_kernel(int n, const float *__restrict__ W, long ldw, double *ratio)
{
    __shared__ double rmx[32], rmn[32];
    double mx = 0.0, mn = INFINITY;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        const double d = (double)W[i + i * ldw];
        mx = fmax(mx, d * d);
        mn = fmin(mn, d * d);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        mn = fmin(mn, __shfl_down_sync(0xffffffffu, mn, o));
    }
    if ((threadIdx.x & 31) == 0) {
        rmx[threadIdx.x >> 5] = mx;
        rmn[threadIdx.x >> 5] = mn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mx = fmax(mx, rmx[w]);
            mn = fmin(mn, rmn[w]);
        }
        *ratio = mn > 0.0 ? mx / mn : INFINITY;
    }
}

// F (n x n, ld n) = the lower triangle of A, zeros above: the FP64 copy the
// fallback factorisation works on (the strict upper part of A is never read)
__global__ void copy_lower_f64_kernel(int n, const double *__restrict__ A, long lda, double *__restrict__ F)
{
    const long j = blockIdx.x;
    for (long i = threadIdx.x; i < n; i += blockDim.x) F[i + j * n] = i >= j ? A[i + j * lda] : 0.0;
}

struct SolverWs {
    float *W;              // n x n FP32 working factor (ld = n)
    void *panel;           // split panels of the tensor-core factorisation
    double *R;             // n x nrhs FP64 residual
    float *Y;              // n x nrhs FP32 right-hand side / correction
    void *sweep;           // inverted 64 x 64 diagonal blocks + flags of the 64-row POTRS sweeps
    float *band;           // inverses of the nb x nb diagonal tiles (tile T at band + T * ldk * ldk), or null
    float *band_t;         // the same tiles transposed (the backward sweep's operand)
    void *tsw;             // scratch of the tile-row sweeps (tsw_scratch_bytes)
    double *partials;      // K-split partials of the residual
    float2 *xs;            // double-float split of X (n x 16 per group of 16 columns)
    int *sx;               // per-column scale exponents of X
    void *rtc_xs;          // x digit slices of the tensor-core residual
    void *rtc_a;           // the 8 digit slices of A (cut once per matrix, kept with the factor)
    float *rowsum;         // n/64 x n row sums of the slicing pass, for ||A||_inf
    double *berr;          // nrhs
    int *done;             // nrhs
    double *P, *Qn, *Zp;   // n x nrhs each: direction, -A p and the previous z of the conjugate-gradient steps
    double *rho;           // nrhs: r.z of the conjugate-gradient steps
    int *brk;              // breakdown word of the conjugate-gradient steps
    int *rexp;             // nrhs: power-of-two scales of the FP32 right-hand sides
    unsigned long long *anorm_bits;
    int *info, *err;
    size_t panel_bytes;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The tile-row sweeps need the factorisation's diagonal-tile inverses (tiles
// of order <= 1024 inverted by the cooperative diagonal kernel) and slabs of
// 32 rows that tile each nb x nb tile.
static bool tile_sweep_ok(int nb) { return nb > 0 && nb % TSW_SLAB == 0 && nb <= GB300_DIAG_TILE_MAX; }

// L y = b then L^T x = y with the inverted nb x nb diagonal tiles in `band`
// (ld ldk, tile T at band + T * ldk * ldk; band_t, optional: the same tiles
// transposed): one persistent launch per sweep and group of 16 right-hand
// sides.  scratch: tsw_scratch_bytes(n, nb).
static void tile_sweeps(cudaStream_t s, int n, int nrhs, int nb, const float *L, long ldl, const float *band, long ldk,
                        float *Y, long ldy, void *scratch, int *err, int upper = 0, const float *band_t = nullptr)
{
    if (n <= 0 || nrhs <= 0) return;
    TileSweepArgs a;
    a.n = n;
    a.nb = nb;
    a.ntiles = (n + nb - 1) / nb;
    a.spt = nb / TSW_SLAB;
    a.total = (unsigned)((size_t)a.spt * a.ntiles * (a.ntiles + 1) / 2);
    size_t yt_off = 0, zp_off = 0, cnt_off = 0;
    tsw_scratch_bytes(n, nb, &yt_off, &zp_off, &cnt_off);
    a.L = L;
    a.ldl = ldl;
    a.Dinv = band;
    a.DinvT = band_t;
    a.ldd = ldk;
    a.dstride = ldk * ldk;
    a.ldb = ldy;
    a.Zt = (float *)scratch;
    a.Yt = (float *)((char *)scratch + yt_off);
    a.Zp = (float *)((char *)scratch + zp_off);
    int *cnt = (int *)((char *)scratch + cnt_off);
    a.zcount = cnt;
    a.ycount = cnt + a.ntiles;
    a.pcount = cnt + 2 * a.ntiles;
    a.ticket = (unsigned *)(cnt + 3 * a.ntiles);
    a.err = err;
    a.upper = upper;
    a.budget_ns = gb300_wait_budget_ns();
    // persistent CTAs: as many as fit on the device, and at least one per slab
    // of a tile row (the diagonal tasks of a tile row wait for one another)
    const void *fns[3] = {(const void *)tile_sweep_kernel<false, false>, (const void *)tile_sweep_kernel<true, false>,
                          (const void *)tile_sweep_kernel<true, true>};
    static thread_local int per_sm[16][3];
    int dev = 0;
    cudaGetDevice(&dev);
    int *per = per_sm[dev & 15];
    if (!per[0]) {
        // the table is filled only once all three kernels are set up
        int occ[3];
        for (int i = 0; i < 3; ++i) {
            if (gb300_func_dyn_smem(fns[i], TSW_DSMEM) ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[i], fns[i], TSW_T, TSW_DSMEM) != cudaSuccess) {
                // the kernels cannot run on this device: report it in the error word
                if (err) cudaMemsetAsync(err, 1, 1, s);
                return;
            }
        }
        for (int i = 2; i >= 0; --i) per[i] = std::max(occ[i], 1);
    }
    const int sms = gb300_device_sms();
    auto grid = [&](int which) {
        const long g = std::min<long>((long)a.total, (long)per[which] * sms);
        return (unsigned)std::max<long>(g, a.spt);
    };
    auto al = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    const bool vec = al(L) && al(band) && (!band_t || al(band_t)) && ldl % 4 == 0 && ldk % 4 == 0;
    const size_t cbytes = (3 * (size_t)a.ntiles + 1) * sizeof(int);
    for (int c0 = 0; c0 < nrhs; c0 += 16) {
        a.nrhs = std::min(16, nrhs - c0);
        a.B = Y + (long)c0 * ldy;
        a.vec = vec;
        cudaMemsetAsync(cnt, 0, cbytes, s);
        gb300_count_launch(), tile_sweep_kernel<false, false><<<grid(0), TSW_T, TSW_DSMEM, s>>>(a);
        cudaMemsetAsync(cnt, 0, cbytes, s);
        if (upper) gb300_count_launch(), tile_sweep_kernel<true, true><<<grid(2), TSW_T, TSW_DSMEM, s>>>(a);
        else gb300_count_launch(), tile_sweep_kernel<true, false><<<grid(1), TSW_T, TSW_DSMEM, s>>>(a);
    }
}

// band_t = the nb x nb tiles of band transposed (ld ldk each, ntiles tiles),
// for the backward sweep's direct reads; 32 x 32 blocks through shared memory
__global__ void transpose_tiles_kernel(int ldk, const float *__restrict__ band, float *__restrict__ band_t)
{
    __shared__ float t[32][33];
    const long base = (long)blockIdx.z * ldk * ldk;
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) t[y][threadIdx.x] = band[base + r0 + threadIdx.x + (long)(c0 + y) * ldk];
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y)
        band_t[base + c0 + threadIdx.x + (long)(r0 + y) * ldk] = t[threadIdx.x][y];
}

static size_t layout(int n, int nrhs, int nb, void *base, SolverWs *ws)
{
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    // what the factor phase leaves behind comes first and does not depend on
    // nrhs, so a kept factor can be refined later with any nrhs up to the
    // workspace's capacity
    const size_t oW = take((size_t)n * n * sizeof(float));
    const size_t panel_bytes = starpu_gb300_spotrf_tc_workspace(n, nb);
    const size_t oP = take(panel_bytes);
    const size_t oT = take(potrs_sweep_workspace<float>(n));
    const bool tiles = tile_sweep_ok(nb);
    const size_t ldk = ((size_t)(nb > 0 ? nb : 1) + 63) / 64 * 64, ntiles = nb > 0 ? ((size_t)n + nb - 1) / nb : 0;
    const size_t oB = tiles ? take(2 * ntiles * ldk * ldk * sizeof(float)) : 0;
    const size_t oZ = tiles ? take(tsw_scratch_bytes(n, nb)) : 0;
    const size_t oA = take(residual_tc_a_bytes(n));
    const size_t oN = take((size_t)((n + 63) / 64) * n * sizeof(float));
    const size_t oS = take(4 * sizeof(unsigned long long));
    const size_t oR = take((size_t)n * nrhs * sizeof(double));
    const size_t oY = take((size_t)n * nrhs * sizeof(float));
    const size_t oE = take((size_t)nrhs * sizeof(double));
    const size_t oD = take((size_t)nrhs * sizeof(int));
    const size_t oQ = take(residual_partials(n, nrhs) * sizeof(double));
    const size_t oX = take((size_t)n * 16 * ((nrhs + 15) / 16) * sizeof(float2));
    const size_t oI = take((size_t)nrhs * sizeof(int));
    const size_t oJ = take((size_t)nrhs * sizeof(int));
    const size_t oK = take(residual_tc_xs_bytes(n, nrhs));
    const size_t oG = take(3 * (size_t)n * nrhs * sizeof(double));
    const size_t oH = take((size_t)nrhs * sizeof(double) + 16);
    if (ws && base) {
        char *b = (char *)base;
        ws->W = (float *)(b + oW);
        ws->panel = b + oP;
        ws->panel_bytes = panel_bytes;
        ws->R = (double *)(b + oR);
        ws->Y = (float *)(b + oY);
        ws->sweep = b + oT;
        ws->band = tiles ? (float *)(b + oB) : nullptr;
        ws->band_t = tiles ? ws->band + ntiles * ldk * ldk : nullptr;
        ws->tsw = tiles ? (void *)(b + oZ) : nullptr;
        ws->rtc_a = b + oA;
        ws->rowsum = (float *)(b + oN);
        ws->partials = (double *)(b + oQ);
        ws->xs = (float2 *)(b + oX);
        ws->sx = (int *)(b + oI);
        ws->rexp = (int *)(b + oJ);
        ws->rtc_xs = b + oK;
        ws->berr = (double *)(b + oE);
        ws->P = (double *)(b + oG);
        ws->Qn = ws->P + (size_t)n * nrhs;
        ws->Zp = ws->Qn + (size_t)n * nrhs;
        ws->rho = (double *)(b + oH);
        ws->brk = (int *)(ws->rho + nrhs);
        ws->done = (int *)(b + oD);
        ws->anorm_bits = (unsigned long long *)(b + oS);
        ws->info = (int *)(b + oS + 8);
        ws->err = (int *)(b + oS + 12);  // read back together with info
    }
    return off;
}


// y <- L^-T L^-1 y with the FP32 factor W: tile-row sweeps when the
// factorisation kept its diagonal-tile inverses, else 64-row sweeps.
static void correction_solve(cudaStream_t s, int n, int nrhs, int nb, const SolverWs &ws)
{
    const long ldk = ((long)nb + 63) / 64 * 64;
    // the factor phase mirrors L^T into W's strictly upper part (outside the diagonal tiles)
    if (ws.band) tile_sweeps(s, n, nrhs, nb, ws.W, n, ws.band, ldk, ws.Y, n, ws.tsw, ws.err, 1, ws.band_t);
    else potrs_sweep<float>(s, n, nrhs, ws.W, n, ws.sweep, ws.Y, n, ws.err);
}

// Streams and fork / join event pairs per host thread and device.  The
// factor phase runs the factorisation of W on a high-priority stream and the
// passes that only read A (the residual's digit slices, the infinity norm) on
// a lowest-priority side stream: the side work then takes only the SMs the
// factorisation leaves idle (its diagonal tiles are latency-bound) instead of
// holding the GPU while the first diagonal tile waits.
struct SideStream {
    int dev = -1;
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~SideStream()
    {
        if (s) cudaStreamDestroy(s);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
    }
};

// which = 0: the lowest-priority side stream of the slicing; 1: the
// factorisation's stream, one priority level below the top (the top is kept
// for the trailing updates that run beside a panel); 2: the lowest-priority
// stream that mirrors each finished column block of L into W's upper part
static SideStream *aux_stream(int which)
{
    thread_local SideStream ss[3][16];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return nullptr;
    SideStream &x = ss[which][dev];
    if (!x.s) {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        const int prio = which == 1 ? std::min(least, greatest + 1) : least;
        if (cudaStreamCreateWithPriority(&x.s, cudaStreamNonBlocking, prio) != cudaSuccess ||
            cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        x.dev = dev;
    }
    return &x;
}

// Rows of the trailing triangle below which the slicing of A starts beside
// the factorisation (GB300_SLICE_ROWS; default n/2, measured at n = 32768:
// from the first step 77.3 ms per solve, from 16384 rows 76.8, from 10240
// 76.7, from 6144 78.1, after the factorisation 80.3).
static int slice_rows(int n)
{
    static int v = -2;
    if (v == -2) {
        const char *e = getenv("GB300_SLICE_ROWS");
        v = e && *e ? atoi(e) : -1;
    }
    return v < 0 ? n / 2 : v;
}

// prepared: W and max |A_ij| were written while A was gathered from the host
// (gather_convert_kernel), the first pass is skipped
static int factor_phase(cudaStream_t s, int n, int nb, int nterms, const double *A, int lda, const SolverWs &ws,
                        bool prepared, const TcArrival *arr = nullptr)
{
    // columns arriving over time: the passes over all of A wait for the last superblock
    cudaEvent_t all_in = arr && arr->nsb > 0 ? arr->ready[arr->nsb - 1] : nullptr;
    // anorm_bits[0] = ||A||_inf, [1] = info + err, [2] = max |A_ij|
    // the first column block is converted first; the rest converts beside the
    // first panel, which reads nothing else, and the factorisation waits for
    // it before its first update
    const int first = std::min(n, nb);
    if (!prepared) {
        cudaMemsetAsync(ws.anorm_bits, 0, 4 * sizeof(unsigned long long), s);
        gb300_count_launch(), convert_lower_max_kernel<<<first, 256, 0, s>>>(n, A, lda, ws.W, n, ws.anorm_bits + 2);
    }
    // the residuals' slices of A and ||A||_inf, beside the factorisation: on
    // the lowest-priority side stream, started once the factorisation's steps
    // become bound by their diagonal tiles (trailing triangles of at most
    // slice_rows rows) and leave most of the GPU idle
    SideStream *ss = aux_stream(0), *fs = aux_stream(1), *ms = aux_stream(2);
    if (!ss || !fs || !ms) return gb300_record_cuda_error(cudaGetLastError());
    cudaEventRecord(fs->fork, s);
    cudaStreamWaitEvent(fs->s, fs->fork, 0);
    cudaEvent_t converted = nullptr;
    if (!prepared && n > first) {
        cudaStreamWaitEvent(ss->s, fs->fork, 0);
        gb300_count_launch(), convert_lower_max_kernel<<<n - first, 256, 0, ss->s>>>(n, A, lda, ws.W, n,
                                                                                   ws.anorm_bits + 2, first);
        cudaEventRecord(ss->join, ss->s);
        converted = ss->join;
    }
    int side_rc = 0;
    auto slice = [&](cudaStream_t from) {
        cudaEventRecord(ss->fork, from);
        cudaStreamWaitEvent(ss->s, ss->fork, 0);
        if (all_in) cudaStreamWaitEvent(ss->s, all_in, 0);
        side_rc = residual_tc_slice_a(ss->s, n, A, lda, ws.anorm_bits + 2, ws.rtc_a, ws.rowsum);
        gb300_count_launch(), norm_from_rowsums_kernel<<<(n + 255) / 256, 256, 0, ss->s>>>(
            n, (n + 63) / 64, ws.rowsum, ws.anorm_bits + 2, ws.anorm_bits);
        cudaEventRecord(ss->join, ss->s);
    };
    // each finished column block of L mirrored into W's upper part, for the backward sweeps
    bool mirrored = false;
    auto mirror = [&](cudaStream_t from, int c0, int w) {
        const int r0 = c0 + w;
        if (!ws.band || r0 >= n) return;
        cudaEventRecord(ms->fork, from);
        cudaStreamWaitEvent(ms->s, ms->fork, 0);
        const dim3 g((unsigned)((n - r0 + 31) / 32), (unsigned)((w + 31) / 32));
        gb300_count_launch(), mirror_block_kernel<<<g, dim3(32, 8), 0, ms->s>>>(n, c0, w, r0, ws.W, n);
        mirrored = true;
    };
    int rc = potrf_tc(fs->s, n, ws.W, n, nb, nterms, ws.panel, ws.info, ws.err, ws.band, slice, slice_rows(n),
                      mirror, converted, arr);
    if (all_in) cudaStreamWaitEvent(s, all_in, 0);
    if (!rc) rc = side_rc;
    if (mirrored) {
        cudaEventRecord(ms->join, ms->s);
        cudaStreamWaitEvent(s, ms->join, 0);
    }
    cudaEventRecord(fs->join, fs->s);
    cudaStreamWaitEvent(s, fs->join, 0);
    cudaStreamWaitEvent(s, ss->join, 0);  // joined before anything reads the factor, the slices or the norm
    if (rc) return rc;
    if (!ws.band) potrs_sweep_prepare<float>(s, n, ws.W, n, ws.sweep);
    else {
        const long ldk = ((long)nb + 63) / 64 * 64;
        const unsigned nt = (unsigned)((n + nb - 1) / nb), bt = (unsigned)(ldk / 32);
        gb300_count_launch(), transpose_tiles_kernel<<<dim3(bt, bt, nt), dim3(32, 8), 0, s>>>((int)ldk, ws.band,
                                                                                            ws.band_t);
    }
    return gb300_last_launch_status();
}

// Factor phase of the mixed solve: W = fp32(A) (lower) with ||A||_inf, the
// tensor-core tiled Cholesky of W and the inverted diagonal blocks the POTRS
// sweeps use.  Synchronises once to read the factorisation status.  The
// workspace then holds everything a later refine phase needs, so a factor can
// be kept on the device and reused for new right-hand sides.
void dsposv_prepared_targets(int n, int nrhs, int nb, void *work, float **W, unsigned long long **amax_block)
{
    SolverWs ws;
    layout(n, nrhs, nb, work, &ws);
    *W = ws.W;
    *amax_block = ws.anorm_bits;
}

int dsposv_factor(cudaStream_t s, int n, int nrhs, const double *A, int lda, int nb, int nterms, void *work,
                  starpu_gb300_ir_info *out, bool prepared, const TcArrival *arr)
{
    SolverWs ws;
    layout(n, nrhs, nb, work, &ws);
    int rc = factor_phase(s, n, nb, nterms, A, lda, ws, prepared, arr);
    int hinfo[2] = {0, 0};
    if (!rc) rc = gb300_record_cuda_error(cudaMemcpyAsync(hinfo, ws.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (!rc) rc = gb300_record_cuda_error(cudaStreamSynchronize(s));
    if (rc) return rc;
    if (out) {
        out->potrf_info = hinfo[0];
        out->factor_terms = nterms;
    }
    if (hinfo[1]) {
        if (out) out->status = GB300_ETIMEDOUT;
        return GB300_ETIMEDOUT;
    }
    if (hinfo[0]) {
        if (out) out->status = GB300_EDOM;
        return GB300_EDOM;
    }
    return GB300_OK;
}

// How the refinement proceeds (STARPU_GB300_REFINE, or
// starpu_gb300_dsposv_set_refinement): 0 classic corrections only ("ir"),
// 1 conjugate gradients from the first correction on ("pcg"), 2 (default)
// classic corrections until one contracts the backward error by less than
// PCG_SWITCH, then conjugate gradients.
static std::atomic<int> g_refine{-1};
static int refine_mode()
{
    int m = g_refine.load(std::memory_order_relaxed);
    if (m >= 0) return m;
    const char *e = getenv("STARPU_GB300_REFINE");
    m = (e && !strcmp(e, "ir")) ? 0 : (e && !strcmp(e, "pcg")) ? 1 : 2;
    int expect = -1;
    g_refine.compare_exchange_strong(expect, m);
    return g_refine.load(std::memory_order_relaxed);
}
// A classic correction that leaves more than this fraction of the backward
// error marks an ill-conditioned system (kappa times the factor's error near
// 1e-1): from there conjugate gradients with the same factor as
// preconditioner contract the error faster per correction.
static constexpr double PCG_SWITCH = 0.05;
// A pivot ratio above this (kappa at least that large; on the Gram test
// matrices the ratio is ~0.6 sqrt(kappa)) starts with conjugate gradients:
// the classic correction it would replace is known to contract slowly.
static constexpr double PCG_PIVOT_RATIO = 300.0;
// corrections without halving the best backward error seen: stalled
static constexpr int STALL_STEPS = 6;

// Refine phase: x = L^-T L^-1 b in FP32, then FP64 refinement with the factor
// left in the workspace by dsposv_factor (for the same A): classic
// corrections x += L^-T L^-1 r, switching to flexible preconditioned
// conjugate gradients (preconditioner L L^T, FP64 vectors, the recurrence
// residual checked against a true residual before it is accepted) when the
// corrections contract slowly.  *stalled (optional): set when the refinement
// stopped without converging (max_iter corrections, or no progress) -- the
// case in which LAPACK dsposv falls back to the FP64 factorisation.
int dsposv_refine(cudaStream_t s, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                  int ldx, int nb, double tol, int max_iter, void *work, starpu_gb300_ir_info *out, bool *stalled)
{
    SolverWs ws;
    layout(n, nrhs, nb, work, &ws);
    if (stalled) *stalled = false;
    const unsigned gx = (unsigned)std::min<long>(((long)n + 255) / 256, 1024);
    cudaMemsetAsync(ws.done, 0, nrhs * sizeof(int), s);
    cudaMemsetAsync(ws.err, 0, sizeof(int), s);
    cudaMemsetAsync(ws.brk, 0, sizeof(int), s);
    gb300_count_launch(), colmax_exp_kernel<<<nrhs, 256, 0, s>>>(n, B, ldb, ws.rexp);
    gb300_count_launch(), to_f32_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, B, ldb, ws.Y, n, ws.rexp);
    int slot = gb300_prof_begin(s, GB300_PROF_SOLVE);
    correction_solve(s, n, nrhs, nb, ws);
    gb300_prof_end(s, slot, 2.0 * n * (double)n * nrhs, 4.0 * n * (double)n);
    gb300_count_launch(), accumulate_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, ws.Y, n, X, ldx, 0, nullptr,
                                                                           ws.rexp);
    double *hberr = (double *)malloc(sizeof(double) * (size_t)nrhs);
    int status = GB300_ETIMEDOUT;
    int it = 0, rc = 0;
    const int mode = refine_mode();
    bool pcg = false, restart = true, true_residual = true;
    double hratio = 0.0;
    if (mode == 2) {  // the factor's pivot ratio, read with the first backward error
        gb300_count_launch(), pivot_ratio_kernel<<<1, 1024, 0, s>>>(n, ws.W, n, ws.rho);
        cudaMemcpyAsync(&hratio, ws.rho, sizeof(double), cudaMemcpyDeviceToHost, s);
    }
    double worst = INFINITY, prev = INFINITY, best = INFINITY;
    int since_best = 0;
    // read the backward errors (and the wait-timeout word) of the step just queued
    auto read_berr = [&](int *herr, int *hbreak) -> int {
        int r = gb300_record_cuda_error(cudaMemcpyAsync(hberr, ws.berr, sizeof(double) * nrhs,
                                                        cudaMemcpyDeviceToHost, s));
        if (!r) r = gb300_record_cuda_error(cudaMemcpyAsync(herr, ws.err, sizeof(int), cudaMemcpyDeviceToHost, s));
        if (!r) r = gb300_record_cuda_error(cudaMemcpyAsync(hbreak, ws.brk, sizeof(int), cudaMemcpyDeviceToHost, s));
        if (!r) r = gb300_record_cuda_error(cudaStreamSynchronize(s));
        worst = 0;
        for (int j = 0; j < nrhs; ++j) worst = fmax(worst, hberr[j]);
        return r;
    };
    for (;;) {
        int herr = 0, hbreak = 0;
        if (true_residual) {
            // r = b - A x, its backward error; every column's done flag from it
            slot = gb300_prof_begin(s, GB300_PROF_RESIDUAL);
            if ((rc = residual_mixed(s, n, nrhs, A, lda, X, ldx, B, ldb, ws.R, n, ws.partials, ws.xs, ws.sx,
                                     ws.rtc_a, ws.rtc_xs, ws.anorm_bits, ws.err)))
                break;
            gb300_prof_end(s, slot, 2.0 * n * (double)n * nrhs, 8.0 * n * (double)n + 32.0 * n * nrhs);
            gb300_count_launch(), backward_error_kernel<<<nrhs, 256, 0, s>>>(n, ws.R, n, X, ldx, B, ldb,
                                                                             ws.anorm_bits, tol, ws.berr, ws.done,
                                                                             ws.rexp);
            if ((rc = read_berr(&herr, &hbreak))) break;
            if (herr) {  // a wait that ran out in a sweep or a residual invalidates the iteration
                status = GB300_ETIMEDOUT;
                break;
            }
            if (worst <= tol) {
                status = GB300_OK;
                break;
            }
            if (pcg) restart = true;  // the recurrence residual had drifted: start again from the true one
            else if (mode == 1 || (mode == 2 && it >= 1 && worst > PCG_SWITCH * prev) ||
                     (mode == 2 && it == 0 && hratio > PCG_PIVOT_RATIO))
                pcg = true;
        }
        if (worst < 0.5 * best) {
            best = worst;
            since_best = 0;
        } else if (++since_best >= STALL_STEPS) {
            if (stalled) *stalled = true;
            break;
        }
        if (it >= max_iter) {
            if (stalled) *stalled = true;
            break;
        }
        prev = worst;
        // the preconditioner / correction solve on the scaled residual
        gb300_count_launch(), to_f32_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, ws.R, n, ws.Y, n, ws.rexp);
        slot = gb300_prof_begin(s, GB300_PROF_SOLVE);
        correction_solve(s, n, nrhs, nb, ws);
        gb300_prof_end(s, slot, 2.0 * n * (double)n * nrhs, 4.0 * n * (double)n);
        ++it;
        if (!pcg) {
            gb300_count_launch(), accumulate_kernel<<<dim3(gx, nrhs), 256, 0, s>>>(n, nrhs, ws.Y, n, X, ldx, 1,
                                                                                   ws.done, ws.rexp);
            true_residual = true;
            continue;
        }
        // conjugate-gradient step: direction, -A p, step and the recurrence residual's backward error
        gb300_count_launch(), pcg_direction_kernel<<<nrhs, 512, 0, s>>>(n, ws.Y, n, ws.rexp, ws.R, n, ws.Zp, ws.P,
                                                                        ws.rho, ws.done, restart ? 1 : 0);
        restart = false;
        slot = gb300_prof_begin(s, GB300_PROF_RESIDUAL);
        if ((rc = residual_mixed(s, n, nrhs, A, lda, ws.P, n, nullptr, 0, ws.Qn, n, ws.partials, ws.xs, ws.sx,
                                 ws.rtc_a, ws.rtc_xs, ws.anorm_bits, ws.err)))
            break;
        gb300_prof_end(s, slot, 2.0 * n * (double)n * nrhs, 8.0 * n * (double)n + 32.0 * n * nrhs);
        gb300_count_launch(), pcg_step_kernel<<<nrhs, 512, 0, s>>>(n, ws.P, ws.Qn, ws.rho, X, ldx, ws.R, n, B, ldb,
                                                                   ws.anorm_bits, tol, ws.berr, ws.done, ws.rexp,
                                                                   ws.brk);
        if ((rc = read_berr(&herr, &hbreak))) break;
        if (herr) {
            status = GB300_ETIMEDOUT;
            break;
        }
        // accepted only after a true residual agrees; a breakdown restarts from one
        true_residual = worst <= tol || hbreak;
        if (hbreak) cudaMemsetAsync(ws.brk, 0, sizeof(int), s);
    }
    free(hberr);
    if (rc) return rc;
    if (out) {
        out->iterations = it;
        out->backward_error = worst;
        out->status = status;
        out->method = pcg ? 1 : 0;
        unsigned long long ab = 0;
        cudaMemcpyAsync(&ab, ws.anorm_bits, sizeof ab, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        double an;
        memcpy(&an, &ab, sizeof an);
        out->anorm = an;
    }
    return status;
}

// LAPACK dsposv's fallback (ITER < 0): the FP64 tiled Cholesky of A on the GPU
// and its two triangular solves, when the mixed factorisation failed or its
// refinement did not converge.  The FP64 factor takes the place of the
// residual's digit slices in the workspace (16 n ldk bytes >= 8 n^2), which
// are cut again from A afterwards for the backward error; the FP32 factor in
// the workspace is not valid after a fallback.
int dsposv_fp64(cudaStream_t s, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                int ldx, int nb, double tol, void *work, starpu_gb300_ir_info *out)
{
    SolverWs ws;
    layout(n, nrhs, nb, work, &ws);
    double *F = (double *)ws.rtc_a;
    gb300_count_launch(), copy_lower_f64_kernel<<<n, 256, 0, s>>>(n, A, lda, F);
    int rc = gb300_record_cuda_error(cudaMemcpy2DAsync(X, sizeof(double) * ldx, B, sizeof(double) * ldb,
                                                       sizeof(double) * n, nrhs, cudaMemcpyDeviceToDevice, s));
    if (!rc) rc = starpu_gb300_dpotrf(s, n, F, n, nb, ws.info);
    int hinfo = 0;
    if (!rc) rc = gb300_record_cuda_error(cudaMemcpyAsync(&hinfo, ws.info, sizeof hinfo, cudaMemcpyDeviceToHost, s));
    if (!rc) rc = gb300_record_cuda_error(cudaStreamSynchronize(s));
    if (rc) return rc;
    if (out) out->potrf_info = hinfo;
    if (hinfo) {
        if (out) out->status = GB300_EDOM;
        return GB300_EDOM;
    }
    if ((rc = starpu_gb300_dpotrs(s, n, nrhs, F, n, X, ldx))) return rc;
    // the factor is no longer needed: A is cut into its digit slices again
    // (max |A_ij| and ||A||_inf from the lower triangle on the way) and
    // r = b - A x is formed as the refinement forms it
    cudaMemsetAsync(ws.anorm_bits, 0, 4 * sizeof(unsigned long long), s);
    gb300_count_launch(), convert_lower_max_kernel<<<n, 256, 0, s>>>(n, A, lda, nullptr, 0, ws.anorm_bits + 2);
    if ((rc = residual_tc_slice_a(s, n, A, lda, ws.anorm_bits + 2, ws.rtc_a, ws.rowsum))) return rc;
    gb300_count_launch(), norm_from_rowsums_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, (n + 63) / 64, ws.rowsum,
                                                                                  ws.anorm_bits + 2, ws.anorm_bits);
    if ((rc = residual_mixed(s, n, nrhs, A, lda, X, ldx, B, ldb, ws.R, n, ws.partials, ws.xs, ws.sx, ws.rtc_a,
                             ws.rtc_xs, ws.anorm_bits, ws.err)))
        return rc;
    gb300_count_launch(), backward_error_kernel<<<nrhs, 256, 0, s>>>(n, ws.R, n, X, ldx, B, ldb, ws.anorm_bits, tol,
                                                                     ws.berr, ws.done, nullptr);
    std::vector<double> hb((size_t)nrhs);
    unsigned long long ab = 0;
    rc = gb300_record_cuda_error(cudaMemcpyAsync(hb.data(), ws.berr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    if (!rc) rc = gb300_record_cuda_error(cudaMemcpyAsync(&ab, ws.anorm_bits, sizeof ab, cudaMemcpyDeviceToHost, s));
    if (!rc) rc = gb300_record_cuda_error(cudaStreamSynchronize(s));
    if (rc) return rc;
    double worst = 0;
    for (double v : hb) worst = fmax(worst, v);
    const int status = worst <= tol ? GB300_OK : GB300_ETIMEDOUT;
    if (out) {
        out->backward_error = worst;
        memcpy(&out->anorm, &ab, sizeof ab);
        out->status = status;
    }
    return status;
}

// The ladder of one mixed solve: the factor and its refinement, then LAPACK's
// FP64 fallback when the factor failed (GB300_EDOM: fallback 1, ITER = -3) or
// the refinement stalled (fallback 2, ITER = -31).  STARPU_GB300_FP64_FALLBACK=0
// turns the fallback off (the mixed outcome is returned as it is).
static std::atomic<int> g_fallback{-1};
static bool fp64_fallback_enabled()
{
    int f = g_fallback.load(std::memory_order_relaxed);
    if (f < 0) {
        const char *e = getenv("STARPU_GB300_FP64_FALLBACK");
        int expect = -1;
        g_fallback.compare_exchange_strong(expect, (e && !strcmp(e, "0")) ? 0 : 1);
        f = g_fallback.load(std::memory_order_relaxed);
    }
    return f != 0;
}

int dsposv_ladder(cudaStream_t s, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                  int ldx, int nb, int nterms, double tol, int max_iter, void *work, starpu_gb300_ir_info *out,
                  bool prepared, const TcArrival *arr)
{
    int rc = dsposv_factor(s, n, nrhs, A, lda, nb, nterms, work, out, prepared, arr);
    int reason = 0;
    if (rc == GB300_EDOM) reason = 1;
    else if (rc) return rc;
    if (!reason) {
        bool stalled = false;
        rc = dsposv_refine(s, n, nrhs, A, lda, B, ldb, X, ldx, nb, tol, max_iter, work, out, &stalled);
        if (rc != GB300_ETIMEDOUT || !stalled) return rc;
        reason = 2;
    }
    if (!fp64_fallback_enabled()) return rc;
    if (out) out->fallback = reason;
    return dsposv_fp64(s, n, nrhs, A, lda, B, ldb, X, ldx, nb, tol, work, out);
}

} // namespace gb300

using namespace gb300;

extern "C" {

int starpu_gb300_dsposv_set_refinement(int mode)
{
    const int prev = refine_mode();
    if (mode >= 0 && mode <= 2) g_refine.store(mode);
    return prev;
}

int starpu_gb300_dsposv_set_fp64_fallback(int on)
{
    const int prev = fp64_fallback_enabled() ? 1 : 0;
    if (on >= 0) g_fallback.store(on ? 1 : 0);
    return prev;
}

size_t starpu_gb300_dsposv_workspace(int n, int nrhs, int nb)
{
    if (n < 0 || nrhs < 0) return 0;
    if (nb <= 0) nb = 1024;
    return layout(n, nrhs, nb, nullptr, nullptr);
}

int starpu_gb300_dsposv(void *stream, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                        int ldx, int nb, int nterms, double tol, int max_iter, void *work, size_t lwork,
                        starpu_gb300_ir_info *out)
{
    if (out) memset(out, 0, sizeof *out);
    if (n < 0 || nrhs < 0 || lda < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1) || ldx < (n > 1 ? n : 1) ||
        (nterms != 1 && nterms != 3) || max_iter < 0 || !(tol >= 0))
        return GB300_EINVAL;
    if (nb <= 0) nb = 1024;
    if (!work || lwork < starpu_gb300_dsposv_workspace(n, nrhs, nb)) return GB300_EINVAL;
    if (!n || !nrhs) return GB300_OK;
    return gb300::dsposv_ladder((cudaStream_t)stream, n, nrhs, A, lda, B, ldb, X, ldx, nb, nterms, tol, max_iter,
                                work, out, false);
}

// ---- persistent solver context: device buffers sized once, host-buffer calls

struct starpu_gb300_solver {
    int n_max, nrhs_max, nb, nterms;
    cudaStream_t stream;
    double *A, *B, *X;
    void *work;
    size_t lwork;
    // the pinned-input path's overlap of the host link with the factorisation:
    // a copy stream, one event per superblock, every step's split panel, the diagonal
    cudaStream_t copy = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> ready;
    void *panels = nullptr;
    float *diag = nullptr;
    bool overlap_failed = false;
    int overlap = -1;  // -1: STARPU_GB300_HOST_OVERLAP decides
};

starpu_gb300_solver *starpu_gb300_solver_create(int n_max, int nrhs_max, int nb, int nterms)
{
    if (n_max <= 0 || nrhs_max <= 0 || (nterms != 1 && nterms != 3)) return nullptr;
    starpu_gb300_solver *h = new starpu_gb300_solver();
    h->n_max = n_max;
    h->nrhs_max = nrhs_max;
    h->nb = nb > 0 ? nb : 1024;
    h->nterms = nterms;
    h->lwork = starpu_gb300_dsposv_workspace(n_max, nrhs_max, h->nb);
    bool ok = gb300_record_cuda_error(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) == GB300_OK &&
              gb300_record_cuda_error(cudaMalloc(&h->A, sizeof(double) * (size_t)n_max * n_max)) == GB300_OK &&
              gb300_record_cuda_error(cudaMalloc(&h->B, sizeof(double) * (size_t)n_max * nrhs_max)) == GB300_OK &&
              gb300_record_cuda_error(cudaMalloc(&h->X, sizeof(double) * (size_t)n_max * nrhs_max)) == GB300_OK &&
              gb300_record_cuda_error(cudaMalloc(&h->work, h->lwork)) == GB300_OK;
    if (!ok) {
        starpu_gb300_solver_destroy(h);
        return nullptr;
    }
    return h;
}

int starpu_gb300_solver_destroy(starpu_gb300_solver *h)
{
    if (!h) return GB300_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy) cudaStreamSynchronize(h->copy);
    cudaFree(h->A);
    cudaFree(h->B);
    cudaFree(h->X);
    cudaFree(h->work);
    cudaFree(h->panels);
    cudaFree(h->diag);
    for (cudaEvent_t e : h->ready) cudaEventDestroy(e);
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->copy) cudaStreamDestroy(h->copy);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GB300_OK;
}

void *starpu_gb300_solver_stream(starpu_gb300_solver *h) { return h ? (void *)h->stream : nullptr; }

int starpu_gb300_solver_host_overlap(starpu_gb300_solver *h, int on)
{
    if (!h) return GB300_EINVAL;
    const int prev = h->overlap;
    if (on >= 0) h->overlap = on ? 1 : 0;
    return prev;
}

// column panel width of the host-to-device copy of A's lower triangle
static constexpr int HOST_PANEL = 512;

// Column j of the lower triangle (rows j..n-1) from host memory the device
// can read (pinned, mapped), fused with the factor phase's first pass: into
// D (FP64) and W (FP32), and
// the integer max of |A_ij|'s bit patterns into *amax_bits -- what
// convert_lower_max_kernel computes -- so the host path reads A over the link
// once and the factor phase skips its own conversion.  16-byte loads, four in
// flight per thread.
__device__ __forceinline__ void gather_convert_column(int n, const double *__restrict__ H, long ldh,
                                                      double *__restrict__ D, long ldd, float *__restrict__ W,
                                                      long ldw, unsigned long long *amax_bits, long j)
{
    const double *src = H + j * ldh;
    double *dst = D + j * ldd;
    float *w = W + j * ldw;
    unsigned long long m = 0;
    auto take = [&](long i, double v) {
        m = max(m, (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull);
        dst[i] = v;
        w[i] = (float)v;
    };
    long i0 = j;
    if (i0 < n && ((uintptr_t)(src + i0) & 15)) {
        if (threadIdx.x == 0) take(i0, src[i0]);
        ++i0;
    }
    const bool vec = !((uintptr_t)(src + i0) & 15) && !((uintptr_t)(dst + i0) & 15) && !((uintptr_t)(w + i0) & 7);
    if (vec) {
        const double2 *s2 = (const double2 *)(src + i0);
        double2 *d2 = (double2 *)(dst + i0);
        float2 *w2 = (float2 *)(w + i0);
        const long n2 = (n - i0) / 2;
        for (long p = threadIdx.x; p < n2; p += 4 * 256) {
            double2 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (p + u * 256 < n2) v[u] = s2[p + u * 256];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (p + u * 256 >= n2) break;
                m = max(m, (unsigned long long)__double_as_longlong(v[u].x) & 0x7FFFFFFFFFFFFFFFull);
                m = max(m, (unsigned long long)__double_as_longlong(v[u].y) & 0x7FFFFFFFFFFFFFFFull);
                d2[p + u * 256] = v[u];
                w2[p + u * 256] = make_float2((float)v[u].x, (float)v[u].y);
            }
        }
        if (((n - i0) & 1) && threadIdx.x == 0) take(n - 1, src[n - 1]);
    } else {
        for (long i = i0 + threadIdx.x; i < n; i += 256) take(i, src[i]);
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)m, o));
    __shared__ unsigned long long red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < 8; ++q) m = max(m, red[q]);
        atomicMax(amax_bits, m);
    }
}

__global__ void __launch_bounds__(256) gather_convert_kernel(int n, const double *__restrict__ H, long ldh,
                                                             double *__restrict__ D, long ldd, float *__restrict__ W,
                                                             long ldw, unsigned long long *amax_bits, int j0 = 0,
                                                             int j1 = -1)
{
    // one column per CTA (j1 < 0), or columns j0 + blockIdx.x, + gridDim.x, ... below j1
    const int jend = j1 < 0 ? j0 + (int)gridDim.x : j1;
    for (long j = j0 + (long)blockIdx.x; j < jend; j += gridDim.x) {
        gather_convert_column(n, H, ldh, D, ldd, W, ldw, amax_bits, j);
        __syncthreads();  // the column's reduction buffer is free
    }
}

// d[i] = fp32(A_ii) from the mapped host matrix (the factorisation's row
// bounds need the whole diagonal before the columns have arrived)
__global__ void gather_diag_kernel(int n, const double *__restrict__ H, long ldh, float *__restrict__ d)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = (float)H[i + i * ldh];
}

// Device address of a pinned (page-locked, mapped) host buffer, or NULL when
// `p` is not one -- ordinary pageable memory takes the copy path.
static const double *device_view_of_pinned(const double *p)
{
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (pa.type != cudaMemoryTypeHost || !pa.devicePointer) return nullptr;
    return (const double *)pa.devicePointer;
}

// The device view of a whole column-major n x n host matrix (ld lda): both
// its first and its last element must be pinned and mapped at the same
// offset, else the copy path is taken.
static const double *device_view_of_pinned_matrix(const double *A, int n, int lda)
{
    const double *d0 = device_view_of_pinned(A);
    if (!d0) return nullptr;
    const size_t last = (size_t)(n - 1) + (size_t)(n - 1) * lda;
    const double *d1 = device_view_of_pinned(A + last);
    return d1 == d0 + last ? d0 : nullptr;
}

// The overlapped gather (STARPU_GB300_HOST_OVERLAP=1; off by default) needs
// a copy stream, one event per superblock, a store for every step's split
// panel and the diagonal, allocated once for n_max; it applies to the
// tensor-core path with a lookahead (n > 2 nb) and tile sizes the
// diagonal-tile kernel handles.  Measured at n = 32768 it is slower than
// gathering first (104-111 ms against 91 ms per host-buffer solve): the early
// steps, their updates cut to the columns that have arrived, lose the overlap
// of the diagonal tile with a large update, and the replays of the late
// columns crowd the lookahead stream.
static constexpr int GATHER_CTAS = 48;
static bool overlap_ready(starpu_gb300_solver *h, int n, int nb)
{
    static const bool env_on = [] {
        const char *e = getenv("STARPU_GB300_HOST_OVERLAP");
        return e && !strcmp(e, "1");
    }();
    const bool on = h->overlap >= 0 ? h->overlap != 0 : env_on;
    if (!on || h->overlap_failed || n <= 2 * nb || nb > GB300_DIAG_TILE_MAX || h->nterms != 3) return false;
    if (!h->copy) {
        const int nsb_max = (h->n_max + 2 * nb - 1) / (2 * nb);
        bool ok = cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming) == cudaSuccess &&
                  cudaMalloc(&h->panels, tc_arrival_store_bytes(h->n_max, nb)) == cudaSuccess &&
                  cudaMalloc((void **)&h->diag, sizeof(float) * (size_t)h->n_max) == cudaSuccess;
        for (int q = 0; ok && q < nsb_max; ++q) {
            cudaEvent_t e = nullptr;
            ok = cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
            if (ok) h->ready.push_back(e);
        }
        if (!ok) {  // no room: gather the whole matrix first, as before
            cudaGetLastError();
            h->overlap_failed = true;
            return false;
        }
    }
    return true;
}

int starpu_gb300_solver_dsposv_host(starpu_gb300_solver *h, int n, int nrhs, const double *A, int lda,
                                    const double *B, int ldb, double *X, int ldx, double tol, int max_iter,
                                    starpu_gb300_ir_info *info)
{
    if (!h || n < 0 || nrhs < 0 || n > h->n_max || nrhs > h->nrhs_max || lda < n || ldb < n || ldx < n)
        return GB300_EINVAL;
    if (!n || !nrhs) return GB300_OK;
    cudaStream_t s = h->stream;
    int rc;
    int slot = gb300_prof_begin(s, GB300_PROF_TRANSFER);
    // only the lower triangle is read by the solve: copy it as trapezoidal
    // column panels (rows j0..n-1 of columns j0..j0+w-1), each one pitched
    // copy of whole column segments -- n^2/2 + n w/2 elements instead of n^2
    double abytes = 0.0;
    const double *mapped = device_view_of_pinned_matrix(A, n, lda);
    const int nb_eff = h->nb > 0 ? h->nb : 1024;
    TcArrival arr;
    std::vector<int> starts;
    if (mapped) {
        // pinned host memory the GPU can read: one kernel pulls exactly the
        // lower triangle over the host link (pitched copies of column
        // segments run far below the link rate) and writes the factor
        // phase's FP32 copy and max |A_ij| on the way
        float *W = nullptr;
        unsigned long long *amax = nullptr;
        dsposv_prepared_targets(n, nrhs, nb_eff, h->work, &W, &amax);
        cudaMemsetAsync(amax, 0, 4 * sizeof(unsigned long long), s);
        if (overlap_ready(h, n, nb_eff)) {
            // superblocks of two column blocks on the copy stream, each
            // announced by an event: the factorisation starts on the first
            // columns while the rest is still crossing the host link
            const int sbw = 2 * nb_eff, nsb = (n + sbw - 1) / sbw;
            starts.resize(nsb + 1);
            for (int q = 0; q <= nsb; ++q) starts[q] = std::min(n, q * sbw);
            cudaEventRecord(h->fork, s);
            cudaStreamWaitEvent(h->copy, h->fork, 0);
            gb300_count_launch(), gather_diag_kernel<<<(n + 255) / 256, 256, 0, h->copy>>>(n, mapped, lda, h->diag);
            for (int q = 0; q < nsb; ++q) {
                // a few CTAs, each with its columns' loads in flight: they reach the
                // link rate and fit beside the factorisation's kernels on their SMs
                gb300_count_launch(), gather_convert_kernel<<<std::min(GATHER_CTAS, starts[q + 1] - starts[q]), 256, 0,
                                                              h->copy>>>(n, mapped, lda, h->A, n, W, n, amax + 2,
                                                                         starts[q], starts[q + 1]);
                cudaEventRecord(h->ready[q], h->copy);
            }
            arr.nsb = nsb;
            arr.start = starts.data();
            arr.ready = h->ready.data();
            arr.diag = h->diag;
            arr.panel_store = h->panels;
        } else {
            gb300_count_launch(), gather_convert_kernel<<<n, 256, 0, s>>>(n, mapped, lda, h->A, n, W, n, amax + 2);
        }
        if ((rc = gb300_last_launch_status())) return rc;
        abytes = 8.0 * n * (n + 1.0) / 2.0;
    } else {
        for (int j0 = 0; j0 < n; j0 += HOST_PANEL) {
            const int w = std::min(HOST_PANEL, n - j0);
            const size_t rows = (size_t)(n - j0);
            if ((rc = gb300_record_cuda_error(cudaMemcpy2DAsync(h->A + j0 + (size_t)j0 * n, sizeof(double) * n,
                                                                A + j0 + (size_t)j0 * lda, sizeof(double) * lda,
                                                                sizeof(double) * rows, w, cudaMemcpyHostToDevice,
                                                                s))))
                return rc;
            abytes += 8.0 * rows * w;
        }
    }
    if ((rc = gb300_record_cuda_error(
             ldb == n ? cudaMemcpyAsync(h->B, B, sizeof(double) * (size_t)n * nrhs, cudaMemcpyHostToDevice, s)
                      : cudaMemcpy2DAsync(h->B, sizeof(double) * n, B, sizeof(double) * ldb, sizeof(double) * n,
                                          nrhs, cudaMemcpyHostToDevice, s))))
        return rc;
    gb300_prof_end(s, slot, 0.0, abytes + 8.0 * n * (double)nrhs);
    int status;
    if (mapped) {
        // the factor phase's first pass was fused into the gather
        if (info) memset(info, 0, sizeof *info);
        if ((h->nterms != 1 && h->nterms != 3) || max_iter < 0 || !(tol >= 0)) return GB300_EINVAL;
        status = dsposv_ladder(s, n, nrhs, h->A, n, h->B, n, h->X, n, nb_eff, h->nterms, tol, max_iter, h->work,
                               info, true, arr.nsb ? &arr : nullptr);
    } else {
        status = starpu_gb300_dsposv(s, n, nrhs, h->A, n, h->B, n, h->X, n, h->nb, h->nterms, tol, max_iter, h->work,
                                     h->lwork, info);
    }
    if (status != GB300_OK && status != GB300_ETIMEDOUT) return status;
    slot = gb300_prof_begin(s, GB300_PROF_TRANSFER);
    if ((rc = gb300_record_cuda_error(
             ldx == n ? cudaMemcpyAsync(X, h->X, sizeof(double) * (size_t)n * nrhs, cudaMemcpyDeviceToHost, s)
                      : cudaMemcpy2DAsync(X, sizeof(double) * ldx, h->X, sizeof(double) * n, sizeof(double) * n,
                                          nrhs, cudaMemcpyDeviceToHost, s))))
        return rc;
    gb300_prof_end(s, slot, 0.0, 8.0 * n * (double)nrhs);
    if ((rc = gb300_record_cuda_error(cudaStreamSynchronize(s)))) return rc;
    return status;
}

// Host check of the tile sweeps' ticket order for ntiles tile rows of spt
// slabs: every ticket decodes to one task, each task appears once, and every
// task a ticket waits for has a smaller ticket -- a product of tile row u with
// earlier row v waits for all spt diagonal tasks of v, a diagonal task of row
// u for all u spt products of u.  With at least spt CTAs taking tickets in
// order, that makes the sweeps deadlock-free.  0 on success.
int starpu_gb300_selftest_sweep_tickets(int ntiles, int spt)
{
    if (ntiles <= 0 || spt <= 0) return -1;
    const unsigned total = (unsigned)((size_t)spt * ntiles * (ntiles + 1) / 2);
    std::vector<int> diag_done(ntiles, 0), prod_done(ntiles, 0);
    std::vector<char> seen((size_t)ntiles * (ntiles + 1) * spt, 0);
    for (unsigned t = 0; t < total; ++t) {
        int u;
        unsigned r;
        tsw_decode(t, spt, u, r);
        if (u < 0 || u >= ntiles || r >= (unsigned)((u + 1) * spt)) return 1;
        char &mark = seen[((size_t)u * (ntiles + 1) + r / spt) * spt + r % spt];
        if (mark) return 2;
        mark = 1;
        if (r < (unsigned)(u * spt)) {
            if (diag_done[r / spt] != spt) return 3;
            ++prod_done[u];
        } else {
            if (prod_done[u] != u * spt) return 4;
            ++diag_done[u];
        }
    }
    for (int u = 0; u < ntiles; ++u)
        if (diag_done[u] != spt || prod_done[u] != u * spt) return 5;
    return 0;
}

size_t starpu_gb300_spotrs_inv_tiles_workspace(int n, int nb)
{
    if (n < 0 || !tile_sweep_ok(nb)) return 0;
    return tsw_scratch_bytes(n, nb);
}

int starpu_gb300_spotrs_inv_tiles(void *stream, int n, int nrhs, int nb, const float *L, int ldl, const float *Dinv,
                                  int ldd, float *B, int ldb, void *work, size_t lwork, int *d_err)
{
    if (n < 0 || nrhs < 0 || !tile_sweep_ok(nb) || ldl < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1) || ldd < nb ||
        (n && (!L || !Dinv || !B || !work || !d_err || lwork < starpu_gb300_spotrs_inv_tiles_workspace(n, nb))))
        return GB300_EINVAL;
    if (!n || !nrhs) return GB300_OK;
    tile_sweeps((cudaStream_t)stream, n, nrhs, nb, L, ldl, Dinv, ldd, B, ldb, work, d_err);
    return gb300_last_launch_status();
}

// ---- symmetric residual R = B - A X with the tensor-core slice products ----

static size_t syres_layout(int n, int nrhs, char *base, double **partials, float2 **xs, int **sx, void **rxs,
                           unsigned long long **an, void **rta, float **rsum)
{
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const size_t oP = take(residual_partials(n, nrhs) * sizeof(double));
    const size_t oX = take((size_t)n * 16 * ((nrhs + 15) / 16) * sizeof(float2));
    const size_t oS = take((size_t)nrhs * sizeof(int));
    const size_t oR = take(residual_tc_xs_bytes(n, nrhs));
    const size_t oA = take(4 * sizeof(unsigned long long));
    const size_t oT = take(residual_tc_a_bytes(n));
    const size_t oN = take((size_t)((n + 63) / 64) * n * sizeof(float));
    if (base) {
        *partials = (double *)(base + oP);
        *xs = (float2 *)(base + oX);
        *sx = (int *)(base + oS);
        *rxs = base + oR;
        *an = (unsigned long long *)(base + oA);
        *rta = base + oT;
        *rsum = (float *)(base + oN);
    }
    return off;
}

size_t starpu_gb300_dsyresidual_workspace(int n, int nrhs)
{
    if (n <= 0 || nrhs <= 0) return 0;
    return syres_layout(n, nrhs, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int starpu_gb300_dsyresidual(void *stream, int n, int nrhs, const double *A, int lda, const double *X, int ldx,
                             const double *B, int ldb, double *R, int ldr, void *work, size_t lwork, int *d_err)
{
    if (n <= 0 || nrhs <= 0) return n < 0 || nrhs < 0 ? GB300_EINVAL : GB300_OK;
    if (lda < n || ldx < n || ldb < n || ldr < n || !A || !X || !B || !R || !work || !d_err ||
        lwork < starpu_gb300_dsyresidual_workspace(n, nrhs))
        return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    double *partials;
    float2 *xs;
    int *sx;
    void *rxs, *rta;
    unsigned long long *an;
    float *rsum;
    syres_layout(n, nrhs, (char *)work, &partials, &xs, &sx, &rxs, &an, &rta, &rsum);
    cudaMemsetAsync(an, 0, 4 * sizeof *an, s);
    gb300_count_launch(), convert_lower_max_kernel<<<n, 256, 0, s>>>(n, A, lda, nullptr, 0, an + 2);
    int rc = residual_tc_slice_a(s, n, A, lda, an + 2, rta, rsum);
    if (rc) return rc;
    gb300_count_launch(), norm_from_rowsums_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, (n + 63) / 64, rsum, an + 2, an);
    return residual_mixed(s, n, nrhs, A, lda, X, ldx, B, ldb, R, ldr, partials, xs, sx, rta, rxs, an, d_err);
}

size_t starpu_gb300_backward_error_workspace(int n, int nrhs)
{
    return align256((size_t)n * nrhs * sizeof(double)) + align256((size_t)nrhs * (sizeof(double) + sizeof(int))) +
           256 + align256(residual_partials(n, nrhs) * sizeof(double));
}

int starpu_gb300_backward_error(void *stream, int n, int nrhs, const double *A, int lda, const double *X, int ldx,
                                const double *B, int ldb, void *work, size_t lwork, double *berr_host)
{
    if (n <= 0 || nrhs <= 0 || lda < n || ldx < n || ldb < n || !work || !berr_host ||
        lwork < starpu_gb300_backward_error_workspace(n, nrhs))
        return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    char *w = (char *)work;
    double *R = (double *)w;
    w += align256((size_t)n * nrhs * sizeof(double));
    double *berr = (double *)w;
    int *done = (int *)(berr + nrhs);
    w += align256((size_t)nrhs * (sizeof(double) + sizeof(int)));
    unsigned long long *an = (unsigned long long *)w;
    double *partials = (double *)(w + 256);
    cudaMemsetAsync(an, 0, sizeof *an, s);
    gb300_count_launch(), convert_lower_norm_kernel<<<n, 256, 0, s>>>(n, A, lda, nullptr, 0, an);
    residual_f64(s, n, nrhs, A, lda, X, ldx, B, ldb, R, n, partials);
    gb300_count_launch(), backward_error_kernel<<<nrhs, 256, 0, s>>>(n, R, n, X, ldx, B, ldb, an, 0.0, berr, done, nullptr);
    int rc = gb300_record_cuda_error(cudaMemcpyAsync(berr_host, berr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    if (rc) return rc;
    return gb300_record_cuda_error(cudaStreamSynchronize(s));
}

// Plain FP64 solve (LAPACK dposv): the baseline the mixed path is measured against.
int starpu_gb300_dposv(void *stream, int n, int nrhs, double *A, int lda, double *B, int ldb, int nb, int *d_info)
{
    int rc = starpu_gb300_dpotrf(stream, n, A, lda, nb, d_info);
    if (rc) return rc;
    return starpu_gb300_dpotrs(stream, n, nrhs, A, lda, B, ldb);
}

} // extern "C"
