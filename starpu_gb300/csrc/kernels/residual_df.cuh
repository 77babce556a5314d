// Residual r = b - A x of the refinement loop (A symmetric, lower triangle
// read) on the FP32 pipe in double-float arithmetic.  GB300 issues FP64 FMAs at ~1/60 of its FP32 rate, so the FP64
// residual (2 n^2 nrhs flops) is compute-bound at the FP64 peak; the same sum
// is formed here from FP32 pairs (hi + lo, 48 significant bits):
//
//   A, X scaled by powers of two (A by 2^-ea, ea = exponent of ||A||_inf; each
//   column of X by 2^-ex_j) so that every FP32 part is in range; tiny parts
//   below 2^-126 of the scale are dropped (relative weight < 2^-74).
//   a = a_h + a_l: a_h = the top 24 bits of a's mantissa (bit truncation),
//   a_l = the rest rounded to 24 bits -- integer operations only, no FP64.
//   x = x_h + x_l: round-to-nearest splits (done once per column).
//   Each product a*x: p = a_h*x_h exactly as p + fma(a_h, x_h, -p) (two-prod),
//   plus a_h*x_l + a_l*x_h; the running sum keeps an error-free two-sum of the
//   high parts and a low-part accumulator.  Every 128 terms the pair is added
//   to an FP64 accumulator, bounding the growth of the low-part rounding.
//
// Relative accuracy ~2^-47 of sum |a||x| per 128-term block (random errors
// add in quadrature across blocks): the refinement's stopping test at 1e-12
// sees an error ~1e-14.  The partials (one per K chunk) are reduced in FP64
// in a fixed order, so the result is deterministic.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "df_arith.cuh"

namespace gb300 {

constexpr int RDF_BM = 128;     // rows per CTA
constexpr int RDF_BK = 32;      // k per stage
constexpr int RDF_FLUSH = 4;    // stages per FP64 flush (128 terms)

// One CTA per column j of X: ex_j = exponent of max_k |x_kj|, and
// Xs[(j / 16) n 16 + k 16 + j % 16] = split(x_kj * 2^-ex_j).
__global__ void __launch_bounds__(256) df_split_x_kernel(int n, const double *__restrict__ X, long ldx,
                                                         float2 *__restrict__ Xs, int *__restrict__ sx)
{
    const int j = blockIdx.x;
    const double *x = X + (long)j * ldx;
    double m = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) m = fmax(m, fabs(x[k]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ double red[8];
    __shared__ int s_ex;
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
        s_ex = df_scale_exp(m);
        sx[j] = s_ex;
    }
    __syncthreads();
    const double sc = scalbn(1.0, -s_ex);
    float2 *out = Xs + (long)(j / 16) * n * 16 + (j % 16);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double v = x[k] * sc;
        const float h = __double2float_rn(v);
        out[(long)k * 16] = make_float2(h, __double2float_rn(v - (double)h));
    }
}

// Stage layout of a 128-row x 32-column block of the symmetric A read from
// its lower triangle only: blocks strictly below the diagonal are read as
// they are (threads along rows: coalesced), blocks strictly above as the
// transpose of the mirror block (threads along k: coalesced), blocks that
// cross the diagonal element by element.
enum { RDF_LOWER = 0, RDF_UPPER = 1, RDF_DIAG = 2 };
__device__ __forceinline__ int rdf_mode(int i0, int k0)
{
    if (k0 + RDF_BK <= i0) return RDF_LOWER;
    if (k0 >= i0 + RDF_BM) return RDF_UPPER;
    return RDF_DIAG;
}
// element e (0 .. 4095) of a stage -> (row, kk)
__device__ __forceinline__ void rdf_coords(int mode, int e, int &row, int &kk)
{
    if (mode == RDF_UPPER) {
        kk = e & (RDF_BK - 1);
        row = e >> 5;
    } else {
        row = e & (RDF_BM - 1);
        kk = e >> 7;
    }
}

// P[z n nrhs + i + j n] = -(A[i, kz] X[kz, j]) over the K chunk z = blockIdx.z
// (kchunk a multiple of RDF_BK), rows i of the 128-row block blockIdx.x,
// columns j of the group of 16 blockIdx.y.  A is symmetric and only its lower
// triangle is read.  256 threads: thread (r = tid % 64, g = tid / 64) owns
// rows r, r + 64 and columns 4g .. 4g+3.  The next stage's A block is loaded
// into registers while the current one is multiplied from shared memory.
__global__ void __launch_bounds__(256, 2) residual_df_kernel(int n, int nrhs, const double *__restrict__ A, long lda,
                                                             const float2 *__restrict__ Xs, const int *__restrict__ sx,
                                                             const unsigned long long *__restrict__ anorm_bits,
                                                             int kchunk, double *__restrict__ P)
{
    // one float2 of padding per row: the transposed (upper) stages store along k
    __shared__ float2 As[RDF_BK][RDF_BM + 1];
    __shared__ __align__(16) float2 Xt[RDF_BK][16];
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * RDF_BM;
    const int grp = blockIdx.y;
    const int j0 = grp * 16;
    const int ncols = min(16, nrhs - j0);
    const int kz0 = blockIdx.z * kchunk;
    const int kz1 = min(n, kz0 + kchunk);
    const int ea = df_scale_exp(__longlong_as_double((long long)*anorm_bits));
    const float2 *Xg = Xs + (long)grp * n * 16;
    const int r = tid & 63, g = tid >> 6;

    double ra[16];
    float4 rx;
    auto load_stage = [&](int k0) {
        const int mode = rdf_mode(i0, k0);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            int row, kk;
            rdf_coords(mode, tid + 256 * q, row, kk);
            const int i = i0 + row, k = k0 + kk;
            double v = 0.0;
            if (i < n && k < kz1) {
                const bool mirror = mode == RDF_UPPER || (mode == RDF_DIAG && k > i);
                v = __ldg(mirror ? &A[(long)k + (long)i * lda] : &A[(long)i + (long)k * lda]);
            }
            ra[q] = v;
        }
        const int k = k0 + (tid >> 3), c = (tid & 7) * 2;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (k < kz1) {
            const float2 a = Xg[(long)k * 16 + c], b = Xg[(long)k * 16 + c + 1];
            if (c < ncols) v.x = a.x, v.y = a.y;
            if (c + 1 < ncols) v.z = b.x, v.w = b.y;
        }
        rx = v;
    };

    float sh[2][4], sl[2][4];
    double acc[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < 4; ++c) sh[h][c] = sl[h][c] = 0.0f, acc[h][c] = 0.0;

    if (kz0 < kz1) load_stage(kz0);
    int stage = 0;
    for (int k0 = kz0; k0 < kz1; k0 += RDF_BK) {
        __syncthreads();  // the previous stage's reads of As / Xt are done
        const int mode = rdf_mode(i0, k0);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            int row, kk;
            rdf_coords(mode, tid + 256 * q, row, kk);
            As[kk][row] = df_split_scaled(ra[q], ea);
        }
        reinterpret_cast<float4 *>(&Xt[0][0])[tid] = rx;
        __syncthreads();
        if (k0 + RDF_BK < kz1) load_stage(k0 + RDF_BK);
#pragma unroll 4
        for (int kk = 0; kk < RDF_BK; ++kk) {
            const float2 a0 = As[kk][r], a1 = As[kk][r + 64];
            const float4 x01 = *reinterpret_cast<const float4 *>(&Xt[kk][4 * g]);
            const float4 x23 = *reinterpret_cast<const float4 *>(&Xt[kk][4 * g + 2]);
            df_mac(sh[0][0], sl[0][0], a0.x, a0.y, x01.x, x01.y);
            df_mac(sh[0][1], sl[0][1], a0.x, a0.y, x01.z, x01.w);
            df_mac(sh[0][2], sl[0][2], a0.x, a0.y, x23.x, x23.y);
            df_mac(sh[0][3], sl[0][3], a0.x, a0.y, x23.z, x23.w);
            df_mac(sh[1][0], sl[1][0], a1.x, a1.y, x01.x, x01.y);
            df_mac(sh[1][1], sl[1][1], a1.x, a1.y, x01.z, x01.w);
            df_mac(sh[1][2], sl[1][2], a1.x, a1.y, x23.x, x23.y);
            df_mac(sh[1][3], sl[1][3], a1.x, a1.y, x23.z, x23.w);
        }
        if (++stage == RDF_FLUSH) {
            stage = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    acc[h][c] += (double)sh[h][c] + (double)sl[h][c];
                    sh[h][c] = sl[h][c] = 0.0f;
                }
        }
    }
    double *Pz = P + (long)blockIdx.z * n * nrhs;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = i0 + r + 64 * h;
        if (i >= n) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int jj = 4 * g + c;
            if (jj >= ncols) continue;
            const double v = acc[h][c] + ((double)sh[h][c] + (double)sl[h][c]);
            Pz[(long)i + (long)(j0 + jj) * n] = -scalbn(v, ea + sx[j0 + jj]);
        }
    }
}

} // namespace gb300
