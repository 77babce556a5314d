// Persistent batched SPD solve: one launch factors and solves many
// independent systems of different sizes (n <= 1024), FP32 blocked Cholesky
// + FP64 iterative refinement, one CTA per system at a time.
//
// Work distribution: systems are visited in the order given by `order`
// (largest first); each CTA takes the next system with an atomic ticket, so
// big systems start early and the small ones fill the tail.  A CTA runs the
// whole pipeline for its system with a fixed sequence of operations, so a
// system's result does not depend on which other systems share the launch.
//
// Per system (256 threads, FP32 work copy W of the lower triangle):
//   W = fp32(A), ||A||_inf                        (A FP64, column-major, ld = n)
//   right-looking blocked Cholesky with block NB (the tuned parameter):
//     POTRF of the NB x NB diagonal block in shared memory
//     TRSM of the panel rows, one row per thread, registers
//     lower-triangular trailing update in 64 x 64 tiles staged in shared memory
//   x = fp64(L^-T L^-1 fp32(b)); repeat r = b - A x (FP64), berr, x += corr.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb300 {

constexpr int BAT_THREADS = 256;
constexpr int BAT_MAXN = 1024;
constexpr int BAT_MAXRHS = 8;
constexpr int BAT_TILE = 64;

struct BatchedArgs {
    int nsys;
    const int *n;                 // [nsys]
    const long long *a_off;       // offset (doubles) of system i in A / (floats) in W
    const long long *b_off;       // offset (doubles) of system i in B and X
    const int *order;             // visiting order (largest first)
    const double *A;
    const double *B;
    double *X;
    float *W;                     // FP32 work copies (same offsets as A)
    float *Y;                     // FP32 rhs/corrections (same offsets as B)
    double *R;                    // FP64 residuals (same offsets as B)
    int nrhs;
    double tol;
    int max_iter;
    int *status;                  // [nsys] iterations (>= 0) or -(info) / -1000 not converged
    double *berr;                 // [nsys] final max backward error
    unsigned *ticket;
    const signed char *nb_of_bucket;  // block size per size bucket (log2 of ceil(n/32))
};

__device__ __forceinline__ int bucket_of(int n)
{
    int b = 0;
    int t = (n + 31) / 32;
    while ((1 << b) < t) ++b;
    return b > 5 ? 5 : b;  // 32, 64, 128, 256, 512, 1024
}

// ----------------------------------------------------------------- factor
template <int NB>
__device__ int bat_factor(float *W, int n, float *smem)
{
    float(*D)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(smem);   // diagonal block
    float *As = smem + NB * (NB + 1);                                  // [NB][64] panel slice (k-major)
    float *Bs = As + NB * BAT_TILE;                                    // [NB][64]
    __shared__ int s_info;
    const int tid = threadIdx.x;
    if (tid == 0) s_info = 0;
    __syncthreads();
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = min(NB, n - k0);
        // ---- POTRF of the diagonal block
        for (int idx = tid; idx < NB * NB; idx += BAT_THREADS) {
            const int i = idx % NB, j = idx / NB;
            D[i][j] = (i < kb && j < kb && i >= j) ? W[(k0 + i) + (long)(k0 + j) * n] : 0.0f;
        }
        __syncthreads();
        constexpr int CL = BAT_THREADS / NB;  // column lanes for the rank-1 update
        const int ti = tid % NB, tc = tid / NB;
        for (int z = 0; z < kb; ++z) {
            if (tid == 0) {
                const float d = D[z][z];
                if (!(d > 0.0f) && s_info == 0) s_info = k0 + z + 1;
                D[z][z] = sqrtf(d);
            }
            __syncthreads();
            const float inv = 1.0f / D[z][z];
            if (tc == 0 && ti > z && ti < kb) D[ti][z] *= inv;
            __syncthreads();
            if (ti > z && ti < kb) {
                const float liz = D[ti][z];
                for (int c = z + 1 + tc; c <= ti; c += CL) D[ti][c] = fmaf(-liz, D[c][z], D[ti][c]);
            }
            __syncthreads();
        }
        for (int idx = tid; idx < kb * kb; idx += BAT_THREADS) {
            const int i = idx % kb, j = idx / kb;
            if (i >= j) W[(k0 + i) + (long)(k0 + j) * n] = D[i][j];
        }
        if (s_info) break;
        const int r0 = k0 + kb, m = n - r0;
        if (m <= 0) break;
        // ---- TRSM: W[i, k0:k0+kb] <- W[i, k0:k0+kb] L_kk^-T, one row per thread
        for (int i = r0 + tid; i < n; i += BAT_THREADS) {
            float x[NB];
#pragma unroll
            for (int c = 0; c < NB; ++c) x[c] = (c < kb) ? W[i + (long)(k0 + c) * n] : 0.0f;
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                if (j < kb) {
                    x[j] = x[j] / D[j][j];
#pragma unroll
                    for (int c = j + 1; c < NB; ++c) x[c] = fmaf(-D[c][j], x[j], x[c]);
                }
            }
#pragma unroll
            for (int c = 0; c < NB; ++c)
                if (c < kb) W[i + (long)(k0 + c) * n] = x[c];
        }
        __syncthreads();
        // ---- trailing update of the lower triangle, 64 x 64 tiles
        const int nt = (m + BAT_TILE - 1) / BAT_TILE;
        const int tr = tid % 16, tcn = tid / 16;  // 16 x 16 threads, 4 x 4 outputs each
        for (int tj = 0; tj < nt; ++tj) {
            // stage the panel rows of tile column tj once per column
            for (int idx = tid; idx < NB * BAT_TILE; idx += BAT_THREADS) {
                const int rr = idx % BAT_TILE, p = idx / BAT_TILE;
                const int row = r0 + tj * BAT_TILE + rr;
                Bs[p * BAT_TILE + rr] = (p < kb && row < n) ? W[row + (long)(k0 + p) * n] : 0.0f;
            }
            for (int ti2 = tj; ti2 < nt; ++ti2) {
                for (int idx = tid; idx < NB * BAT_TILE; idx += BAT_THREADS) {
                    const int rr = idx % BAT_TILE, p = idx / BAT_TILE;
                    const int row = r0 + ti2 * BAT_TILE + rr;
                    As[p * BAT_TILE + rr] = (p < kb && row < n) ? W[row + (long)(k0 + p) * n] : 0.0f;
                }
                __syncthreads();
                float acc[4][4];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
                for (int p = 0; p < kb; ++p) {
                    float av[4], bv[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) av[a] = As[p * BAT_TILE + tr + 16 * a];
#pragma unroll
                    for (int b = 0; b < 4; ++b) bv[b] = Bs[p * BAT_TILE + tcn + 16 * b];
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
                }
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int col = r0 + tj * BAT_TILE + tcn + 16 * b;
                    if (col >= n) continue;
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int row = r0 + ti2 * BAT_TILE + tr + 16 * a;
                        if (row < n && row >= col) W[row + (long)col * n] -= acc[a][b];
                    }
                }
                __syncthreads();
            }
        }
    }
    __syncthreads();
    return s_info;
}

// --------------------------------------------------------------- solves
// Mirror the factor into the upper triangle of W (W[j, i] = L[i, j]) so that
// both sweeps below read contiguous columns.
__device__ void bat_mirror_upper(float *W, int n)
{
    for (long idx = threadIdx.x; idx < (long)n * n; idx += BAT_THREADS) {
        const int i = (int)(idx % n), j = (int)(idx / n);  // write (i, j) with i < j from (j, i)
        if (i < j) W[i + (long)j * n] = W[j + (long)i * n];
    }
    __syncthreads();
}

// Y (n x nrhs, ld n) <- L^-T L^-1 Y.  Column-oriented substitution: at step j
// the owner of row j finishes y_j, then every thread updates its rows with
// column j of L (forward) or of L^T (backward, read from the mirrored upper
// triangle); both reads are contiguous along the rows the threads own.
__device__ void bat_potrs(const float *W, int n, float *Y, int nrhs)
{
    const int tid = threadIdx.x;
    for (int j = 0; j < n; ++j) {
        const float *Lj = W + (long)j * n;  // L[:, j]
        if (j % BAT_THREADS == tid) {
            const float d = Lj[j];
            for (int c = 0; c < nrhs; ++c) Y[j + (long)c * n] /= d;
        }
        __syncthreads();
        for (int i = j + 1 + ((tid - (j + 1) % BAT_THREADS + BAT_THREADS) % BAT_THREADS); i < n; i += BAT_THREADS) {
            const float l = Lj[i];
            for (int c = 0; c < nrhs; ++c) Y[i + (long)c * n] = fmaf(-l, Y[j + (long)c * n], Y[i + (long)c * n]);
        }
    }
    __syncthreads();
    for (int j = n - 1; j >= 0; --j) {
        const float *Uj = W + (long)j * n;  // U[:, j] = L[j, :] in rows 0..j
        if (j % BAT_THREADS == tid) {
            const float d = Uj[j];
            for (int c = 0; c < nrhs; ++c) Y[j + (long)c * n] /= d;
        }
        __syncthreads();
        for (int i = tid; i < j; i += BAT_THREADS) {
            const float u = Uj[i];
            for (int c = 0; c < nrhs; ++c) Y[i + (long)c * n] = fmaf(-u, Y[j + (long)c * n], Y[i + (long)c * n]);
        }
    }
    __syncthreads();
}

// -------------------------------------------------------------- kernel
__global__ void __launch_bounds__(BAT_THREADS, 2) batched_dposv_kernel(BatchedArgs a)
{
    extern __shared__ __align__(16) float bat_smem[];
    __shared__ unsigned s_sys;
    __shared__ double s_red[4][BAT_THREADS / 32];
    __shared__ double s_anorm;
    __shared__ int s_done;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_sys = atomicAdd(a.ticket, 1u);
        __syncthreads();
        const unsigned t = s_sys;
        __syncthreads();
        if (t >= (unsigned)a.nsys) return;
        const int sys = a.order[t];
        const int n = a.n[sys];
        const double *A = a.A + a.a_off[sys];
        float *W = a.W + a.a_off[sys];
        const double *B = a.B + a.b_off[sys];
        double *X = a.X + a.b_off[sys];
        float *Y = a.Y + a.b_off[sys];
        double *R = a.R + a.b_off[sys];
        const int nrhs = a.nrhs;
        // W = fp32(lower A); row sums of |A| -> ||A||_inf
        double rowmax = 0.0;
        for (int i = tid; i < n; i += BAT_THREADS) {
            double s = 0.0;
            for (int j = 0; j < n; ++j) {
                const double v = A[i + (long)j * n];
                s += fabs(v);
                if (i >= j) W[i + (long)j * n] = (float)v;
            }
            rowmax = fmax(rowmax, s);
        }
        for (int o = 16; o > 0; o >>= 1) rowmax = fmax(rowmax, __shfl_xor_sync(0xffffffffu, rowmax, o));
        if ((tid & 31) == 0) s_red[0][tid >> 5] = rowmax;
        __syncthreads();
        if (tid == 0) {
            double m = 0;
            for (int w = 0; w < BAT_THREADS / 32; ++w) m = fmax(m, s_red[0][w]);
            s_anorm = m;
        }
        __syncthreads();
        const int nb = a.nb_of_bucket[bucket_of(n)];
        int info;
        if (nb == 16) info = bat_factor<16>(W, n, bat_smem);
        else if (nb == 32) info = bat_factor<32>(W, n, bat_smem);
        else info = bat_factor<64>(W, n, bat_smem);
        if (info) {
            if (tid == 0) {
                a.status[sys] = -info;
                a.berr[sys] = INFINITY;
            }
            __syncthreads();
            continue;
        }
        bat_mirror_upper(W, n);
        // initial solve
        for (int idx = tid; idx < n * nrhs; idx += BAT_THREADS) Y[idx] = (float)B[idx];
        __syncthreads();
        bat_potrs(W, n, Y, nrhs);
        for (int idx = tid; idx < n * nrhs; idx += BAT_THREADS) X[idx] = (double)Y[idx];
        __syncthreads();
        int it = 0;
        double worst = INFINITY;
        for (;; ++it) {
            // R = B - A X, columns of A streamed, one row per thread (coalesced)
            for (int i = tid; i < n; i += BAT_THREADS) {
                double acc[BAT_MAXRHS];
#pragma unroll
                for (int c = 0; c < BAT_MAXRHS; ++c) acc[c] = (c < nrhs) ? B[i + (long)c * n] : 0.0;
                for (int j = 0; j < n; ++j) {
                    const double av = A[i + (long)j * n];
#pragma unroll
                    for (int c = 0; c < BAT_MAXRHS; ++c)
                        if (c < nrhs) acc[c] = fma(-av, X[j + (long)c * n], acc[c]);
                }
#pragma unroll
                for (int c = 0; c < BAT_MAXRHS; ++c)
                    if (c < nrhs) R[i + (long)c * n] = acc[c];
            }
            __syncthreads();
            // backward error per right-hand side, max over them
            double w = 0.0;
            for (int c = 0; c < nrhs; ++c) {
                double rm = 0, xm = 0, bm = 0;
                for (int i = tid; i < n; i += BAT_THREADS) {
                    rm = fmax(rm, fabs(R[i + (long)c * n]));
                    xm = fmax(xm, fabs(X[i + (long)c * n]));
                    bm = fmax(bm, fabs(B[i + (long)c * n]));
                }
                for (int o = 16; o > 0; o >>= 1) {
                    rm = fmax(rm, __shfl_xor_sync(0xffffffffu, rm, o));
                    xm = fmax(xm, __shfl_xor_sync(0xffffffffu, xm, o));
                    bm = fmax(bm, __shfl_xor_sync(0xffffffffu, bm, o));
                }
                if ((tid & 31) == 0) {
                    s_red[0][tid >> 5] = rm;
                    s_red[1][tid >> 5] = xm;
                    s_red[2][tid >> 5] = bm;
                }
                __syncthreads();
                if (tid == 0) {
                    for (int q = 1; q < BAT_THREADS / 32; ++q) {
                        rm = fmax(rm, s_red[0][q]);
                        xm = fmax(xm, s_red[1][q]);
                        bm = fmax(bm, s_red[2][q]);
                    }
                    const double den = s_anorm * xm + bm;
                    const double e = den > 0 ? rm / den : (rm > 0 ? INFINITY : 0.0);
                    s_red[3][0] = fmax(c == 0 ? 0.0 : s_red[3][0], e);
                }
                __syncthreads();
            }
            w = s_red[3][0];
            worst = w;
            if (tid == 0) s_done = (w <= a.tol) || it >= a.max_iter;
            __syncthreads();
            if (s_done) break;
            __syncthreads();
            for (int idx = tid; idx < n * nrhs; idx += BAT_THREADS) Y[idx] = (float)R[idx];
            __syncthreads();
            bat_potrs(W, n, Y, nrhs);
            for (int idx = tid; idx < n * nrhs; idx += BAT_THREADS) X[idx] += (double)Y[idx];
            __syncthreads();
        }
        if (tid == 0) {
            a.status[sys] = (worst <= a.tol) ? it : -1000;
            a.berr[sys] = worst;
        }
        __syncthreads();
    }
}

} // namespace gb300
