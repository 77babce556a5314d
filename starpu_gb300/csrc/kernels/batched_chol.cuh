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
//     lower-triangular trailing update in 64 x 64 tiles staged in shared memory,
//       on the tensor cores (warp-level TF32 MMAs on split operands)
//   x = fp64(L^-T L^-1 fp32(b)); repeat r = b - A x, berr, x += corr.
//   The residual runs in double-float arithmetic on the FP32 pipe (A split
//   per element, X split once per residual into shared memory, FP64 flush
//   every 128 terms; ~2^-47 relative per block), GB300 issuing FP64 FMAs at
//   ~1/60 of its FP32 rate; with more right-hand sides than the shared
//   memory holds it runs in FP64.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "df_arith.cuh"

namespace gb300 {

constexpr int BAT_THREADS = 256;
constexpr int BAT_MAXN = 1024;
constexpr int BAT_MAXRHS = 8;
constexpr int BAT_TILE = 64;
constexpr int BAT_TP = 72;  // pitch of a staged panel slice row (64 + 8): conflict-free MMA fragment loads

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
    size_t smem_bytes;                // dynamic shared memory of the launch
};

__device__ __forceinline__ int bucket_of(int n)
{
    int b = 0;
    int t = (n + 31) / 32;
    while ((1 << b) < t) ++b;
    return b > 5 ? 5 : b;  // 32, 64, 128, 256, 512, 1024
}

// TF32 split of x: hi = tf32(x) (round to nearest), lo = tf32(x - hi)
__device__ __forceinline__ void bat_split_tf32(float x, uint32_t &hi, uint32_t &lo)
{
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
    const float r = x - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}

// d += a b for one 16 x 8 x 8 TF32 tile (warp-wide, FP32 accumulation)
__device__ __forceinline__ void bat_mma_tf32(float d[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ----------------------------------------------------------------- factor
template <int NB>
__device__ int bat_factor(float *W, int n, float *smem)
{
    float(*D)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(smem);   // diagonal block
    float *As = smem + NB * (NB + 1);                                  // [NB][BAT_TP] panel slice (k-major)
    float *Bs = As + NB * BAT_TP;                                      // [NB][BAT_TP]
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
        // ---- trailing update of the lower triangle, 64 x 64 tiles, on the
        // tensor cores: warp-level m16n8k8 TF32 MMAs, three per tile on the
        // split x = hi + lo of both operands (about 21 significant bits, the
        // FP32 factor's working accuracy; the refinement recovers FP64).
        // Warp w owns rows 16 (w % 4) .. + 15 and columns 32 (w / 4) .. + 31
        // of the tile (four n8 fragments); K = the block width, padded to 8
        // with zeros.
        const int nt = (m + BAT_TILE - 1) / BAT_TILE;
        const int kp = (kb + 7) & ~7;
        const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
        const int wr = 16 * (warp & 3), wc = 32 * (warp >> 2);
        for (int tj = 0; tj < nt; ++tj) {
            // stage the panel rows of tile column tj once per column
#pragma unroll 4
            for (int idx = tid; idx < kp * BAT_TILE; idx += BAT_THREADS) {
                const int rr = idx % BAT_TILE, p = idx / BAT_TILE;
                const int row = r0 + tj * BAT_TILE + rr;
                Bs[p * BAT_TP + rr] = (p < kb && row < n) ? W[row + (long)(k0 + p) * n] : 0.0f;
            }
            for (int ti2 = tj; ti2 < nt; ++ti2) {
#pragma unroll 4
                for (int idx = tid; idx < kp * BAT_TILE; idx += BAT_THREADS) {
                    const int rr = idx % BAT_TILE, p = idx / BAT_TILE;
                    const int row = r0 + ti2 * BAT_TILE + rr;
                    As[p * BAT_TP + rr] = (p < kb && row < n) ? W[row + (long)(k0 + p) * n] : 0.0f;
                }
                __syncthreads();
                // this thread's 16 elements of the tile, loaded before the products
                float cv[4][4];
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int col = r0 + tj * BAT_TILE + wc + 8 * j + 2 * t4 + (q & 1);
                        const int row = r0 + ti2 * BAT_TILE + wr + g + 8 * (q >> 1);
                        cv[j][q] = (col < n && row < n && row >= col) ? W[row + (long)col * n] : 0.0f;
                    }
                float acc[4][4];
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[j][q] = 0.0f;
                for (int p = 0; p < kp; p += 8) {
                    uint32_t ah[4], al[4];
                    bat_split_tf32(As[(p + t4) * BAT_TP + wr + g], ah[0], al[0]);
                    bat_split_tf32(As[(p + t4) * BAT_TP + wr + g + 8], ah[1], al[1]);
                    bat_split_tf32(As[(p + t4 + 4) * BAT_TP + wr + g], ah[2], al[2]);
                    bat_split_tf32(As[(p + t4 + 4) * BAT_TP + wr + g + 8], ah[3], al[3]);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        uint32_t bh[2], bl[2];
                        bat_split_tf32(Bs[(p + t4) * BAT_TP + wc + 8 * j + g], bh[0], bl[0]);
                        bat_split_tf32(Bs[(p + t4 + 4) * BAT_TP + wc + 8 * j + g], bh[1], bl[1]);
                        bat_mma_tf32(acc[j], al, bh);  // the small terms first
                        bat_mma_tf32(acc[j], ah, bl);
                        bat_mma_tf32(acc[j], ah, bh);
                    }
                }
                // fragment element q of n-tile j: row wr + g + 8 (q / 2), column wc + 8 j + 2 t4 + q % 2
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int col = r0 + tj * BAT_TILE + wc + 8 * j + 2 * t4 + (q & 1);
                        const int row = r0 + ti2 * BAT_TILE + wr + g + 8 * (q >> 1);
                        if (col < n && row < n && row >= col) W[row + (long)col * n] = cv[j][q] - acc[j][q];
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
__device__ void bat_mirror_upper(float *W, int n, float *smem)
{
    // 32 x 32 tiles below the diagonal, transposed through shared memory so
    // that both the reads (down the columns of L) and the writes (down the
    // columns of the upper part) are coalesced; 8 warps, one tile row each
    float(*T)[33] = reinterpret_cast<float(*)[33]>(smem) + (threadIdx.x >> 5) * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nt = (n + 31) / 32;
    for (int t = warp; t < nt * (nt + 1) / 2; t += BAT_THREADS / 32) {
        int ti = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
        while (ti * (ti + 1) / 2 > t) --ti;
        while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
        const int tj = t - ti * (ti + 1) / 2;  // tile (ti, tj), tj <= ti
        const int r0 = 32 * ti, c0 = 32 * tj;
        for (int c = 0; c < 32; ++c)
            T[c][lane] = (r0 + lane < n && c0 + c < n) ? W[r0 + lane + (long)(c0 + c) * n] : 0.0f;
        __syncwarp();
        // W(c0 + lane, r0 + r) = L(r0 + r, c0 + lane) for c0 + lane < r0 + r
        for (int r = 0; r < 32; ++r)
            if (r0 + r < n && c0 + lane < n && c0 + lane < r0 + r) W[c0 + lane + (long)(r0 + r) * n] = T[lane][r];
        __syncwarp();
    }
    __syncthreads();
}

// Y (n x nrhs, ld n) <- L^-T L^-1 Y, in blocks of 32 columns.  Per block,
// the 32 x 32 diagonal block is staged in shared memory (coalesced) and warp
// 0 solves it (lane = row, the solved entry broadcast by shuffles) into
// shared memory; then every thread updates its rows outside the block with
// the block's 32 columns of L (forward) or of L^T (backward, read from the
// mirrored upper triangle), all 32 loads of a row in flight at once.  Each
// row sees its updates in the same column order as a column-by-column
// substitution.
__device__ void bat_potrs(const float *W, int n, float *Y, int nrhs, float *smem)
{
    const int tid = threadIdx.x, lane = tid & 31;
    float(*D)[33] = reinterpret_cast<float(*)[33]>(smem);  // D[c][r] = block (r, c)
    float *ys = smem + 32 * 33;                             // ys[j * BAT_MAXRHS + c]: the solved block
    for (int pass = 0; pass < 2; ++pass) {
        const bool fwd = pass == 0;
        const int nblk = (n + 31) / 32;
        for (int bb = 0; bb < nblk; ++bb) {
            const int j0 = fwd ? 32 * bb : 32 * (nblk - 1 - bb), jb = min(32, n - j0);
            // stage the diagonal block (forward: L, backward: the mirrored U = L^T)
            for (int e = tid; e < 32 * 32; e += BAT_THREADS) {
                const int r = e & 31, c = e >> 5;
                D[c][r] = (r < jb && c < jb) ? W[j0 + r + (long)(j0 + c) * n] : 0.0f;
            }
            __syncthreads();
            if (tid < 32) {
                float y[BAT_MAXRHS];
#pragma unroll
                for (int c = 0; c < BAT_MAXRHS; ++c)
                    y[c] = (c < nrhs && lane < jb) ? Y[j0 + lane + (long)c * n] : 0.0f;
                for (int q = 0; q < jb; ++q) {
                    const int j = fwd ? q : jb - 1 - q;
                    const float l = D[j][lane];  // (lane, j) of the block
                    if (lane == j) {
#pragma unroll
                        for (int c = 0; c < BAT_MAXRHS; ++c) y[c] /= l;
                    }
#pragma unroll
                    for (int c = 0; c < BAT_MAXRHS; ++c) {
                        const float yj = __shfl_sync(0xffffffffu, y[c], j);
                        if (fwd ? lane > j : lane < j) y[c] = fmaf(-l, yj, y[c]);
                    }
                }
                if (lane < jb) {
#pragma unroll
                    for (int c = 0; c < BAT_MAXRHS; ++c) {
                        ys[lane * BAT_MAXRHS + c] = y[c];
                        if (c < nrhs) Y[j0 + lane + (long)c * n] = y[c];
                    }
                }
            }
            __syncthreads();
            // rows outside the block: below it (forward) or above it (backward)
            const int i_lo = fwd ? j0 + jb : 0, i_hi = fwd ? n : j0;
            for (int i = i_lo + tid; i < i_hi; i += BAT_THREADS) {
                float l[32];
#pragma unroll
                for (int q = 0; q < 32; ++q) l[q] = q < jb ? W[i + (long)(j0 + q) * n] : 0.0f;
                float y[BAT_MAXRHS];
#pragma unroll
                for (int c = 0; c < BAT_MAXRHS; ++c) y[c] = c < nrhs ? Y[i + (long)c * n] : 0.0f;
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    const int j = fwd ? q : 31 - q;
                    if (j < jb) {
#pragma unroll
                        for (int c = 0; c < BAT_MAXRHS; ++c) y[c] = fmaf(-l[j], ys[j * BAT_MAXRHS + c], y[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < BAT_MAXRHS; ++c)
                    if (c < nrhs) Y[i + (long)c * n] = y[c];
            }
            __syncthreads();
        }
    }
}

// R = B - A X (n x nrhs) in double-float arithmetic on the FP32 pipe: A
// scaled by 2^-ea (ea = exponent of ||A||_inf, an upper bound of |a_ij|) and
// split per element by bit operations, each column of X scaled by 2^-ex_c
// and split once into shared memory (Xs[k nrhs + c]); per row (one thread)
// and right-hand side an error-free running sum, flushed to FP64 every 128
// terms, in a fixed order (deterministic).
__device__ void bat_residual_df(const double *A, int n, const double *X, const double *B, double *R, int nrhs,
                                double anorm, float *smem)
{
    __shared__ int s_ex[BAT_MAXRHS];
    __shared__ double s_xm[BAT_THREADS / 32];
    const int tid = threadIdx.x;
    float2 *Xs = reinterpret_cast<float2 *>(smem);
    for (int c = 0; c < nrhs; ++c) {
        double m = 0.0;
        for (int k = tid; k < n; k += BAT_THREADS) m = fmax(m, fabs(X[k + (long)c * n]));
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((tid & 31) == 0) s_xm[tid >> 5] = m;
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < BAT_THREADS / 32; ++w) m = fmax(m, s_xm[w]);
            s_ex[c] = df_scale_exp(m);
        }
        __syncthreads();
    }
    for (int e = tid; e < n * nrhs; e += BAT_THREADS) {
        const int k = e / nrhs, c = e - k * nrhs;
        Xs[e] = df_split_scaled(X[k + (long)c * n], s_ex[c]);
    }
    __syncthreads();
    const int ea = df_scale_exp(anorm);
    for (int i = tid; i < n; i += BAT_THREADS) {
        double acc[BAT_MAXRHS];
        float sh[BAT_MAXRHS], sl[BAT_MAXRHS];
#pragma unroll
        for (int c = 0; c < BAT_MAXRHS; ++c) {
            acc[c] = c < nrhs ? B[i + (long)c * n] : 0.0;
            sh[c] = 0.0f;
            sl[c] = 0.0f;
        }
        for (int j0 = 0; j0 < n; j0 += 128) {
            const int j1 = min(n, j0 + 128);
            for (int j = j0; j < j1; j += 8) {
                // eight loads of the row in flight before their products
                double av8[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) av8[u] = j + u < j1 ? A[i + (long)(j + u) * n] : 0.0;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (j + u >= j1) break;
                    const float2 av = df_split_scaled(av8[u], ea);
#pragma unroll
                    for (int c = 0; c < BAT_MAXRHS; ++c)
                        if (c < nrhs) {
                            const float2 xv = Xs[(j + u) * nrhs + c];
                            df_mac(sh[c], sl[c], av.x, av.y, xv.x, xv.y);
                        }
                }
            }
#pragma unroll
            for (int c = 0; c < BAT_MAXRHS; ++c)
                if (c < nrhs) {
                    acc[c] -= ldexp((double)sh[c] + (double)sl[c], ea + s_ex[c]);
                    sh[c] = 0.0f;
                    sl[c] = 0.0f;
                }
        }
#pragma unroll
        for (int c = 0; c < BAT_MAXRHS; ++c)
            if (c < nrhs) R[i + (long)c * n] = acc[c];
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
            for (int j = 0; j < n; j += 8) {
                double v8[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v8[u] = j + u < n ? A[i + (long)(j + u) * n] : 0.0;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    s += fabs(v8[u]);
                    if (j + u < n && i >= j + u) W[i + (long)(j + u) * n] = (float)v8[u];
                }
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
        bat_mirror_upper(W, n, bat_smem);
        // initial solve
        for (int idx = tid; idx < n * nrhs; idx += BAT_THREADS) Y[idx] = (float)B[idx];
        __syncthreads();
        bat_potrs(W, n, Y, nrhs, bat_smem);
        for (int idx = tid; idx < n * nrhs; idx += BAT_THREADS) X[idx] = (double)Y[idx];
        __syncthreads();
        int it = 0;
        double worst = INFINITY;
        // the double-float residual's X split fits the shared memory
        const bool df = (size_t)n * nrhs * sizeof(float2) <= a.smem_bytes;
        for (;; ++it) {
            if (df) {
                bat_residual_df(A, n, X, B, R, nrhs, s_anorm, bat_smem);
            } else
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
            bat_potrs(W, n, Y, nrhs, bat_smem);
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
