// Single-launch triangular sweeps of POTRS (L y = b, then L^T x = y) for up
// to 16 right-hand sides, with explicitly inverted W x W diagonal blocks.
//
// One CTA per block row.  A CTA takes a ticket (atomicAdd) when it starts and
// solves the block row of that rank in solve order, so it only ever waits on
// block rows whose CTAs started before it: the sweep cannot deadlock however
// the hardware schedules CTAs.  Each CTA accumulates the contributions of the
// already-solved block rows as their "done" flags appear (acquire loads, data
// read through L2), multiplies by the inverted diagonal block, stores its
// rows and publishes its own flag (release).  Every wait is bounded by a
// %globaltimer budget; on timeout the CTA records an error, still publishes,
// and the whole launch finishes instead of hanging.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb300 {

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Linv[i] (W x W, column-major, ld W, at Linv + i*W*W) = inverse of the
// lower-triangular diagonal block i of L (rows/cols i*W .. i*W+w-1; a ragged
// last block is padded with the identity).  One CTA per block; thread c owns
// column c of the inverse and runs the forward substitution L X = I.
template <typename T, int W>
__global__ void __launch_bounds__(W) invert_diag_blocks_kernel(int n, const T *__restrict__ L, long ldl,
                                                               T *__restrict__ Linv)
{
    __shared__ T Ls[W][W + 1];
    const int i0 = blockIdx.x * W;
    const int w = min(W, n - i0);
    const int c = threadIdx.x;
    for (int idx = c; idx < W * W; idx += W) {
        const int r = idx % W, q = idx / W;
        T v;
        if (r < w && q < w) v = (r >= q) ? L[(long)(i0 + r) + (long)(i0 + q) * ldl] : T(0);
        else v = (r == q) ? T(1) : T(0);
        Ls[r][q] = v;
    }
    __syncthreads();
    T x[W];
#pragma unroll
    for (int r = 0; r < W; ++r) {
        T s = (r == c) ? T(1) : T(0);
#pragma unroll
        for (int p = 0; p < r; ++p) s = fma(-Ls[r][p], x[p], s);
        x[r] = s / Ls[r][r];
    }
    T *out = Linv + (long)blockIdx.x * W * W;
#pragma unroll
    for (int r = 0; r < W; ++r) out[r + (long)c * W] = x[r];
}

// TRANS = false: forward  y_i = Linv_ii (b_i - sum_{j<i} L_ij y_j)
// TRANS = true : backward x_i = Linv_ii^T (y_i - sum_{j>i} L_ji^T x_j)
// B (n x nrhs, nrhs <= 16) is overwritten in place.  flags[nblk] and
// *ticket must be zero at launch.  256 threads: thread (r = tid % W,
// g = tid / W) owns rows r, columns g*4 .. g*4+3 (W = 64).
template <typename T, int W, bool TRANS>
__global__ void __launch_bounds__(256) trsv_sweep_kernel(int n, int nrhs, const T *__restrict__ L, long ldl,
                                                         const T *__restrict__ Linv, T *B, long ldb,
                                                         unsigned *ticket, int *flags, int *err,
                                                         unsigned long long budget_ns)
{
    static_assert(W == 64, "thread layout assumes 64-row blocks");
    __shared__ T S[W][W + 1];   // staged L tile (rows of the tile = first index)
    __shared__ T Ys[W][16];     // right-hand-side block of a solved block row
    __shared__ unsigned s_ticket;
    __shared__ int s_skip;
    const int tid = threadIdx.x;
    const int nblk = (n + W - 1) / W;
    if (tid == 0) {
        s_ticket = atomicAdd(ticket, 1u);
        s_skip = 0;
    }
    __syncthreads();
    const int t = (int)s_ticket;
    if (t >= nblk) return;
    const int bi = TRANS ? (nblk - 1 - t) : t;
    const int r0 = bi * W;
    const int wr = min(W, n - r0);
    const int r = tid % W, g = tid / W;

    T acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = g * 4 + q;
        acc[q] = (r < wr && c < nrhs) ? B[(long)(r0 + r) + (long)c * ldb] : T(0);
    }

    for (int s = 0; s < t; ++s) {
        const int bj = TRANS ? (nblk - 1 - s) : s;
        const int c0 = bj * W;
        const int wc = min(W, n - c0);
        // stage the L tile: forward L[r0.., c0..] (rows r, cols p); backward L[c0.., r0..] (rows p, cols r)
        const int tr0 = TRANS ? c0 : r0, tc0 = TRANS ? r0 : c0;
        const int th = TRANS ? wc : wr, tw = TRANS ? wr : wc;
        for (int idx = tid; idx < W * W; idx += 256) {
            const int rr = idx % W, cc = idx / W;
            S[rr][cc] = (rr < th && cc < tw) ? L[(long)(tr0 + rr) + (long)(tc0 + cc) * ldl] : T(0);
        }
        if (tid == 0) {
            if (ld_acquire(&flags[bj]) == 0 && !s_skip) {
                const uint64_t t0 = gtimer();
                while (ld_acquire(&flags[bj]) == 0) {
                    if (*(volatile int *)err || gtimer() - t0 > budget_ns) {
                        atomicCAS(err, 0, 1);
                        s_skip = 1;
                        break;
                    }
                }
            }
        }
        __syncthreads();
        for (int idx = tid; idx < W * 16; idx += 256) {
            const int p = idx % W, c = idx / W;
            Ys[p][c] = (p < wc && c < nrhs) ? __ldcg(&B[(long)(c0 + p) + (long)c * ldb]) : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int p = 0; p < W; ++p) {
            const T l = TRANS ? S[p][r] : S[r][p];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fma(-l, Ys[p][g * 4 + q], acc[q]);
        }
        __syncthreads();
    }

    // diagonal block: out = Linv (or Linv^T) * acc
#pragma unroll
    for (int q = 0; q < 4; ++q) Ys[r][g * 4 + q] = acc[q];
    const T *Li = Linv + (long)bi * W * W;
    for (int idx = tid; idx < W * W; idx += 256) {
        const int rr = idx % W, cc = idx / W;
        S[rr][cc] = Li[rr + (long)cc * W];
    }
    __syncthreads();
    T out[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll 8
    for (int p = 0; p < W; ++p) {
        const T l = TRANS ? S[p][r] : S[r][p];
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = fma(l, Ys[p][g * 4 + q], out[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = g * 4 + q;
        if (r < wr && c < nrhs) B[(long)(r0 + r) + (long)c * ldb] = out[q];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(&flags[bi], 1);
}

} // namespace gb300
