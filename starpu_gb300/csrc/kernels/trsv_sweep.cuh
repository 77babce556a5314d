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

// Inverse of the lower-triangular diagonal block i of L (rows/cols i*W ..
// i*W+w-1), column-major with leading dimension ldo, at Linv + i*bstride.
// clip = false: the full W x W block is written, a ragged last block padded
// with the identity; clip = true: only its w x w part.  One CTA per block;
// thread c owns column c of the inverse and runs the forward substitution
// L X = I.
template <typename T, int W>
__global__ void __launch_bounds__(W) invert_diag_blocks_kernel(int n, const T *__restrict__ L, long ldl,
                                                               T *__restrict__ Linv, long ldo, long bstride, bool clip)
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
    T *out = Linv + (long)blockIdx.x * bstride;
    if (!clip || c < w) {
#pragma unroll
        for (int r = 0; r < W; ++r)
            if (!clip || r < w) out[r + (long)c * ldo] = x[r];
    }
}

// ---- 64 x 64 FP32 tiles in shared memory: column-major, 16-byte chunks of a
// column XOR-swizzled by the column index, so that both a warp reading one
// row-element per lane (rows r..r+31 of column p) and 8 lanes reading one
// 4-row chunk each of 8 consecutive columns hit 32 distinct banks.
__device__ __forceinline__ int swz64(int col, int row)
{
    return col * 64 + ((((row >> 2) ^ (col & 15)) << 2) | (row & 3));
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Stage the th x tw tile at G (column-major, ld) into a swizzled 64 x 64 tile,
// zero-filling rows >= th and columns >= tw.  vec: G and ld allow 16-byte
// copies (G 16-byte aligned, ld % 4 == 0) -- asynchronous cp.async, else plain
// loads.  256 threads.
__device__ __forceinline__ void stage_tile64(float *tile, const float *G, long ld, int th, int tw, bool vec)
{
    const int tid = threadIdx.x;
    if (vec) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int q = tid + 256 * k;
            const int col = q >> 4, ch = q & 15;
            const int rows = min(4, th - ch * 4);
            const int bytes = (col < tw && rows > 0) ? rows * 4 : 0;
            const float *src = bytes ? G + ch * 4 + (long)col * ld : G;
            cp_async16(tile + col * 64 + ((ch ^ (col & 15)) << 2), src, bytes);
        }
    } else {
        for (int q = tid; q < 64 * 64; q += 256) {
            const int col = q >> 6, row = q & 63;
            tile[swz64(col, row)] = (row < th && col < tw) ? G[row + (long)col * ld] : 0.0f;
        }
    }
}

// TRANS = false: forward  y_i = Linv_ii (b_i - sum_{j<i} L_ij y_j)
// TRANS = true : backward x_i = Linv_ii^T (y_i - sum_{j>i} L_ji^T x_j)
// FP32, 64-row blocks, B (n x nrhs, nrhs <= 16) overwritten in place.
// flags[nblk] and *ticket must be zero at launch.  256 threads: thread
// (r = tid % 64, g = tid / 64) owns row r, columns 4g .. 4g+3.  The L tile of
// the next block row is copied (cp.async, double-buffered) while the current
// one is waited for and applied; the inverted diagonal block is staged at
// start.  Dynamic shared memory: SWEEP_SMEM bytes.
constexpr int SWEEP_YS = 20;  // row stride of the right-hand-side block: conflict-free float4 rows
constexpr int SWEEP_SMEM = (3 * 64 * 64 + 64 * SWEEP_YS) * 4;

template <bool TRANS>
__global__ void __launch_bounds__(256) trsv_sweep_kernel(int n, int nrhs, const float *__restrict__ L, long ldl,
                                                         const float *__restrict__ Linv, float *B, long ldb,
                                                         unsigned *ticket, int *flags, int *err,
                                                         unsigned long long budget_ns)
{
    extern __shared__ __align__(16) float sm[];
    float *tiles = sm;                  // 2 x 64 x 64, swizzled
    float *linv = sm + 2 * 64 * 64;     // 64 x 64, swizzled
    float *ys = sm + 3 * 64 * 64;       // 64 rows x 16 columns, row-major, row stride SWEEP_YS
    __shared__ unsigned s_ticket;
    __shared__ int s_skip;
    const int tid = threadIdx.x;
    const int nblk = (n + 63) / 64;
    if (tid == 0) {
        s_ticket = atomicAdd(ticket, 1u);
        s_skip = 0;
    }
    __syncthreads();
    const int t = (int)s_ticket;
    if (t >= nblk) return;
    const int bi = TRANS ? (nblk - 1 - t) : t;
    const int r0 = bi * 64;
    const int wr = min(64, n - r0);
    const int r = tid & 63, g = tid >> 6;
    const bool vec = ((reinterpret_cast<uintptr_t>(L) & 15) == 0) && (ldl % 4 == 0);

    // group 0: the inverted diagonal block (64 x 64 contiguous, 16-byte aligned)
    stage_tile64(linv, Linv + (long)bi * 64 * 64, 64, 64, 64, true);
    cp_async_commit();
    auto tile_of = [&](int s, float *dst) {
        const int bj = TRANS ? (nblk - 1 - s) : s;
        const int c0 = bj * 64, wc = min(64, n - c0);
        if (TRANS) stage_tile64(dst, L + c0 + (long)r0 * ldl, ldl, wc, wr, vec);
        else stage_tile64(dst, L + r0 + (long)c0 * ldl, ldl, wr, wc, vec);
    };
    // group 1: the first off-diagonal tile
    if (t > 0) tile_of(0, tiles);
    cp_async_commit();

    float acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = g * 4 + q;
        acc[q] = (r < wr && c < nrhs) ? B[(long)(r0 + r) + (long)c * ldb] : 0.0f;
    }

    for (int s = 0; s < t; ++s) {
        const int bj = TRANS ? (nblk - 1 - s) : s;
        const int c0 = bj * 64, wc = min(64, n - c0);
        if (tid == 0 && !s_skip && ld_acquire(&flags[bj]) == 0) {
            const uint64_t t0 = gtimer();
            while (ld_acquire(&flags[bj]) == 0) {
                if (*(volatile int *)err || gtimer() - t0 > budget_ns) {
                    atomicCAS(err, 0, 1);
                    s_skip = 1;
                    break;
                }
            }
        }
        __syncthreads();  // flag seen; the previous block's tile and ys are free
        if (s + 1 < t) tile_of(s + 1, tiles + ((s + 1) & 1) * 64 * 64);
        cp_async_commit();
        float yv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = g * 4 + q;
            yv[q] = (r < wc && c < nrhs) ? __ldcg(&B[(long)(c0 + r) + (long)c * ldb]) : 0.0f;
        }
        *reinterpret_cast<float4 *>(&ys[r * SWEEP_YS + g * 4]) = make_float4(yv[0], yv[1], yv[2], yv[3]);
        cp_async_wait<1>();  // everything but the tile just requested: this block's tile
        __syncthreads();
        const float *T = tiles + (s & 1) * 64 * 64;
        if (!TRANS) {
#pragma unroll 16
            for (int p = 0; p < 64; ++p) {
                const float l = T[swz64(p, r)];
                const float4 y = *reinterpret_cast<const float4 *>(&ys[p * SWEEP_YS + g * 4]);
                acc[0] = fmaf(-l, y.x, acc[0]);
                acc[1] = fmaf(-l, y.y, acc[1]);
                acc[2] = fmaf(-l, y.z, acc[2]);
                acc[3] = fmaf(-l, y.w, acc[3]);
            }
        } else {
#pragma unroll 4
            for (int pc = 0; pc < 16; ++pc) {
                const float4 l4 = *reinterpret_cast<const float4 *>(&T[r * 64 + ((pc ^ (r & 15)) << 2)]);
                const float lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float4 y = *reinterpret_cast<const float4 *>(&ys[(pc * 4 + e) * SWEEP_YS + g * 4]);
                    acc[0] = fmaf(-lv[e], y.x, acc[0]);
                    acc[1] = fmaf(-lv[e], y.y, acc[1]);
                    acc[2] = fmaf(-lv[e], y.z, acc[2]);
                    acc[3] = fmaf(-lv[e], y.w, acc[3]);
                }
            }
        }
    }

    // diagonal block: out = Linv * acc (forward) or Linv^T * acc (backward)
    __syncthreads();
    *reinterpret_cast<float4 *>(&ys[r * SWEEP_YS + g * 4]) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    cp_async_wait<0>();
    __syncthreads();
    float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (!TRANS) {
#pragma unroll 16
        for (int p = 0; p < 64; ++p) {
            const float l = linv[swz64(p, r)];
            const float4 y = *reinterpret_cast<const float4 *>(&ys[p * SWEEP_YS + g * 4]);
            out[0] = fmaf(l, y.x, out[0]);
            out[1] = fmaf(l, y.y, out[1]);
            out[2] = fmaf(l, y.z, out[2]);
            out[3] = fmaf(l, y.w, out[3]);
        }
    } else {
#pragma unroll 4
        for (int pc = 0; pc < 16; ++pc) {
            const float4 l4 = *reinterpret_cast<const float4 *>(&linv[r * 64 + ((pc ^ (r & 15)) << 2)]);
            const float lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float4 y = *reinterpret_cast<const float4 *>(&ys[(pc * 4 + e) * SWEEP_YS + g * 4]);
                out[0] = fmaf(lv[e], y.x, out[0]);
                out[1] = fmaf(lv[e], y.y, out[1]);
                out[2] = fmaf(lv[e], y.z, out[2]);
                out[3] = fmaf(lv[e], y.w, out[3]);
            }
        }
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
