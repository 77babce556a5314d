// One cooperative launch that factors an FP32 diagonal tile of order
// n <= 1024 (lower Cholesky, in place) and writes its lower-triangular
// inverse: the POTRF of the mixed solve's diagonal tile and the operand of
// its tensor-core panel TRSM (P <- P L_kk^-T as P * Linv^T).
//
// The tile is handled in 64 x 64 blocks, right-looking, as the tile loop of
// examples/cholesky/cholesky_implicit.c:244-318 with the POTRF/TRSM/SYRK/GEMM
// codelet arithmetic of cholesky_kernels.c (unblocked POTRF leaf: sqrt, scale
// by 1/l_zz, rank-1 update; column-oriented TRSM; GEMM updates).  Step k:
//   A  every CTA of block row i >= k loads the diagonal block, factors it in
//      shared memory (the same instructions in every CTA, so every copy is
//      bit-identical), then the CTA of row k stores it and inverts it while
//      the others solve their block L_ik = A_ik L_kk^-T;
//   B  the trailing blocks A_ij -= L_ik L_jk^T (k < j <= i) are spread over
//      the grid.
// Then the inverse of the whole tile by doubling: for h = 64, 128, ...,
// [L11 0; L21 L22]^-1 = [I11 0; -I22 L21 I11  I22] on pairs of order-h
// diagonal blocks, T = L21 I11 into scratch, then X21 = -I22 T.
//
// Phases are separated by grid barriers: a launch counter that each CTA
// bumps, waited on with acquire loads.  The launch is cooperative (every CTA
// resident), each wait is bounded by %globaltimer; on a timeout the CTA sets
// *err and returns, and the CTAs still waiting time out in turn.  Data other
// CTAs wrote is read through L2 (ld.global.cg), never from a stale L1 line.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb300 {

__device__ __forceinline__ uint64_t dc_timer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int DC_B = 64;         // block order
constexpr int DC_T = 256;        // threads per CTA
constexpr int DC_LD = DC_B + 1;  // pitch of a shared tile (column-major: s[c * DC_LD + r])
constexpr int DC_MAXN = 1024;
constexpr int DC_ERR_TIMEOUT = 4;  // *err code of a barrier wait that ran out
constexpr uint64_t DC_WAIT_NS = 1000000000ull;

struct DiagCoopArgs {
    int n;
    float *A;
    long lda;
    float *Linv;  // n x n, strict upper part zeroed by the caller
    long ldi;
    float *T;  // scratch of the doubling products: n * n floats
    int *info;
    int info_base;
    unsigned *bar;  // barrier counter, zero at launch
    int *err;
    int invert;  // 0: factor only (no inverse is written)
};

__device__ __forceinline__ unsigned dc_ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier number `phase` (1, 2, ...).  False: a wait timed out here or
// another CTA has flagged an error -- the caller returns.
__device__ __forceinline__ bool dc_sync(const DiagCoopArgs &a, unsigned phase, int *s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        atomicAdd(a.bar, 1u);
        const unsigned target = phase * gridDim.x;
        if (dc_ld_acquire(a.bar) < target) {
            const uint64_t t0 = dc_timer();
            while (dc_ld_acquire(a.bar) < target) {
                if (*(volatile int *)a.err || dc_timer() - t0 > DC_WAIT_NS) {
                    atomicCAS(a.err, 0, DC_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// rows x cols block of a column-major global matrix into a 64 x 64 shared
// tile, zero outside.
__device__ __forceinline__ void dc_load(float *s, const float *g, long ld, int rows, int cols)
{
    for (int e = threadIdx.x; e < DC_B * DC_B; e += DC_T) {
        const int r = e & (DC_B - 1), c = e >> 6;
        s[c * DC_LD + r] = (r < rows && c < cols) ? __ldcg(g + r + (long)c * ld) : 0.0f;
    }
}

// Cholesky of the nb x nb (nb <= 32) lower block of D at offset `off`, in
// place, by one warp: lane i holds row i in registers, the step loop is
// unrolled (static register indices) and column values travel by shuffles,
// so no CTA barrier sits on the chain.  Lanes i >= nb hold identity rows.
// 1/l_zz comes from rsqrtf: this factor is the mixed solve's FP32 working
// factor, refined afterwards, so the last ulp of the pivots does not matter.
// invd[i] = 1 / l_ii.  The first non-positive pivot sets *info (first wins).
__device__ __noinline__ void dc_potf2_32(float *D, int off, int nb, float *invd, int *info, int info_base,
                                            bool report)
{
    const unsigned FULL = 0xffffffffu;
    const int i = threadIdx.x & 31;
    float a[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) a[c] = (i < nb) ? ((c <= i) ? D[off + c * DC_LD + i] : 0.0f) : (c == i ? 1.0f : 0.0f);
    int badz = -1;
    float myinv = 1.0f;
#pragma unroll
    for (int z = 0; z < 32; ++z) {
        const float d = __shfl_sync(FULL, a[z], z);
        if (!(d > 0.0f) && badz < 0) badz = z;
        const float inv = rsqrtf(d);
        const float li = a[z] * inv;
        if (i == z) {
            a[z] = d * inv;
            myinv = inv;
        } else if (i > z) {
            a[z] = li;
        }
#pragma unroll
        for (int c = z + 1; c < 32; ++c) {
            const float lc = __shfl_sync(FULL, li, c);
            if (i >= c) a[c] = fmaf(-li, lc, a[c]);
        }
    }
    if (i < nb) {
#pragma unroll
        for (int c = 0; c < 32; ++c)
            if (c <= i) D[off + c * DC_LD + i] = a[c];
    }
    invd[i] = myinv;
    if (report && i == 0 && badz >= 0 && badz < nb && info) atomicCAS(info, 0, info_base + badz + 1);
}

// Cholesky of the bk x bk (bk <= 64) lower block in D (shared), in place:
// 32 x 32 blocks -- warp 0 factors L11, warp 1 solves L21 = A21 L11^-T (lane
// = row, unrolled column-oriented substitution), the CTA updates
// A22 -= L21 L21^T, warp 0 factors L22.  invd[j] = 1 / l_jj (1 for j >= bk).
__device__ __forceinline__ void dc_potf2(float *D, int bk, float *invd, int *info, int info_base, bool report)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) dc_potf2_32(D, 0, min(bk, 32), invd, info, info_base, report);
    __syncthreads();
    if (bk > 32) {
        if (warp == 1) {
            const int r = 32 + lane;
            float x[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) x[c] = D[c * DC_LD + r];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                x[j] *= invd[j];
#pragma unroll
                for (int c = j + 1; c < 32; ++c) x[c] = fmaf(-D[j * DC_LD + c], x[j], x[c]);
            }
            if (r < bk) {
#pragma unroll
                for (int c = 0; c < 32; ++c) D[c * DC_LD + r] = x[c];
            }
        }
        __syncthreads();
        for (int e = tid; e < 32 * 32; e += DC_T) {
            const int r = 32 + (e & 31), c = 32 + (e >> 5);
            if (c <= r && r < bk) {
                float acc = D[c * DC_LD + r];
#pragma unroll 8
                for (int p = 0; p < 32; ++p) acc = fmaf(-D[p * DC_LD + r], D[p * DC_LD + c], acc);
                D[c * DC_LD + r] = acc;
            }
        }
        __syncthreads();
        if (warp == 0) dc_potf2_32(D, 32 * DC_LD + 32, bk - 32, invd + 32, info, info_base + 32, report);
    } else if (tid >= 32 && tid < 64) {
        invd[tid] = 1.0f;
    }
    __syncthreads();
}

// Forward substitution with the factored 64 x 64 block L in D, one system
// per group of four lanes: lane l of the group holds entries 16 l .. 16 l + 15
// of the group's vector x, which on return is L^-1 x (column-oriented:
// x_j *= 1/l_jj, then x_c -= l_cj x_j for c > j).  The owner of x_j is lane
// j / 16, its register j % 16 (a static index: j runs as 4 rolled groups of
// 16 unrolled steps); x_j reaches the other lanes by a shuffle.
__device__ __forceinline__ void dc_fwd_subst(const float *D, const float *invd, float x[16])
{
    const int l = threadIdx.x & 3, src0 = threadIdx.x & 28;
#pragma unroll 1
    for (int G = 0; G < 4; ++G) {
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
            const int j = 16 * G + jj;
            const float xo = x[jj] * invd[j];
            if (l == G) x[jj] = xo;
            const float xj = __shfl_sync(0xffffffffu, xo, src0 | G);
            const float *Dj = D + j * DC_LD + 16 * l;
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (l > G || (l == G && q > jj)) x[q] = fmaf(-Dj[q], xj, x[q]);
        }
    }
}

// Bs (64 rows, bk columns, shared) <- Bs L^-T with L the factored block in D:
// row r of Bs is the system of lane group r (threads 4r .. 4r + 3).
__device__ __forceinline__ void dc_trsm(const float *D, float *Bs, const float *invd)
{
    const int r = threadIdx.x >> 2, l = threadIdx.x & 3;
    float x[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) x[q] = Bs[(16 * l + q) * DC_LD + r];
    dc_fwd_subst(D, invd, x);
#pragma unroll
    for (int q = 0; q < 16; ++q) Bs[(16 * l + q) * DC_LD + r] = x[q];
    __syncthreads();
}

// X = L^-1 of the factored bk x bk block in D, written to the global block g
// (ld ldg, lower part only): column c of X solves L x = e_c in lane group c.
__device__ __forceinline__ void dc_trtri(const float *D, int bk, const float *invd, float *g, long ldg)
{
    const int c = threadIdx.x >> 2, l = threadIdx.x & 3;
    float x[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) x[q] = (16 * l + q == c) ? 1.0f : 0.0f;
    dc_fwd_subst(D, invd, x);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int r = 16 * l + q;
        if (r < bk && c < bk && r >= c) g[r + (long)c * ldg] = x[q];
    }
}

// acc (thread's 4 x 4 of a 64 x 64 tile) += As * op(Bs): As 64 x 64, Bs
// 64 x 64 read as B (NN) or B^T (NT).  Thread (tr = tid % 16, tn = tid / 16)
// owns rows tr + 16 a and columns tn + 16 b.
template <bool NT>
__device__ __forceinline__ void dc_mma(const float *As, const float *Bs, float acc[4][4])
{
    const int tr = threadIdx.x & 15, tn = threadIdx.x >> 4;
#pragma unroll 4
    for (int p = 0; p < DC_B; ++p) {
        float av[4], bv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) av[a] = As[p * DC_LD + tr + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) bv[b] = NT ? Bs[p * DC_LD + tn + 16 * b] : Bs[(tn + 16 * b) * DC_LD + p];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
    }
}

// row index ii, column index jj <= ii of the t-th block of a lower triangle
// (row by row: (0,0), (1,0), (1,1), (2,0), ...)
__device__ __forceinline__ void dc_tri_index(int t, int &ii, int &jj)
{
    int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    ii = i;
    jj = t - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(DC_T) diag_coop_kernel(DiagCoopArgs a)
{
    __shared__ float s0[DC_B * DC_LD], s1[DC_B * DC_LD];
    __shared__ float invd[DC_B];
    __shared__ int s_ok;
    const int n = a.n, nblk = (n + DC_B - 1) / DC_B;
    const int tid = threadIdx.x, tr = tid & 15, tn = tid >> 4;
    unsigned phase = 0;

    for (int k = 0; k < nblk; ++k) {
        const int k0 = k * DC_B, bk = min(DC_B, n - k0);
        // ---- A: diagonal block and the block rows i = k + blockIdx.x, + gridDim.x, ... below it
        if (k + (int)blockIdx.x < nblk) {
            float *Akk = a.A + k0 + (long)k0 * a.lda;
            dc_load(s0, Akk, a.lda, bk, bk);
            __syncthreads();
            dc_potf2(s0, bk, invd, a.info, a.info_base + k0, blockIdx.x == 0);
            for (int i = k + (int)blockIdx.x; i < nblk; i += gridDim.x) {
                if (i == k) {
                    for (int e = tid; e < DC_B * DC_B; e += DC_T) {
                        const int r = e & 63, c = e >> 6;
                        if (r < bk && c <= r) Akk[r + (long)c * a.lda] = s0[c * DC_LD + r];
                    }
                    if (a.invert) dc_trtri(s0, bk, invd, a.Linv + k0 + (long)k0 * a.ldi, a.ldi);
                } else {
                    const int i0 = i * DC_B, ri = min(DC_B, n - i0);
                    float *Aik = a.A + i0 + (long)k0 * a.lda;
                    __syncthreads();  // s1 of the previous block row has been stored
                    dc_load(s1, Aik, a.lda, ri, bk);
                    __syncthreads();
                    dc_trsm(s0, s1, invd);
                    for (int e = tid; e < DC_B * DC_B; e += DC_T) {
                        const int r = e & 63, c = e >> 6;
                        if (r < ri && c < bk) Aik[r + (long)c * a.lda] = s1[c * DC_LD + r];
                    }
                }
            }
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
        if (k == nblk - 1) break;
        // ---- B: trailing update of the blocks (i, j), k < j <= i
        const int m = nblk - k - 1, ntiles = m * (m + 1) / 2;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            int ii, jj;
            dc_tri_index(t, ii, jj);
            const int bi = k + 1 + ii, bj = k + 1 + jj;
            const int i0 = bi * DC_B, j0 = bj * DC_B, ri = min(DC_B, n - i0), rj = min(DC_B, n - j0);
            __syncthreads();  // the previous tile's shared operands are free
            dc_load(s0, a.A + i0 + (long)k0 * a.lda, a.lda, ri, bk);
            dc_load(s1, a.A + j0 + (long)k0 * a.lda, a.lda, rj, bk);
            __syncthreads();
            float acc[4][4] = {};
            dc_mma<true>(s0, s1, acc);
            float *Cij = a.A + i0 + (long)j0 * a.lda;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int c = tn + 16 * b;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = tr + 16 * q;
                    if (r < ri && c < rj && (bi != bj || c <= r)) {
                        float *p = Cij + r + (long)c * a.lda;
                        *p = __ldcg(p) - acc[q][b];
                    }
                }
            }
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
    }

    // ---- inverse of the whole tile by doubling
    for (int h = DC_B; a.invert && h < n; h *= 2) {
        const int th = h / DC_B;
        const int npairs = (n - h + 2 * h - 1) / (2 * h);  // pairs whose second half starts below n
        // stage 1: T_p = L21 I11 (r2 x h), tiles (ta, tb); I11's block (c, tb) is zero for c < tb
        int tiles = 0;
        for (int p = 0; p < npairs; ++p) tiles += ((min(h, n - (2 * p + 1) * h) + DC_B - 1) / DC_B) * th;
        for (int u = blockIdx.x; u < tiles; u += gridDim.x) {
            int p = 0, rem = u, r2 = 0, tr2 = 0;
            for (;; ++p) {
                r2 = min(h, n - (2 * p + 1) * h);
                tr2 = (r2 + DC_B - 1) / DC_B;
                if (rem < tr2 * th) break;
                rem -= tr2 * th;
            }
            const int ta = rem % tr2, tb = rem / tr2, o = 2 * p * h;
            const int rows = min(DC_B, r2 - ta * DC_B);
            float acc[4][4] = {};
            for (int c = tb; c < th; ++c) {
                __syncthreads();
                dc_load(s0, a.A + (o + h + ta * DC_B) + (long)(o + c * DC_B) * a.lda, a.lda, rows, DC_B);
                dc_load(s1, a.Linv + (o + c * DC_B) + (long)(o + tb * DC_B) * a.ldi, a.ldi, DC_B, DC_B);
                __syncthreads();
                dc_mma<false>(s0, s1, acc);
            }
            float *Tp = a.T + (long)p * h * h;  // r2 x h, ld h
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = ta * DC_B + tr + 16 * q, cc = tb * DC_B + tn + 16 * b;
                    if (r < r2) Tp[r + (long)cc * h] = acc[q][b];
                }
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
        // stage 2: X21 = -I22 T_p into Linv; I22's block (ta, c) is zero for c > ta
        for (int u = blockIdx.x; u < tiles; u += gridDim.x) {
            int p = 0, rem = u, r2 = 0, tr2 = 0;
            for (;; ++p) {
                r2 = min(h, n - (2 * p + 1) * h);
                tr2 = (r2 + DC_B - 1) / DC_B;
                if (rem < tr2 * th) break;
                rem -= tr2 * th;
            }
            const int ta = rem % tr2, tb = rem / tr2, o = 2 * p * h;
            const int rows = min(DC_B, r2 - ta * DC_B);
            const float *Tp = a.T + (long)p * h * h;
            float acc[4][4] = {};
            for (int c = 0; c <= ta; ++c) {
                const int kc = min(DC_B, r2 - c * DC_B);
                __syncthreads();
                dc_load(s0, a.Linv + (o + h + ta * DC_B) + (long)(o + h + c * DC_B) * a.ldi, a.ldi, rows, kc);
                dc_load(s1, Tp + c * DC_B + (long)(tb * DC_B) * h, h, kc, DC_B);
                __syncthreads();
                dc_mma<false>(s0, s1, acc);
            }
            float *X = a.Linv + (o + h + ta * DC_B) + (long)(o + tb * DC_B) * a.ldi;
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = tr + 16 * q, cc = tn + 16 * b;
                    if (r < rows) X[r + (long)cc * a.ldi] = -acc[q][b];
                }
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
    }
}

} // namespace gb300
