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

// Unblocked Cholesky of the bk x bk lower block in D (shared), in place.
// Thread (ti = row, tc = tid / 64) keeps row ti, columns tc, tc + 4, ... in
// registers; column z is published through a double-buffered shared vector,
// one barrier per step.  A non-positive pivot sets info (first wins) when
// `report`.  invd[j] = 1 / l_jj on return.
__device__ __forceinline__ void dc_potf2(float *D, int bk, float *colbuf, float *invd, int *info, int info_base,
                                         bool report)
{
    const int tid = threadIdx.x, ti = tid & 63, tc = tid >> 6;
    float a[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int c = tc + 4 * q;
        a[q] = (ti < bk && c <= ti) ? D[c * DC_LD + ti] : 0.0f;
    }
    bool bad = false;
    for (int z = 0; z < bk; ++z) {
        float *cz = colbuf + (z & 1) * DC_B;
        const int qz = z >> 2;
        if (tc == (z & 3)) {
            float v = a[0];
#pragma unroll
            for (int q = 1; q < 16; ++q)
                if (q == qz) v = a[q];
            cz[ti] = v;
        }
        __syncthreads();
        const float d = cz[z];
        if (!(d > 0.0f) && !bad) {
            bad = true;
            if (report && tid == 0 && info) atomicCAS(info, 0, info_base + z + 1);
        }
        const float lzz = sqrtf(d);
        const float inv = 1.0f / lzz;
        const float li = cz[ti] * inv;
        if (tc == (z & 3) && ti >= z) {
            const float nv = (ti == z) ? lzz : li;
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (q == qz) a[q] = nv;
        }
        if (ti > z) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int c = tc + 4 * q;
                if (c > z && c <= ti) a[q] = fmaf(-li, cz[c] * inv, a[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int c = tc + 4 * q;
        if (ti < bk && c <= ti) D[c * DC_LD + ti] = a[q];
    }
    __syncthreads();
    if (tid < bk) invd[tid] = 1.0f / D[tid * DC_LD + tid];
    __syncthreads();
}

// Bs (rows x bk, shared) <- Bs L^-T, L the factored block in D: every row is
// an independent forward substitution, column-oriented like reference BLAS
// strsm (x_j *= 1/l_jj, then x_c -= l_cj x_j for c > j).  Four lanes per row,
// lane l holding columns l, l + 4, ...; x_j is passed within the lane group.
__device__ __forceinline__ void dc_trsm(const float *D, float *Bs, int bk, const float *invd)
{
    const int tid = threadIdx.x, r = tid >> 2, l = tid & 3, src0 = tid & 28;
    float x[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) x[q] = Bs[(l + 4 * q) * DC_LD + r];
    for (int j = 0; j < bk; ++j) {
        const int qj = j >> 2;
        float xj = 0.0f;
        if (l == (j & 3)) {
            xj = x[0];
#pragma unroll
            for (int q = 1; q < 16; ++q)
                if (q == qj) xj = x[q];
            xj *= invd[j];
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (q == qj) x[q] = xj;
        }
        xj = __shfl_sync(0xffffffffu, xj, src0 | (j & 3));
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int c = l + 4 * q;
            if (c > j) x[q] = fmaf(-D[j * DC_LD + c], xj, x[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) Bs[(l + 4 * q) * DC_LD + r] = x[q];
    __syncthreads();
}

// Lower-triangular inverse X = L^-1 of the factored bk x bk block in D,
// written to the global block g (ld ldg, lower part only): column c of X is
// the forward substitution L x = e_c, four lanes per column.
__device__ __forceinline__ void dc_trtri(const float *D, int bk, const float *invd, float *g, long ldg)
{
    const int tid = threadIdx.x, c = tid >> 2, l = tid & 3, src0 = tid & 28;
    float y[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) y[q] = (l + 4 * q == c) ? 1.0f : 0.0f;
    for (int p = 0; p < bk; ++p) {
        const int qp = p >> 2;
        float xp = 0.0f;
        if (l == (p & 3)) {
            xp = y[0];
#pragma unroll
            for (int q = 1; q < 16; ++q)
                if (q == qp) xp = y[q];
            xp *= invd[p];
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (q == qp) y[q] = xp;
        }
        xp = __shfl_sync(0xffffffffu, xp, src0 | (p & 3));
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int r = l + 4 * q;
            if (r > p) y[q] = fmaf(-D[p * DC_LD + r], xp, y[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int r = l + 4 * q;
        if (r < bk && c < bk && r >= c) g[r + (long)c * ldg] = y[q];
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
    __shared__ float colbuf[2 * DC_B], invd[DC_B];
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
            dc_potf2(s0, bk, colbuf, invd, a.info, a.info_base + k0, blockIdx.x == 0);
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
                    dc_trsm(s0, s1, bk, invd);
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
