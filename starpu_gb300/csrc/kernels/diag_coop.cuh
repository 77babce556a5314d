// One cooperative launch that factors an FP32 diagonal tile of order
// n <= 1024 (lower Cholesky, in place) and writes its lower-triangular
// inverse: the POTRF of the mixed solve's diagonal tile and the operand of
// its tensor-core panel TRSM (P <- P L_kk^-T as P * Linv^T).
//
// The tile is handled in 64 x 64 blocks, right-looking, as the tile loop of
// examples/cholesky/cholesky_implicit.c:244-318 with the POTRF/TRSM/SYRK/GEMM
// codelet arithmetic of cholesky_kernels.c (unblocked POTRF leaf: scale by
// 1/l_zz, rank-1 update; column-oriented TRSM; GEMM updates).  Step k:
//   A  every CTA with a block row i >= k loads the diagonal block and factors
//      it in shared memory (the same instructions in every CTA, so every copy
//      is bit-identical); the CTA of row k stores it and inverts it, the
//      others solve their block L_ik = A_ik L_kk^-T;
//   B  the trailing blocks A_ij -= L_ik L_jk^T (k < j <= i) are spread over
//      the grid.
// The inverse X = L^-1 is built on the way, block row by block row from
// L X = I:  X_kj = -X_kk sum_{p=j}^{k-1} L_kp X_pj.  The products of row k
// run in phase B of step k, their sums and the X_kk multiply in phase A of
// step k+1, both in CTAs the factorisation leaves idle; only the last block
// row follows the factorisation.
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
constexpr int DC_LD = DC_B + 4;  // pitch of a shared tile (column-major: s[c * DC_LD + r]); float4-aligned
constexpr int DC_MAXN = 1024;
constexpr int DC_ERR_TIMEOUT = 4;  // *err code of a barrier wait that ran out
constexpr uint64_t DC_WAIT_NS = 1000000000ull;

struct DiagCoopArgs {
    int n;
    float *A;
    long lda;
    float *Linv;  // n x n, strict upper part zeroed by the caller
    long ldi;
    float *T;  // scratch of the inverse's block products: n * n floats
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

// acc += As * Bs for 64 x 64 shared tiles: As column-major (As[p * DC_LD + r]
// = A(r, p)), Bs stored p-major (Bs[p * DC_LD + c] = B(p, c)) -- which is how
// dc_load stores a tile whose transpose is the operand (NT products).
// Thread (tr = tid % 16, tn = tid / 16) owns rows 4 tr .. 4 tr + 3 and
// columns 4 tn .. 4 tn + 3: two float4 shared loads per 16 FMAs.
__device__ __forceinline__ void dc_mma(const float *As, const float *Bs, float acc[4][4])
{
    const int tr = threadIdx.x & 15, tn = threadIdx.x >> 4;
#pragma unroll 8
    for (int p = 0; p < DC_B; ++p) {
        const float4 av = *reinterpret_cast<const float4 *>(As + p * DC_LD + 4 * tr);
        const float4 bv = *reinterpret_cast<const float4 *>(Bs + p * DC_LD + 4 * tn);
        const float ar[4] = {av.x, av.y, av.z, av.w}, br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(ar[i], br[j], acc[i][j]);
    }
}

// rows x cols block of a column-major global matrix into a shared tile
// stored p-major (s[r * DC_LD + c] = g(r, c)), zero outside: the B operand
// of an NN product.
__device__ __forceinline__ void dc_load_t(float *s, const float *g, long ld, int rows, int cols)
{
    for (int e = threadIdx.x; e < DC_B * DC_B; e += DC_T) {
        const int r = e & (DC_B - 1), c = e >> 6;
        s[r * DC_LD + c] = (r < rows && c < cols) ? __ldcg(g + r + (long)c * ld) : 0.0f;
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

// C (rows x cols of a column-major global matrix) -= acc, where the mask
// `lower` keeps only elements on or below the diagonal.  vec: C and ld allow
// float4 accesses along the thread's four rows.
__device__ __forceinline__ void dc_sub_store(float *C, long ld, int rows, int cols, bool lower, bool vec,
                                             const float acc[4][4])
{
    const int tr = threadIdx.x & 15, tn = threadIdx.x >> 4, r0 = 4 * tr;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = 4 * tn + j;
        if (c >= cols) continue;
        float *p = C + r0 + (long)c * ld;
        if (vec && r0 + 3 < rows && (!lower || c <= r0)) {
            float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
            v.x -= acc[0][j];
            v.y -= acc[1][j];
            v.z -= acc[2][j];
            v.w -= acc[3][j];
            *reinterpret_cast<float4 *>(p) = v;
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (r0 + i < rows && (!lower || c <= r0 + i)) p[i] = __ldcg(p + i) - acc[i][j];
        }
    }
}

// The slot of the product L_kp X_pj (64 x 64, ld 64) in the scratch area.
__device__ __forceinline__ float *dc_slot(const DiagCoopArgs &a, int j, int p)
{
    return a.T + (long)(p * (p + 1) / 2 + j) * (DC_B * DC_B);
}

// slot(j, p) = L_kp X_pj (rows of block row k: rk), X_pj the inverse block
__device__ __forceinline__ void dc_inv_product(const DiagCoopArgs &a, int k, int j, int p, float *s0, float *s1)
{
    const int rk = min(DC_B, a.n - k * DC_B);
    __syncthreads();  // shared tiles free
    dc_load(s0, a.A + k * DC_B + (long)(p * DC_B) * a.lda, a.lda, rk, DC_B);
    dc_load_t(s1, a.Linv + p * DC_B + (long)(j * DC_B) * a.ldi, a.ldi, DC_B, DC_B);
    __syncthreads();
    float acc[4][4] = {};
    dc_mma(s0, s1, acc);
    const int tr = threadIdx.x & 15, tn = threadIdx.x >> 4;
    float *S = dc_slot(a, j, p);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj)
        *reinterpret_cast<float4 *>(S + 4 * tr + (4 * tn + jj) * DC_B) =
            make_float4(acc[0][jj], acc[1][jj], acc[2][jj], acc[3][jj]);
}

// X_kj = -X_kk (sum_{p = j}^{k-1} slot(j, p)), summed in p order
__device__ __forceinline__ void dc_inv_combine(const DiagCoopArgs &a, int k, int j, float *s0, float *s1)
{
    const int rk = min(DC_B, a.n - k * DC_B);
    __syncthreads();  // shared tiles free
    for (int e = threadIdx.x; e < DC_B * DC_B; e += DC_T) {
        float v = 0.0f;
        for (int p = j; p < k; ++p) v += __ldcg(dc_slot(a, j, p) + e);
        s1[(e & (DC_B - 1)) * DC_LD + (e >> 6)] = v;
    }
    dc_load(s0, a.Linv + k * DC_B + (long)(k * DC_B) * a.ldi, a.ldi, rk, rk);
    __syncthreads();
    float acc[4][4] = {};
    dc_mma(s0, s1, acc);
    const int tr = threadIdx.x & 15, tn = threadIdx.x >> 4;
    float *X = a.Linv + k * DC_B + (long)(j * DC_B) * a.ldi;
#pragma unroll
    for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (4 * tr + i < rk) X[4 * tr + i + (long)(4 * tn + jj) * a.ldi] = -acc[i][jj];
}

// ---------------------------------------------------------------------------
// The kernel.  Step k, phase A: the tasks t = blockIdx.x, + gridDim.x, ...
// of [factor block rows k .. nblk-1 | combine row k-1 of the inverse];
// phase B: [trailing tile updates | products of row k of the inverse].  The
// inverse is built row by row as X_kj = -X_kk sum_{p=j}^{k-1} L_kp X_pj
// (L X = I, block row k), in CTAs the factorisation leaves idle; only the
// last row runs after the factorisation.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(DC_T) diag_coop_kernel(DiagCoopArgs a)
{
    __shared__ __align__(16) float s0[DC_B * DC_LD];
    __shared__ __align__(16) float s1[DC_B * DC_LD];
    __shared__ float invd[DC_B];
    __shared__ int s_ok;
    const int n = a.n, nblk = (n + DC_B - 1) / DC_B, G = gridDim.x, b = blockIdx.x;
    const int tid = threadIdx.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(a.A) & 15) == 0) && ((a.lda & 3) == 0);
    unsigned phase = 0;

    for (int k = 0; k < nblk; ++k) {
        const int k0 = k * DC_B, bk = min(DC_B, n - k0);
        float *Akk = a.A + k0 + (long)k0 * a.lda;
        // ---- phase A
        const int nf = nblk - k, nc = (a.invert && k >= 2) ? k - 1 : 0;
        bool factored = false;
        for (int t = b; t < nf + nc; t += G) {
            if (t < nf) {
                if (!factored) {
                    dc_load(s0, Akk, a.lda, bk, bk);
                    __syncthreads();
                    dc_potf2(s0, bk, invd, a.info, a.info_base + k0, b == 0);
                    factored = true;
                }
                const int i = k + t;
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
            } else {
                dc_inv_combine(a, k - 1, t - nf, s0, s1);  // factor tasks come first: s0 is free
            }
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
        if (k == nblk - 1) break;
        // ---- phase B
        const int m = nblk - k - 1, nu = m * (m + 1) / 2;
        const int np = (a.invert && k >= 1) ? k * (k + 1) / 2 : 0;
        for (int t = b; t < nu + np; t += G) {
            if (t < nu) {
                int ii, jj;
                dc_tri_index(t, ii, jj);
                const int bi = k + 1 + ii, bj = k + 1 + jj;
                const int i0 = bi * DC_B, j0 = bj * DC_B, ri = min(DC_B, n - i0), rj = min(DC_B, n - j0);
                __syncthreads();  // the previous task's shared operands are free
                dc_load(s0, a.A + i0 + (long)k0 * a.lda, a.lda, ri, bk);
                dc_load(s1, a.A + j0 + (long)k0 * a.lda, a.lda, rj, bk);
                __syncthreads();
                float acc[4][4] = {};
                dc_mma(s0, s1, acc);
                dc_sub_store(a.A + i0 + (long)j0 * a.lda, a.lda, ri, rj, bi == bj, vec, acc);
            } else {
                int p, j;
                dc_tri_index(t - nu, p, j);
                dc_inv_product(a, k, j, p, s0, s1);
            }
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
    }

    // ---- the last row of the inverse
    if (a.invert && nblk >= 2) {
        const int k = nblk - 1;
        for (int t = b; t < k * (k + 1) / 2; t += G) {
            int p, j;
            dc_tri_index(t, p, j);
            dc_inv_product(a, k, j, p, s0, s1);
        }
        if (!dc_sync(a, ++phase, &s_ok)) return;
        for (int t = b; t < k; t += G) dc_inv_combine(a, k, t, s0, s1);
    }
}

} // namespace gb300
