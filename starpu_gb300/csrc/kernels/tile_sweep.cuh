// Single-launch triangular sweeps of the mixed solve's FP32 correction solve
// (POTRS with the factor L: L y = b, then L^T x = y) in tile rows of the
// factorisation's tile order nb, with the explicitly inverted nb x nb
// diagonal tiles the factorisation leaves behind.  The chain of dependent
// steps is n / nb long (32 at n = 32768, nb = 1024) instead of n / 64.
//
// Persistent CTAs take tasks by ticket, in solve order.  Tile row u of the
// solve order (u = T forward, T = ntiles - 1 - u backward) has, for each of
// its 32-row slabs s:
//   u products   P_{u,v,s} = L_{slab, tile v} y_v for the earlier tile rows v
//                (backward: (L_{v, slab})^T x_v), each waiting only for tile
//                row v to be solved, written to its own partial block;
//   one diagonal task: z_s = b_s - sum_v P_{u,v,s} (v in order: deterministic),
//                published (Z rows, zcount[u]); once the tile row's z is
//                complete, y_s = (L_TT^-1)_{slab, 0..slab end} z_T (backward
//                the transposed inverse), stored in place of b (ycount[u]).
// Tickets run over the products of tile row u (v ascending, slabs inner),
// then its diagonal tasks, then tile row u + 1.  The products of a tile row
// therefore spread over all CTAs instead of running one after the other in
// the slab's own CTA, and only the product with the newest tile row and the
// diagonal task are on the chain.  A CTA waits only on tasks with smaller
// tickets (already held by running CTAs) or, in a diagonal task, on the other
// diagonal tasks of its tile row, which publish before they wait; with at
// least as many CTAs as slabs per tile row the sweep cannot deadlock however
// CTAs are scheduled.  Every wait is bounded by a %globaltimer budget; on
// timeout the CTA records an error and stops waiting, so the launch ends.
//
// The products are register-blocked: the K range of every chunk (128 columns)
// is split over the 8 warps, each lane keeps 4 rows x 4 right-hand sides, and
// the next two chunks are fetched into registers while the current one is
// used; a task's operand is prefetched into L2 before it waits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb300 {

constexpr int TSW_SLAB = 32;   // rows per CTA
constexpr int TSW_KC = 128;    // K chunk
constexpr int TSW_MP = 36;     // pitch of one K index of the operand chunk (32 rows + 4)
constexpr int TSW_VP = 20;     // pitch of one K index of the right-hand-side chunk (16 + 4)
constexpr int TSW_T = 256;

struct TileSweepArgs {
    int n, nrhs, nb;
    int ntiles, spt;  // tile rows; slabs per tile row (nb / 32)
    unsigned total;   // tasks: spt * ntiles * (ntiles + 1) / 2
    const float *L;
    long ldl;
    const float *Dinv;  // tile T's inverse at Dinv + T * dstride, leading dimension ldd
    long ldd, dstride;
    float *B;  // right-hand sides in, solution out (n x nrhs, ld ldb)
    long ldb;
    float *Z;   // n x 16 scratch, ld n
    float *Zp;  // partial products: pair (u, v < u) at Zp + (u (u - 1) / 2 + v) * nb * 16, slab-major 32 x 16
    unsigned *ticket;
    int *zcount, *ycount, *pcount;  // per tile row of the solve order, zero at launch
    int *err;
    unsigned long long budget_ns;
    int vec;  // L, Dinv, B, Z and their leading dimensions allow 16-byte loads
    // backward sweep: 1 when the strictly upper part of L's storage holds L^T
    // outside the diagonal tiles (L(j, i) also at (i, j)), so the slab's rows
    // of L^T are read column by column like the forward sweep's operands
    int upper;
};

// Bytes of scratch a sweep pair needs: Z (n x 16), the partial products of
// every pair of tile rows, and the 3 ntiles + 1 counters.
inline size_t tsw_scratch_bytes(int n, int nb, size_t *zp_off = nullptr, size_t *cnt_off = nullptr)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t nt = ((size_t)n + nb - 1) / nb;
    const size_t z = al((size_t)n * 16 * sizeof(float));
    const size_t zp = al(nt * (nt > 0 ? nt - 1 : 0) / 2 * (size_t)nb * 16 * sizeof(float));
    if (zp_off) *zp_off = z;
    if (cnt_off) *cnt_off = z + zp;
    return z + zp + al((3 * nt + 1) * sizeof(int));
}

__device__ __forceinline__ int tsw_ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t tsw_timer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait (thread 0, then the CTA) until *cnt >= target.  On timeout or an
// error seen elsewhere the CTA stops waiting from then on (*skip).
__device__ __forceinline__ void tsw_wait(const TileSweepArgs &a, const int *cnt, int target, int *skip)
{
    if (threadIdx.x == 0 && !*skip && tsw_ld_acquire(cnt) < target) {
        const uint64_t t0 = tsw_timer();
        while (tsw_ld_acquire(cnt) < target) {
            if (*(volatile int *)a.err || tsw_timer() - t0 > a.budget_ns) {
                atomicCAS(a.err, 0, 1);
                *skip = 1;
                break;
            }
            __nanosleep(64);
        }
    }
    __syncthreads();
}

// Prefetch into L2 the 32 x K operand a slab is about to multiply (it does
// not depend on the flag the slab waits for, so its HBM latency overlaps the
// wait): TR = false, one 128-byte line of 32 rows per column; TR = true, the
// K consecutive elements of each of the 32 columns.
template <bool TR>
__device__ __forceinline__ void tsw_prefetch_l2(const float *M, long ldm, int rows, int K)
{
    if (!TR) {
        for (int p = threadIdx.x; p < K; p += TSW_T)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(M + (long)p * ldm));
    } else {
        const int lines = (K + 31) / 32;
        for (int e = threadIdx.x; e < rows * lines; e += TSW_T) {
            const int r = e / lines, l = e - r * lines;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(M + (long)r * ldm + 32 * l));
        }
    }
}

// Register-staged chunk of the operand M (32 x kc, element (r, p)) and of the
// right-hand sides V (kc x 16, element (p, c)).
//   TR = false: M(r, p) = M[r + p * ldm]  (rows of L or of the inverse)
//   TR = true : M(r, p) = M[p + r * ldm]  (columns: the transposed operand)
//   V(p, c) = V[p + c * ldv]
struct TswStage {
    float4 m[4];
    float4 v[2];
};

// Element maps (1024 float4 of M, 512 of V per chunk), chosen so that the
// transposing shared stores of tsw_put hit 32 distinct banks:
//   M, TR = false: float4 = 4 consecutive rows r of column p (coalesced rows);
//   M, TR = true : lane = row r, a thread's 4 float4 = 16 consecutive p (two
//                  whole 32-byte sectors of column r);
//   V: lane = (c = lane % 16, half-warp h), float4 f = 16 u + 2 w + h of
//      column c (V is small and stays in L2).
template <bool TR>
__device__ __forceinline__ void tsw_map_m(int u, int &r, int &p)
{
    const int tid = threadIdx.x;
    if (!TR) {
        const int e = tid + TSW_T * u;
        r = (e & 7) * 4;
        p = e >> 3;
    } else {
        r = tid & 31;
        p = ((tid >> 5) * 4 + u) * 4;
    }
}
__device__ __forceinline__ void tsw_map_v(int u, int &p, int &c)
{
    const int tid = threadIdx.x;
    c = tid & 15;
    p = (16 * u + (tid >> 4)) * 4;
}

template <bool TR>
__device__ __forceinline__ void tsw_fetch(TswStage &st, const float *M, long ldm, int rows, const float *V, long ldv,
                                          int kc, int nrhs, bool vec)
{
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        int r, p;
        tsw_map_m<TR>(u, r, p);
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!TR) {
            if (p < kc) {
                const float *src = M + r + (long)p * ldm;
                if (vec && r + 3 < rows) x = __ldcg(reinterpret_cast<const float4 *>(src));
                else {
                    if (r < rows) x.x = __ldcg(src);
                    if (r + 1 < rows) x.y = __ldcg(src + 1);
                    if (r + 2 < rows) x.z = __ldcg(src + 2);
                    if (r + 3 < rows) x.w = __ldcg(src + 3);
                }
            }
        } else {
            if (r < rows) {
                const float *src = M + p + (long)r * ldm;
                if (vec && p + 3 < kc) x = __ldcg(reinterpret_cast<const float4 *>(src));
                else {
                    if (p < kc) x.x = __ldcg(src);
                    if (p + 1 < kc) x.y = __ldcg(src + 1);
                    if (p + 2 < kc) x.z = __ldcg(src + 2);
                    if (p + 3 < kc) x.w = __ldcg(src + 3);
                }
            }
        }
        st.m[u] = x;
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        int p, c;
        tsw_map_v(u, p, c);
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < nrhs) {
            const float *src = V + p + (long)c * ldv;
            if (vec && p + 3 < kc) x = __ldcg(reinterpret_cast<const float4 *>(src));
            else {
                if (p < kc) x.x = __ldcg(src);
                if (p + 1 < kc) x.y = __ldcg(src + 1);
                if (p + 2 < kc) x.z = __ldcg(src + 2);
                if (p + 3 < kc) x.w = __ldcg(src + 3);
            }
        }
        st.v[u] = x;
    }
}

template <bool TR>
__device__ __forceinline__ void tsw_put(const TswStage &st, float *Ms, float *Vs)
{
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        int r, p;
        tsw_map_m<TR>(u, r, p);
        if (!TR) {
            *reinterpret_cast<float4 *>(Ms + p * TSW_MP + r) = st.m[u];
        } else {
            Ms[p * TSW_MP + r] = st.m[u].x;
            Ms[(p + 1) * TSW_MP + r] = st.m[u].y;
            Ms[(p + 2) * TSW_MP + r] = st.m[u].z;
            Ms[(p + 3) * TSW_MP + r] = st.m[u].w;
        }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        int p, c;
        tsw_map_v(u, p, c);
        Vs[p * TSW_VP + c] = st.v[u].x;
        Vs[(p + 1) * TSW_VP + c] = st.v[u].y;
        Vs[(p + 2) * TSW_VP + c] = st.v[u].z;
        Vs[(p + 3) * TSW_VP + c] = st.v[u].w;
    }
}

// acc (this warp's share of the K range) += M(32 x K) V(K x 16).  Warp w
// takes K indices 16 w .. 16 w + 15 of every chunk; lane (rr = lane % 8,
// cc = lane / 8) keeps rows 4 rr .. 4 rr + 3 and right-hand sides
// 4 cc .. 4 cc + 3.
template <bool TR>
__device__ __forceinline__ void tsw_chunk_mma(float acc[4][4], const float *Ms, const float *Vs)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, rr = lane & 7, cc = lane >> 3;
#pragma unroll
    for (int pp = 0; pp < 16; ++pp) {
        const int p = warp * 16 + pp;
        const float4 m4 = *reinterpret_cast<const float4 *>(Ms + p * TSW_MP + 4 * rr);
        const float4 v4 = *reinterpret_cast<const float4 *>(Vs + p * TSW_VP + 4 * cc);
        const float mv[4] = {m4.x, m4.y, m4.z, m4.w}, vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(mv[i], vv[j], acc[i][j]);
    }
}

// acc += M(32 x K) V(K x 16), chunks of 128 K, two chunks in flight: chunk
// c + 2 is fetched into the register set chunk c just left while chunk c is
// multiplied from shared memory (the loop is unrolled by two so that both
// register sets stay statically indexed).
template <bool TR>
__device__ __forceinline__ void tsw_product(float acc[4][4], const float *M, long ldm, int rows, const float *V,
                                            long ldv, int K, int nrhs, bool vec, float *Ms, float *Vs)
{
    if (K <= 0) return;
    auto fetch = [&](TswStage &st, int c) {
        const int p0 = c * TSW_KC;
        const float *Mc = TR ? M + p0 : M + (long)p0 * ldm;
        tsw_fetch<TR>(st, Mc, ldm, rows, V + p0, ldv, min(TSW_KC, K - p0), nrhs, vec);
    };
    const int nch = (K + TSW_KC - 1) / TSW_KC;
    TswStage s0, s1;
    fetch(s0, 0);
    if (nch > 1) fetch(s1, 1);
    for (int c = 0; c < nch; c += 2) {
        __syncthreads();  // the previous chunk has been used
        tsw_put<TR>(s0, Ms, Vs);
        __syncthreads();
        if (c + 2 < nch) fetch(s0, c + 2);
        tsw_chunk_mma<TR>(acc, Ms, Vs);
        if (c + 1 >= nch) break;
        __syncthreads();
        tsw_put<TR>(s1, Ms, Vs);
        __syncthreads();
        if (c + 3 < nch) fetch(s1, c + 3);
        tsw_chunk_mma<TR>(acc, Ms, Vs);
    }
}

// Sum the 8 warps' partial products (plus `base` for warp 0's share, the
// right-hand side) into out (32 x 16, shared, row-major with pitch 16).
__device__ __forceinline__ void tsw_reduce(const float acc[4][4], float *red, float *out)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, rr = lane & 7, cc = lane >> 3;
    __syncthreads();  // red may alias the chunk buffers
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) red[warp * 512 + (4 * rr + i) * 16 + 4 * cc + j] = acc[i][j];
    __syncthreads();
    for (int e = threadIdx.x; e < 512; e += TSW_T) {
        float s = 0.0f;
#pragma unroll
        for (int w = 0; w < 8; ++w) s += red[w * 512 + e];
        out[e] = s;
    }
    __syncthreads();
}

// One product task: P_{u,v,s} = L_{slab, tile v} y_v (backward the transposed
// block), written to its partial block and counted in pcount[u].
template <bool TRANS, bool UPPER>
__device__ __forceinline__ void tsw_product_task(const TileSweepArgs &a, int u, int v, int s, float *Ms, float *Vs,
                                                 float *zs, int *skip)
{
    const int T = TRANS ? a.ntiles - 1 - u : u, j = TRANS ? a.ntiles - 1 - v : v;
    const int t0 = T * a.nb, kbT = min(a.nb, a.n - t0);
    const int r0 = t0 + s * TSW_SLAB, rows = min(TSW_SLAB, kbT - s * TSW_SLAB);
    const int j0 = j * a.nb, kbj = min(a.nb, a.n - j0);
    if (rows > 0) {
        constexpr bool direct = !TRANS || UPPER;  // operand read as rows of 32 per column
        if constexpr (direct) tsw_prefetch_l2<false>(a.L + r0 + (long)j0 * a.ldl, a.ldl, rows, kbj);
        else tsw_prefetch_l2<true>(a.L + j0 + (long)r0 * a.ldl, a.ldl, rows, kbj);
        tsw_wait(a, &a.ycount[v], a.spt, skip);
        float acc[4][4] = {};
        if constexpr (direct)
            tsw_product<false>(acc, a.L + r0 + (long)j0 * a.ldl, a.ldl, rows, a.B + j0, a.ldb, kbj, a.nrhs,
                               a.vec != 0, Ms, Vs);
        else
            tsw_product<true>(acc, a.L + j0 + (long)r0 * a.ldl, a.ldl, rows, a.B + j0, a.ldb, kbj, a.nrhs,
                              a.vec != 0, Ms, Vs);
        tsw_reduce(acc, Ms, zs);
        float *P = a.Zp + ((long)u * (u - 1) / 2 + v) * (long)a.nb * 16 + (long)s * TSW_SLAB * 16;
        for (int e = threadIdx.x; e < TSW_SLAB * 16; e += TSW_T) P[e] = zs[e];
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.pcount[u], 1);
}

// The diagonal task of slab s of tile row u: z = b - sum of the partials,
// published; then y = (slab rows of the inverse) z_T once z_T is complete.
template <bool TRANS>
__device__ __forceinline__ void tsw_diag_task(const TileSweepArgs &a, int u, int s, float *Ms, float *Vs, float *zs,
                                              int *skip)
{
    const int T = TRANS ? a.ntiles - 1 - u : u;
    const int t0 = T * a.nb, kbT = min(a.nb, a.n - t0);
    const int r0 = t0 + s * TSW_SLAB, rows = min(TSW_SLAB, kbT - s * TSW_SLAB);
    const float *D = a.Dinv + (long)T * a.dstride;
    if (rows > 0) {
        // the slab's rows (forward) or columns (backward) of the diagonal tile's inverse, needed last
        if (!TRANS) tsw_prefetch_l2<false>(D + s * TSW_SLAB, a.ldd, rows, s * TSW_SLAB + rows);
        else tsw_prefetch_l2<true>(D + s * TSW_SLAB + (long)(s * TSW_SLAB) * a.ldd, a.ldd, rows, kbT - s * TSW_SLAB);
        tsw_wait(a, &a.pcount[u], u * a.spt, skip);
        const float *P = a.Zp + (long)u * (u - 1) / 2 * (long)a.nb * 16 + (long)s * TSW_SLAB * 16;
        for (int e = threadIdx.x; e < TSW_SLAB * 16; e += TSW_T) {
            const int r = e >> 4, c = e & 15;
            if (r < rows && c < a.nrhs) {
                float sum = 0.0f;
                for (int v = 0; v < u; ++v) sum += __ldcg(P + (long)v * a.nb * 16 + e);
                a.Z[(long)(r0 + r) + (long)c * a.n] = __ldcg(&a.B[(long)(r0 + r) + (long)c * a.ldb]) - sum;
            }
        }
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.zcount[u], 1);
    if (rows <= 0) {
        if (threadIdx.x == 0) atomicAdd(&a.ycount[u], 1);
        return;
    }
    tsw_wait(a, &a.zcount[u], a.spt, skip);

    // diagonal tile: forward y_slab = Dinv(slab rows, 0 .. slab end) z_T;
    // backward x_slab = Dinv(slab start .. kbT, slab columns)^T z_T
    float acc2[4][4] = {};
    if (!TRANS) {
        tsw_product<false>(acc2, D + s * TSW_SLAB, a.ldd, rows, a.Z + t0, a.n, s * TSW_SLAB + rows, a.nrhs,
                           a.vec != 0, Ms, Vs);
    } else {
        const int k0 = s * TSW_SLAB;
        tsw_product<true>(acc2, D + k0 + (long)k0 * a.ldd, a.ldd, rows, a.Z + t0 + k0, a.n, kbT - k0, a.nrhs,
                          a.vec != 0, Ms, Vs);
    }
    tsw_reduce(acc2, Ms, zs);
    for (int e = threadIdx.x; e < TSW_SLAB * 16; e += TSW_T) {
        const int r = e >> 4, c = e & 15;
        if (r < rows && c < a.nrhs) a.B[(long)(r0 + r) + (long)c * a.ldb] = zs[e];
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.ycount[u], 1);
}

// UPPER (backward only): the strictly upper part of L's storage holds L^T
// outside the diagonal tiles (args.upper), read like the forward operand
template <bool TRANS, bool UPPER>
__global__ void __launch_bounds__(TSW_T, 2) tile_sweep_kernel(TileSweepArgs a)
{
    __shared__ __align__(16) float Ms[TSW_KC * TSW_MP];  // also the 8 x 512 reduction buffer
    __shared__ __align__(16) float Vs[TSW_KC * TSW_VP];
    __shared__ float zs[TSW_SLAB * 16];
    __shared__ unsigned s_ticket;
    __shared__ int s_skip;
    if (threadIdx.x == 0) s_skip = 0;
    for (;;) {
        __syncthreads();  // the previous task is done with s_ticket and the buffers
        if (threadIdx.x == 0) s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        const unsigned t = s_ticket;
        if (t >= a.total) return;
        // tile row u of the solve order: its tickets start at spt * u (u + 1) / 2
        const unsigned q = t / (unsigned)a.spt;
        int u = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
        while (u > 0 && (unsigned)u * (u + 1) / 2 > q) --u;
        while ((unsigned)(u + 1) * (u + 2) / 2 <= q) ++u;
        const unsigned r = t - (unsigned)a.spt * ((unsigned)u * (u + 1) / 2);
        if (r < (unsigned)(u * a.spt))
            tsw_product_task<TRANS, UPPER>(a, u, (int)(r / a.spt), (int)(r % a.spt), Ms, Vs, zs, &s_skip);
        else
            tsw_diag_task<TRANS>(a, u, (int)(r - u * a.spt), Ms, Vs, zs, &s_skip);
    }
}

} // namespace gb300
