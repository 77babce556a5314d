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
// The products M (32 x K) V (K x 16) read their operand M as 32-row columns
// (L, the mirrored L^T in the upper part, the diagonal-tile inverses and their
// transposes) and V from row-major copies of y / z (16 floats per row) that
// the diagonal tasks keep beside the column-major result.  Both are staged by
// cp.async in a 6-deep ring of 64-column stages (~80 KB in flight per CTA),
// and multiplied on the tensor cores with warp-level m16n8k8 TF32 MMAs, three
// per tile on the split x = hi + lo of both operands (about 21 significant
// bits, the FP32 solve's own accuracy); each warp takes 8 of a stage's 64
// columns and the 8 warps' 32 x 16 blocks are summed in a fixed order.  (A
// 32-row slab and 16 right-hand sides are below the smallest tcgen05 tile, and
// the chain of the sweep wants the accumulator in registers: the warp-level
// MMA is the instruction that fits.)  Operands that are only available
// transposed (the public entry point's L^T and inverses) take a
// register-staged FP32 FMA path with the same partial layout.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb300 {

constexpr int TSW_SLAB = 32;   // rows per CTA
constexpr int TSW_KC = 128;    // K chunk
constexpr int TSW_MP = 36;     // pitch of one K index of the operand chunk (32 rows + 4)
constexpr int TSW_VP = 20;     // pitch of one K index of the right-hand-side chunk (16 + 4)
constexpr int TSW_T = 256;
constexpr int TSW_KS = 64;   // K per cp.async stage
constexpr int TSW_NS = 6;    // stages in the ring
// pitches of the ring's operand and right-hand-side rows, chosen so that the
// tensor-core fragment loads (8 rows x 4 columns per warp) hit 32 banks
constexpr int TSW_DMP = 40, TSW_DVP = 24;
constexpr int TSW_STAGE = TSW_KS * (TSW_DMP + TSW_DVP);  // floats per stage
// dynamic shared memory of the kernel: the ring (the register-staged path and
// the reductions reuse it)
constexpr int TSW_DSMEM = TSW_NS * TSW_STAGE * 4;
static_assert(TSW_NS * TSW_STAGE >= TSW_KC * (TSW_MP + TSW_VP), "register-staged buffers fit the ring");
static_assert(TSW_NS * TSW_STAGE >= 8 * 512, "reduction buffer fits the ring");

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
    float *Zt;  // z of the tile rows, row-major n x 16
    float *Yt;  // solved rows (y forward, x backward), row-major n x 16: the products' right-hand operand
    float *Zp;  // partial products: pair (u, v < u) at Zp + (u (u - 1) / 2 + v) * nb * 16, slab-major 32 x 16
    const float *DinvT;  // optional: tile T's inverse transposed at DinvT + T * dstride (ld ldd)
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

// Bytes of scratch a sweep pair needs: Zt and Yt (n x 16 each), the partial
// products of every pair of tile rows, and the 3 ntiles + 1 counters.
inline size_t tsw_scratch_bytes(int n, int nb, size_t *yt_off = nullptr, size_t *zp_off = nullptr,
                                size_t *cnt_off = nullptr)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t nt = ((size_t)n + nb - 1) / nb;
    const size_t z = al((size_t)n * 16 * sizeof(float));
    const size_t zp = al(nt * (nt > 0 ? nt - 1 : 0) / 2 * (size_t)nb * 16 * sizeof(float));
    if (yt_off) *yt_off = z;
    if (zp_off) *zp_off = 2 * z;
    if (cnt_off) *cnt_off = 2 * z + zp;
    return 2 * z + zp + al((3 * nt + 1) * sizeof(int));
}

__device__ __forceinline__ void tsw_cp16(float *smem, const float *gmem, int src_bytes)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void tsw_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void tsw_cp_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
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
//   V(p, c) = V[16 p + c]                 (row-major, 16-byte aligned rows)
struct TswStage {
    float4 m[4];
    float4 v[2];
};

// Element maps (1024 float4 of M, 512 of V per chunk), chosen so that the
// transposing shared stores of tsw_put hit 32 distinct banks:
//   M, TR = false: float4 = 4 consecutive rows r of column p (coalesced rows);
//   M, TR = true : lane = row r, a thread's 4 float4 = 16 consecutive p (two
//                  whole 32-byte sectors of column r);
//   V: float4 = right-hand sides 4 q .. 4 q + 3 of row p (V is small and
//      stays in L2).
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
__device__ __forceinline__ void tsw_map_v(int u, int &p, int &q)
{
    const int e = threadIdx.x + TSW_T * u;
    p = e >> 2;
    q = e & 3;
}

template <bool TR>
__device__ __forceinline__ void tsw_fetch(TswStage &st, const float *M, long ldm, int rows, const float *V, int kc,
                                          bool vec)
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
        int p, q;
        tsw_map_v(u, p, q);
        st.v[u] = p < kc ? __ldcg(reinterpret_cast<const float4 *>(V + (long)p * 16 + 4 * q))
                         : make_float4(0.f, 0.f, 0.f, 0.f);
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
        int p, q;
        tsw_map_v(u, p, q);
        *reinterpret_cast<float4 *>(Vs + p * TSW_VP + 4 * q) = st.v[u];
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
__device__ __forceinline__ void tsw_product(float acc[4][4], const float *M, long ldm, int rows, const float *V, int K,
                                            bool vec, float *Ms, float *Vs)
{
    if (K <= 0) return;
    auto fetch = [&](TswStage &st, int c) {
        const int p0 = c * TSW_KC;
        const float *Mc = TR ? M + p0 : M + (long)p0 * ldm;
        tsw_fetch<TR>(st, Mc, ldm, rows, V + (long)p0 * 16, min(TSW_KC, K - p0), vec);
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

// TF32 split of x: hi = tf32(x) (round to nearest), lo = tf32(x - hi).
__device__ __forceinline__ void tsw_split_tf32(float x, uint32_t &hi, uint32_t &lo)
{
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
    const float r = x - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}

// d += a b for one 16 x 8 x 8 TF32 tile (warp-wide, FP32 accumulation)
__device__ __forceinline__ void tsw_mma_tf32(float d[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// acc += M(32 x K) V(K x 16) for an operand read as 32-row columns
// (M(r, p) = M[r + p * ldm], 16-byte aligned columns) and a row-major V, in a
// TSW_NS-deep cp.async ring of TSW_KS-column stages; elements past `rows` and
// K are zero-filled.  The products run on the tensor cores as three TF32
// products per tile, hi hi + hi lo + lo hi with x = hi + lo split in
// registers (about 21 significant bits: the FP32 correction solve's own
// accuracy), accumulated in FP32.  Warp w takes columns 8 w .. 8 w + 7 of
// every stage and keeps the whole 32 x 16 block: acc[mt][nt][4] holds the
// m16n8 accumulator fragment of rows 16 mt .., right-hand sides 8 nt ...
__device__ __forceinline__ void tsw_product_direct(float acc[2][2][4], const float *M, long ldm, int rows,
                                                   const float *V, int K, float *ring)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int nst = (K + TSW_KS - 1) / TSW_KS;
    auto issue = [&](int st) {
        float *Ms = ring + (st % TSW_NS) * TSW_STAGE, *Vs = Ms + TSW_KS * TSW_DMP;
        const int p0 = st * TSW_KS, kc = min(TSW_KS, K - p0);
#pragma unroll
        for (int u = 0; u < TSW_KS * 8 / TSW_T; ++u) {
            const int e = tid + TSW_T * u, p = e >> 3, q = e & 7;
            const int valid = p < kc ? max(0, min(4, rows - 4 * q)) : 0;
            tsw_cp16(Ms + p * TSW_DMP + 4 * q, valid ? M + 4 * q + (long)(p0 + p) * ldm : M, 4 * valid);
        }
        if (tid < TSW_KS * 4) {
            const int p = tid >> 2, q = tid & 3;
            tsw_cp16(Vs + p * TSW_DVP + 4 * q, p < kc ? V + (long)(p0 + p) * 16 + 4 * q : V, p < kc ? 16 : 0);
        }
    };
#pragma unroll 1
    for (int st = 0; st < TSW_NS - 1; ++st) {
        if (st < nst) issue(st);
        tsw_cp_commit();
    }
#pragma unroll 1
    for (int st = 0; st < nst; ++st) {
        tsw_cp_wait<TSW_NS - 2>();
        __syncthreads();  // stage st is in; every warp is done with the buffer reloaded next
        if (st + TSW_NS - 1 < nst) issue(st + TSW_NS - 1);
        tsw_cp_commit();
        const float *Ms = ring + (st % TSW_NS) * TSW_STAGE + 8 * warp * TSW_DMP;
        const float *Vs = ring + (st % TSW_NS) * TSW_STAGE + TSW_KS * TSW_DMP + 8 * warp * TSW_DVP;
        // B fragments (k = t, t + 4; right-hand side g of each 8-column half)
        uint32_t bh[2][2], bl[2][2];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            tsw_split_tf32(Vs[t * TSW_DVP + 8 * nt + g], bh[nt][0], bl[nt][0]);
            tsw_split_tf32(Vs[(t + 4) * TSW_DVP + 8 * nt + g], bh[nt][1], bl[nt][1]);
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            // A fragment: rows g, g + 8 of the m-tile, k = t, t + 4
            uint32_t ah[4], al[4];
            tsw_split_tf32(Ms[t * TSW_DMP + 16 * mt + g], ah[0], al[0]);
            tsw_split_tf32(Ms[t * TSW_DMP + 16 * mt + g + 8], ah[1], al[1]);
            tsw_split_tf32(Ms[(t + 4) * TSW_DMP + 16 * mt + g], ah[2], al[2]);
            tsw_split_tf32(Ms[(t + 4) * TSW_DMP + 16 * mt + g + 8], ah[3], al[3]);
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                tsw_mma_tf32(acc[mt][nt], al, bh[nt]);  // the small terms first
                tsw_mma_tf32(acc[mt][nt], ah, bl[nt]);
                tsw_mma_tf32(acc[mt][nt], ah, bh[nt]);
            }
        }
    }
    tsw_cp_wait<0>();
    __syncthreads();  // the ring is free for the reduction
}

// Sum tsw_product_direct's per-warp blocks (the 8 warps in order) into out
// (32 x 16, row-major).  Fragment element (mt, nt, i) of lane (g, t) is
// row 16 mt + g + 8 (i / 2), right-hand side 8 nt + 2 t + i % 2.
__device__ __forceinline__ void tsw_reduce_frag(const float acc[2][2][4], float *red, float *out)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                *reinterpret_cast<float2 *>(red + warp * 512 + (16 * mt + g + 8 * h) * 16 + 8 * nt + 2 * t) =
                    make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]);
    __syncthreads();
    for (int e = threadIdx.x; e < 512; e += TSW_T) {
        float s = 0.0f;
#pragma unroll
        for (int w = 0; w < 8; ++w) s += red[w * 512 + e];
        out[e] = s;
    }
    __syncthreads();
}

// out (32 x 16) = M(32 x K) V(K x 16).  Each form is its own function so that
// its registers are allocated alone (the cp.async path holds 64 accumulators).
__device__ __noinline__ void tsw_gemv_direct(const float *M, long ldm, int rows, const float *V, int K, float *ring,
                                             float *out)
{
    float acc[2][2][4] = {};
    if (K > 0) tsw_product_direct(acc, M, ldm, rows, V, K, ring);
    tsw_reduce_frag(acc, ring, out);
}

template <bool TR>
__device__ __noinline__ void tsw_gemv_staged(const float *M, long ldm, int rows, const float *V, int K, bool vec,
                                             float *ring, float *out)
{
    float acc[4][4] = {};
    tsw_product<TR>(acc, M, ldm, rows, V, K, vec, ring, ring + TSW_KC * TSW_MP);
    tsw_reduce(acc, ring, out);
}

// the cp.async path for a direct operand with aligned columns, else the
// register-staged one (TR: M transposed)
template <bool TR>
__device__ __forceinline__ void tsw_gemv(const float *M, long ldm, int rows, const float *V, int K, bool vec,
                                         float *ring, float *out)
{
    if (!TR && vec) tsw_gemv_direct(M, ldm, rows, V, K, ring, out);
    else tsw_gemv_staged<TR>(M, ldm, rows, V, K, vec, ring, out);
}

// One product task: P_{u,v,s} = L_{slab, tile v} y_v (backward the transposed
// block), written to its partial block and counted in pcount[u].
template <bool TRANS, bool UPPER>
__device__ __forceinline__ void tsw_product_task(const TileSweepArgs &a, int u, int v, int s, float *ring,
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
        if constexpr (direct)
            tsw_gemv<false>(a.L + r0 + (long)j0 * a.ldl, a.ldl, rows, a.Yt + (long)j0 * 16, kbj, a.vec != 0, ring,
                            zs);
        else
            tsw_gemv<true>(a.L + j0 + (long)r0 * a.ldl, a.ldl, rows, a.Yt + (long)j0 * 16, kbj, a.vec != 0, ring,
                           zs);
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
__device__ __forceinline__ void tsw_diag_task(const TileSweepArgs &a, int u, int s, float *ring, float *zs,
                                              int *skip)
{
    const int T = TRANS ? a.ntiles - 1 - u : u;
    const int t0 = T * a.nb, kbT = min(a.nb, a.n - t0);
    const int r0 = t0 + s * TSW_SLAB, rows = min(TSW_SLAB, kbT - s * TSW_SLAB);
    const float *D = a.Dinv + (long)T * a.dstride;
    if (rows > 0) {
        // the slab's rows (forward) or columns (backward) of the diagonal tile's inverse, needed last
        const int k0 = s * TSW_SLAB;
        if (!TRANS) tsw_prefetch_l2<false>(D + k0, a.ldd, rows, k0 + rows);
        else if (a.DinvT) tsw_prefetch_l2<false>(a.DinvT + (long)T * a.dstride + k0 + (long)k0 * a.ldd, a.ldd, rows, kbT - k0);
        else tsw_prefetch_l2<true>(D + k0 + (long)k0 * a.ldd, a.ldd, rows, kbT - k0);
        tsw_wait(a, &a.pcount[u], u * a.spt, skip);
        const float *P = a.Zp + (long)u * (u - 1) / 2 * (long)a.nb * 16 + (long)s * TSW_SLAB * 16;
        for (int e = threadIdx.x; e < TSW_SLAB * 16; e += TSW_T) {
            const int r = e >> 4, c = e & 15;
            if (r < rows && c < a.nrhs) {
                float sum = 0.0f;
                for (int v = 0; v < u; ++v) sum += __ldcg(P + (long)v * a.nb * 16 + e);
                a.Zt[(long)(r0 + r) * 16 + c] = __ldcg(&a.B[(long)(r0 + r) + (long)c * a.ldb]) - sum;
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
    // backward x_slab = Dinv(slab start .. kbT, slab columns)^T z_T (read
    // from the transposed tiles when they are kept)
    const int k0 = s * TSW_SLAB;
    if (!TRANS)
        tsw_gemv<false>(D + k0, a.ldd, rows, a.Zt + (long)t0 * 16, k0 + rows, a.vec != 0, ring, zs);
    else if (a.DinvT)
        tsw_gemv<false>(a.DinvT + (long)T * a.dstride + k0 + (long)k0 * a.ldd, a.ldd, rows,
                        a.Zt + (long)(t0 + k0) * 16, kbT - k0, a.vec != 0, ring, zs);
    else
        tsw_gemv<true>(D + k0 + (long)k0 * a.ldd, a.ldd, rows, a.Zt + (long)(t0 + k0) * 16, kbT - k0, a.vec != 0,
                       ring, zs);
    for (int e = threadIdx.x; e < TSW_SLAB * 16; e += TSW_T) {
        const int r = e >> 4, c = e & 15;
        if (r < rows && c < a.nrhs) {
            a.B[(long)(r0 + r) + (long)c * a.ldb] = zs[e];
            a.Yt[(long)(r0 + r) * 16 + c] = zs[e];
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.ycount[u], 1);
}

// UPPER (backward only): the strictly upper part of L's storage holds L^T
// outside the diagonal tiles (args.upper), read like the forward operand
// Task of ticket t: tile row u of the solve order (its tickets start at
// spt u (u + 1) / 2: u spt products, then spt diagonal tasks) and the rank r
// within the row (r < u spt: product with earlier tile row r / spt, slab
// r % spt; else diagonal task of slab r - u spt).
__host__ __device__ __forceinline__ void tsw_decode(unsigned t, int spt, int &u, unsigned &r)
{
    const unsigned q = t / (unsigned)spt;
    u = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
    while (u > 0 && (unsigned)u * (u + 1) / 2 > q) --u;
    while ((unsigned)(u + 1) * (u + 2) / 2 <= q) ++u;
    r = t - (unsigned)spt * ((unsigned)u * (u + 1) / 2);
}

template <bool TRANS, bool UPPER>
__global__ void __launch_bounds__(TSW_T, 2) tile_sweep_kernel(TileSweepArgs a)
{
    extern __shared__ float4 tsw_dsmem[];
    float *ring = reinterpret_cast<float *>(tsw_dsmem);  // TSW_DSMEM bytes
    __shared__ __align__(16) float zs[TSW_SLAB * 16];
    __shared__ unsigned s_ticket;
    __shared__ int s_skip;
    if (threadIdx.x == 0) s_skip = 0;
    for (;;) {
        __syncthreads();  // the previous task is done with s_ticket and the buffers
        if (threadIdx.x == 0) s_ticket = atomicAdd(a.ticket, 1u);
        __syncthreads();
        const unsigned t = s_ticket;
        if (t >= a.total) return;
        int u;
        unsigned r;
        tsw_decode(t, a.spt, u, r);
        if (r < (unsigned)(u * a.spt))
            tsw_product_task<TRANS, UPPER>(a, u, (int)(r / a.spt), (int)(r % a.spt), ring, zs, &s_skip);
        else
            tsw_diag_task<TRANS>(a, u, (int)(r - u * a.spt), ring, zs, &s_skip);
    }
}

} // namespace gb300
