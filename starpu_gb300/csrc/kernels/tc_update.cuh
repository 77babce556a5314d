// Tensor-core trailing update of the tiled Cholesky on sm_103a:
//
//     C[m x n] -= sum_t  A_t[m x K] * B_t[n x K]^T        (FP32 C, column-major)
//
// with A_t / B_t BF16 panels stored K-major (row i = K contiguous elements),
// staged by TMA (128-byte swizzle) and multiplied by tcgen05.mma (kind::f16,
// FP32 accumulation in TMEM).  This is the SYRK (lower, A == B, cublasSsyrk
// at examples/cholesky/cholesky_kernels.c:177) and GEMM (N,T, cublasSgemm at
// :98) update of every tile of one step k fused into one persistent launch.
//
// Terms: nterms = 1 -> A_hi B_hi^T (plain BF16); nterms = 3 -> the split-BF16
// product A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T, where x = x_hi + x_lo with
// x_hi = bf16(x), x_lo = bf16(x - x_hi), which carries ~16 significant bits of
// the FP32 panel into the product (the dropped A_lo B_lo^T term is ~2^-16
// relative).
//
// Scaled FP16 operands (f16s = 1, the factorisation's panels): row i of a
// panel is multiplied by 2^-k_i, the power of two that brings a bound of its
// elements just below 2^15 (FP16's largest binade), then split as
// x = h + l with h = fp16(x), l = fp16(x - h): 11 + 11 significant bits, and l
// stays a normal FP16 for every element above ~2^-18 of the bound.  The three
// products h_A h_B^T + h_A l_B^T + l_A h_B^T (each exact in FP32) accumulate
// the scaled product; the epilogue multiplies the row's 2^k_i by the column's
// 2^k_j (a power of two: exact) and applies it inside the FMA that updates C.
// The column scales are
// read 4 at a time when rs_b is 16-byte aligned (it is padded past its rows).  The
// dropped l_A l_B^T term weighs 2^-22 of the product.
//
// CTA = 6 warps, one CTA per SM (persistent, static round-robin over tiles):
//   warp 0  TMA producer     (one elected lane)
//   warp 1  MMA issuer       (one elected lane) + TMEM owner (512 columns)
//   warps 2-5 epilogue       (tcgen05.ld: warp w reads TMEM lanes 32*(w%4)..+31)
// Shared memory: STAGES x (A 128x64 + B 256x64 BF16) = STAGES x 48 KB.
// TMEM: two 128x256 FP32 accumulators so the epilogue of tile i overlaps the
// main loop of tile i+1.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sm100_ptx.cuh"

namespace gb300 {

constexpr int TCU_BM = 128;
constexpr int TCU_BN = 256;
constexpr int TCU_BK = 64;        // 64 BF16 = one 128-byte swizzle row
constexpr int TCU_STAGES = 4;
constexpr int TCU_THREADS = 192;
constexpr int TCU_A_BYTES = TCU_BM * TCU_BK * 2;   // 16 KB
constexpr int TCU_B_BYTES = TCU_BN * TCU_BK * 2;   // 32 KB
constexpr int TCU_SMEM = TCU_STAGES * (TCU_A_BYTES + TCU_B_BYTES) + 1024 /*align*/ + 256 /*barriers*/;
constexpr uint32_t TCU_TMEM_COLS = 512;

// error codes written to *err
constexpr int TCU_ERR_TIMEOUT_PRODUCER = 1;
constexpr int TCU_ERR_TIMEOUT_MMA = 2;
constexpr int TCU_ERR_TIMEOUT_EPILOGUE = 3;

struct TcUpdateArgs {
    float *C;
    long ldc;
    int m, n;          // C is m x n
    int K;             // elements per term (panel width)
    int nterms;        // 1 or 3
    int lower;         // 1: only elements with row >= col (square trailing matrix)
    int store;         // 1: C = sum (C is not read), 0: C -= sum
    int f16s;          // 1: scaled FP16 operands (rs_a, rs_b below); 0: BF16
    const float *rs_a, *rs_b;  // f16s: row scales (powers of two) of A (m) and B (n, padded)
    int rs_b_vec;              // rs_b is 16-byte aligned: the column scales load 4 at a time
    int tiles_m, tiles_n, num_tiles;
    int tile_begin, tile_end;  // the launch covers tiles [tile_begin, tile_end) of the num_tiles
    // 1: B is lower triangular in (row, k) (B(c, k) = 0 for k > c, the panel TRSM's
    // inverse), so a tile of columns n0 .. n0 + 255 stops at k = n0 + 255
    int b_lower;
    int *err;
    unsigned long long wait_budget_ns;
};

// K blocks a tile of columns n0 .. needs (all of them unless B is lower triangular)
__device__ __forceinline__ int tcu_tile_kblocks(const TcUpdateArgs &a, int kblocks, int n0)
{
    return a.b_lower ? min(kblocks, (n0 + TCU_BN + TCU_BK - 1) / TCU_BK) : kblocks;
}

// Map a linear tile index to (tm, tn).  Lower: column tn holds tiles
// tm = 2*tn .. tiles_m-1 (a 128-row tile crosses the diagonal of a 256-column
// tile only from tm = 2*tn on).
__device__ __forceinline__ void tcu_tile_coords(const TcUpdateArgs &a, int t, int &tm, int &tn)
{
    if (!a.lower) {
        tm = t % a.tiles_m;
        tn = t / a.tiles_m;
        return;
    }
    int col = 0, acc = 0;
    for (;;) {
        int cnt = a.tiles_m - 2 * col;
        if (t < acc + cnt) {
            tm = 2 * col + (t - acc);
            tn = col;
            return;
        }
        acc += cnt;
        ++col;
    }
}

__global__ void __launch_bounds__(TCU_THREADS, 1)
tc_update_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                 const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                 const TcUpdateArgs args)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte aligned tile area (required by the 128B swizzle atoms)
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + TCU_STAGES * TCU_A_BYTES;
    uint64_t *bars = (uint64_t *)(smem + TCU_STAGES * (TCU_A_BYTES + TCU_B_BYTES));
    uint64_t *full = bars;                    // [STAGES]
    uint64_t *empty = bars + TCU_STAGES;      // [STAGES]
    uint64_t *acc_full = bars + 2 * TCU_STAGES;       // [2]
    uint64_t *acc_empty = bars + 2 * TCU_STAGES + 2;  // [2]
    uint64_t *drain = bars + 2 * TCU_STAGES + 4;      // [1]
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * TCU_STAGES + 5);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TCU_STAGES; ++s) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            ptx::mbar_init(&acc_full[a], 1);
            ptx::mbar_init(&acc_empty[a], 128);
        }
        ptx::mbar_init(drain, 1);
        *abort_flag = 0;
        ptx::fence_mbarrier_init();
    }
    if (warp == 0 && lane == 0) {
        ptx::tma_prefetch_desc(&tm_a_hi);
        ptx::tma_prefetch_desc(&tm_b_hi);
        if (args.nterms > 1) {
            ptx::tma_prefetch_desc(&tm_a_lo);
            ptx::tma_prefetch_desc(&tm_b_lo);
        }
    }
    if (warp == 1) {
        ptx::tmem_alloc(tmem_slot, TCU_TMEM_COLS);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    const int kblocks = (args.K + TCU_BK - 1) / TCU_BK;

    if (warp == 0) {
        // ------------------------------------------------------ TMA producer
        if (ptx::elect_one()) {
            int stage = 0;
            uint32_t phase = 0;
            int issued = 0;
            bool ok = true;
            for (int t = args.tile_begin + blockIdx.x; t < args.tile_end && ok; t += gridDim.x) {
                int tm, tn;
                tcu_tile_coords(args, t, tm, tn);
                const int m0 = tm * TCU_BM, n0 = tn * TCU_BN;
                const int kbt = tcu_tile_kblocks(args, kblocks, n0), total_kb = kbt * args.nterms;
                for (int kb = 0; kb < total_kb; ++kb) {
                    if (!ptx::wait_parity(&empty[stage], phase ^ 1, abort_flag, args.wait_budget_ns)) {
                        ok = false;
                        break;
                    }
                    // the two cross products first, A_hi B_hi^T last: while the
                    // cross products accumulate, the accumulator holds only their
                    // sum (about 2^-8 of the result), so the rounding of each of
                    // their additions is 2^-8 smaller than on top of A_hi B_hi^T
                    const int term = args.nterms == 3 ? (kb / kbt + 1) % 3 : 0;
                    const int kx = (kb % kbt) * TCU_BK;
                    // term 0: A_hi B_hi^T, 1: A_hi B_lo^T, 2: A_lo B_hi^T
                    const CUtensorMap *ma = (term == 2) ? &tm_a_lo : &tm_a_hi;
                    const CUtensorMap *mb = (term == 1) ? &tm_b_lo : &tm_b_hi;
                    ptx::mbar_arrive_expect_tx(&full[stage], TCU_A_BYTES + TCU_B_BYTES);
                    ptx::tma_load_2d(sA + stage * TCU_A_BYTES, ma, &full[stage], kx, m0);
                    ptx::tma_load_2d(sB + stage * TCU_B_BYTES, mb, &full[stage], kx, n0);
                    ++issued;
                    if (++stage == TCU_STAGES) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
            }
            if (!ok) {
                if (!*abort_flag) atomicCAS(args.err, 0, TCU_ERR_TIMEOUT_PRODUCER);
                *abort_flag = 1;
            }
            // drain: make sure every TMA write into shared memory has landed
            // before the CTA can exit (bounded; ignores the abort flag)
            int s = stage;
            uint32_t ph = phase;
            int back = issued < TCU_STAGES ? issued : TCU_STAGES;
            for (int i = 0; i < back; ++i) {
                if (--s < 0) {
                    s = TCU_STAGES - 1;
                    ph ^= 1;
                }
                volatile int never = 0;
                ptx::wait_parity(&full[s], ph, &never, args.wait_budget_ns);
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------- MMA issuer
        if (ptx::elect_one()) {
            const uint32_t idesc = args.f16s ? ptx::make_idesc(TCU_BM, TCU_BN, ptx::FMT_F16)
                                             : ptx::make_idesc(TCU_BM, TCU_BN, ptx::FMT_BF16);
            int stage = 0;
            uint32_t phase = 0;
            int acc = 0;
            uint32_t acc_phase = 0;
            bool ok = true;
            for (int t = args.tile_begin + blockIdx.x; t < args.tile_end && ok; t += gridDim.x) {
                if (!ptx::wait_parity(&acc_empty[acc], acc_phase ^ 1, abort_flag, args.wait_budget_ns)) {
                    ok = false;
                    break;
                }
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem_base + (uint32_t)(acc * TCU_BN);
                int tm, tn;
                tcu_tile_coords(args, t, tm, tn);
                const int total_kb = tcu_tile_kblocks(args, kblocks, tn * TCU_BN) * args.nterms;
                for (int kb = 0; kb < total_kb; ++kb) {
                    if (!ptx::wait_parity(&full[stage], phase, abort_flag, args.wait_budget_ns)) {
                        ok = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t a_addr = ptx::smem_u32(sA + stage * TCU_A_BYTES);
                    const uint32_t b_addr = ptx::smem_u32(sB + stage * TCU_B_BYTES);
#pragma unroll
                    for (int k = 0; k < TCU_BK / 16; ++k) {
                        // advance 16 BF16 = 32 bytes inside the 128-byte swizzled row
                        const uint64_t ad = ptx::make_sdesc_k128(a_addr + k * 32);
                        const uint64_t bd = ptx::make_sdesc_k128(b_addr + k * 32);
                        ptx::mma_f16_ss(d_tmem, ad, bd, idesc, (kb > 0 || k > 0) ? 1u : 0u);
                    }
                    ptx::mma_commit(&empty[stage]);  // frees the smem stage when these MMAs finish
                    if (++stage == TCU_STAGES) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (!ok) break;
                ptx::mma_commit(&acc_full[acc]);  // accumulator ready for the epilogue
                if (++acc == 2) {
                    acc = 0;
                    acc_phase ^= 1;
                }
            }
            if (!ok) {
                if (!*abort_flag) atomicCAS(args.err, 0, TCU_ERR_TIMEOUT_MMA);
                *abort_flag = 1;
            }
            // wait until every MMA issued by this thread has completed
            ptx::mma_commit(drain);
            volatile int never = 0;
            ptx::wait_parity(drain, 0, &never, args.wait_budget_ns);
        }
    } else {
        // --------------------------------------------------------- epilogue
        const int quarter = warp & 3;  // TMEM lane quarter this warp may access
        const int row_in_tile = quarter * 32 + lane;
        int acc = 0;
        uint32_t acc_phase = 0;
        bool ok = true;
        for (int t = args.tile_begin + blockIdx.x; t < args.tile_end; t += gridDim.x) {
            int tm, tn;
            tcu_tile_coords(args, t, tm, tn);
            const int row = tm * TCU_BM + row_in_tile;
            const int n0 = tn * TCU_BN;
            if (!ptx::wait_parity(&acc_full[acc], acc_phase, abort_flag, args.wait_budget_ns)) {
                ok = false;
                break;
            }
            ptx::tc_fence_after();
            const uint32_t tbase = tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * TCU_BN);
            float *crow = args.C + row;
            const bool row_ok = row < args.m;
            // scaled FP16: the row's scale (the columns' below)
            const float rsc = (args.f16s && row_ok) ? args.rs_a[row] : 1.0f;
#pragma unroll 1
            for (int ch = 0; ch < TCU_BN / 32; ++ch) {
                uint32_t r[32];
                ptx::tmem_ld_32x32b_x32(tbase + ch * 32, r);
                ptx::tmem_ld_wait();
                if (ch == TCU_BN / 32 - 1) {
                    ptx::tc_fence_before();
                    ptx::mbar_arrive(&acc_empty[acc]);
                }
                const int c0 = n0 + ch * 32;
                if (row_ok) {
                    float cv[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int col = c0 + j;
                        const bool w = col < args.n && (!args.lower || row >= col);
                        cv[j] = (w && !args.store) ? crow[(long)col * args.ldc] : 0.0f;
                    }
                    float cs[32];
                    if (args.f16s && !args.rs_b_vec) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) cs[j] = args.rs_b[c0 + j];
                    } else if (args.f16s) {
                        const float4 *c4 = reinterpret_cast<const float4 *>(args.rs_b + c0);
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const float4 v = c4[q];
                            cs[4 * q] = v.x;
                            cs[4 * q + 1] = v.y;
                            cs[4 * q + 2] = v.z;
                            cs[4 * q + 3] = v.w;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j) cs[j] = 1.0f;
                    }
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int col = c0 + j;
                        const bool w = col < args.n && (!args.lower || row >= col);
                        // 2^(k_i + k_j) as one exact factor: it cannot overflow where C does
                        // not (a panel scale of 2^105 times an inverse's 2^-75 is fine, while
                        // the accumulator times 2^105 alone is not).  Below FP32's normal
                        // range (both scales tiny, matrices ~1e-30) the two are applied one
                        // after the other instead, the accumulator keeping the product normal.
                        const float sc = rsc * cs[j];
                        const bool tiny = sc < 1.17549435e-38f;
                        const float a = __uint_as_float(r[j]);
                        const float f1 = tiny ? a * rsc : a, f2 = tiny ? cs[j] : sc;
                        if (w) crow[(long)col * args.ldc] = args.store ? f1 * f2 : fmaf(-f1, f2, cv[j]);
                    }
                }
            }
            if (++acc == 2) {
                acc = 0;
                acc_phase ^= 1;
            }
        }
        if (!ok) {
            if (!*abort_flag) atomicCAS(args.err, 0, TCU_ERR_TIMEOUT_EPILOGUE);
            *abort_flag = 1;
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) ptx::tmem_dealloc(tmem_base, TCU_TMEM_COLS);
}

} // namespace gb300
