// Host side of the tensor-core trailing update: TMA descriptor encoding, the
// FP32 -> split (K-major; BF16, or FP16 with row scales) panel converters, and the C-ABI entry points
// that use them (the bare update, and the tiled factorisation whose trailing
// updates run on the tensor cores).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <atomic>
#include <functional>
#include <mutex>
#include <stdio.h>

#include "gb300_internal.h"
#include "kernels/diag_coop.cuh"
#include "kernels/residual_tc.cuh"
#include "kernels/tc_update.cuh"
#include "starpu_gb300_kernels.h"
#include "starpu_gb300_solver.h"

namespace gb300 {

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        else
            cudaGetLastError();
    });
    return g_encode;
}

// K-major BF16 matrix [rows x K] with row stride ld (elements, ld*2 % 16 == 0),
// box = 64 (K) x box_rows, 128-byte swizzle, zero fill out of bounds.
static int make_kmajor_map(CUtensorMap *map, const void *base, int rows, int K, long ld, int box_rows)
{
    auto enc = encode_fn();
    if (!enc) return GB300_ENOTSUP;
    if (((uintptr_t)base & 15) || ((ld * 2) & 15)) return GB300_EINVAL;
    cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)TCU_BK, (cuuint32_t)box_rows};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), gdim, gstride, box, estride,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? GB300_OK : GB300_EINVAL;
}

static int num_sms() { return gb300_device_sms(); }

// P (m x k FP32, column-major, ldp) -> hi = bf16(P), lo = bf16(P - hi), both
// K-major (row i holds P[i, 0..k)), row stride ldk; columns k..ldk-1 zeroed.
// 32x32 tiles transposed through shared memory: coalesced on both sides.
__global__ void split_bf16_kmajor_kernel(int m, int k, const float *__restrict__ P, long ldp,
                                         __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo, long ldk)
{
    __shared__ float t[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        const int r = r0 + threadIdx.x, col = c0 + c;
        t[c][threadIdx.x] = (r < m && col < k) ? P[r + (long)col * ldp] : 0.0f;
    }
    __syncthreads();
    for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
        const int r = r0 + rr, col = c0 + threadIdx.x;
        if (r < m && col < ldk) {
            const float v = t[threadIdx.x][rr];
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            hi[(long)r * ldk + col] = h;
            if (lo) lo[(long)r * ldk + col] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
}

int split_bf16(cudaStream_t s, int m, int k, const float *P, long ldp, void *hi, void *lo, long ldk)
{
    if (m <= 0 || k <= 0) return GB300_OK;
    dim3 g((m + 31) / 32, (unsigned)((ldk + 31) / 32));
    gb300_count_launch(), split_bf16_kmajor_kernel<<<g, dim3(32, 8), 0, s>>>(m, k, P, ldp, (__nv_bfloat16 *)hi, (__nv_bfloat16 *)lo, ldk);
    return gb300_last_launch_status();
}

// ---- scaled FP16 panels (the factorisation's operands) ---------------------
//
// Row i of P (m x k FP32, column-major) is multiplied by 2^-k_i (rk[i] = k_i),
// the power of two that brings a bound b_i of its elements below 2^15, and split as
// x = h + l, h = fp16(x), l = fp16(x - h), both K-major (row i = k contiguous
// halves, row stride ldk, columns k..ldk-1 zero).  About 22 significant bits
// of every element above ~2^-18 b_i reach the tensor cores (16 with the BF16
// split); elements up to about 4 b_i stay below FP16's largest value.
//
// The bounds need no pass over the panel: for the SPD matrix being factored,
// the Schur complement S after any number of steps keeps |S_rj| <=
// sqrt(S_rr S_jj) <= sqrt(A_rr A_jj), and a row of L keeps |L_rj| <= sqrt(A_rr)
// (sum_j L_rj^2 = A_rr).  So with d = diag(A) saved before the factorisation:
// b_r = sqrt(d_r f), f = max of d over the panel's columns for the panel
// before its triangular solve, f = 1 for the solved panel.  A matrix that is
// not SPD may break the bound; its factorisation then fails on a pivot.
struct F16Panel {
    __half *h, *l;
    int *rk;    // row exponents k_i (the split divides by 2^k_i)
    float *rs;  // 2^k_i as floats, for the epilogue; both arrays hold 64 entries past the rows
};

// bytes of one row-scale array (rows + 64 entries of padding: the epilogue
// loads the scales of 32 columns at a time past the last row)
static size_t scale_bytes(size_t rows) { return ((rows + 64) * 4 + 255) & ~(size_t)255; }

__device__ __forceinline__ float pow2f(int k) { return ldexpf(1.0f, k < -149 ? -149 : k); }

// k with bound 2^-k < 2^15
__device__ __forceinline__ int f16_row_exp(float bound)
{
    int e = 0;
    if (bound > 0.0f && isfinite(bound)) frexpf(bound, &e);  // bound = f 2^e, 0.5 <= f < 1
    return e - 15;
}

// rk[i] from the actual row maxima (the inverse of a diagonal tile, whose
// elements have no bound from the matrix): 32 rows per CTA, the k loop split
// over 8 thread rows.
__global__ void panel_row_scale_kernel(int m, int k, const float *__restrict__ P, long ldp, int *__restrict__ rk,
                                       float *__restrict__ rs)
{
    __shared__ float red[8][33];
    const int r = blockIdx.x * 32 + threadIdx.x;
    float mx = 0.0f;
    if (r < m)
        for (int c = threadIdx.y; c < k; c += 8) mx = fmaxf(mx, fabsf(P[r + (long)c * ldp]));
    red[threadIdx.y][threadIdx.x] = mx;
    __syncthreads();
    if (threadIdx.y == 0 && r < m) {
        for (int y = 1; y < 8; ++y) mx = fmaxf(mx, red[y][threadIdx.x]);
        rk[r] = f16_row_exp(mx);
        rs[r] = pow2f(rk[r]);
    }
}

// d[r] = A_rr (from A's diagonal, or from dsrc when given), and dtile[t] =
// max of d over the nb rows of column tile t
__global__ void diag_bounds_kernel(int n, const float *__restrict__ A, long lda, int nb, float *__restrict__ d,
                                   float *__restrict__ dtile, const float *__restrict__ dsrc)
{
    __shared__ float red[256];
    const int t = blockIdx.x;
    float mx = 0.0f;
    for (int r = t * nb + threadIdx.x; r < min(n, (t + 1) * nb); r += blockDim.x) {
        const float v = dsrc ? dsrc[r] : A[r + (long)r * lda];
        d[r] = v;
        mx = fmaxf(mx, fabsf(v));
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) dtile[t] = red[0];
}

// the split; rk given (from_bounds = 0) or computed from d / f (from_bounds = 1:
// rows r0.. of the matrix, d indexed by matrix row, *f or 1 when f is NULL)
__global__ void split_f16s_kmajor_kernel(int m, int k, const float *__restrict__ P, long ldp, int *__restrict__ rk,
                                         float *__restrict__ rs,
                                         int from_bounds, const float *__restrict__ d, int r0,
                                         const float *__restrict__ f, __half *__restrict__ h, __half *__restrict__ l,
                                         long ldk)
{
    __shared__ float t[32][33];
    __shared__ int sh[32];
    const int rb = blockIdx.x * 32, c0 = blockIdx.y * 32;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (tid < 32 && rb + tid < m) {
        int e;
        if (from_bounds) {
            // sqrt(d_r) sqrt(f): no underflow or overflow of the product for
            // matrices scaled far from 1
            e = f16_row_exp(sqrtf(fmaxf(d[r0 + rb + tid], 0.0f)) * (f ? sqrtf(*f) : 1.0f));
            if (blockIdx.y == 0) {
                rk[rb + tid] = e;
                rs[rb + tid] = pow2f(e);
            }
        } else {
            e = rk[rb + tid];
        }
        sh[tid] = -e;
    }
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        const int r = rb + threadIdx.x, col = c0 + c;
        t[c][threadIdx.x] = (r < m && col < k) ? P[r + (long)col * ldp] : 0.0f;
    }
    __syncthreads();
    for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
        const int r = rb + rr, col = c0 + threadIdx.x;
        if (r < m && col < ldk) {
            const int sx = sh[rr];  // exact: a power-of-two scaling (ldexp only outside the normal range)
            const float x = (sx >= -126 && sx <= 127) ? t[threadIdx.x][rr] * __int_as_float((sx + 127) << 23)
                                                      : ldexpf(t[threadIdx.x][rr], sx);
            const __half hh = __float2half_rn(x);
            const long o = (long)r * ldk + col;
            h[o] = hh;
            l[o] = __float2half_rn(x - __half2float(hh));
        }
    }
}

// from the actual row maxima (d == NULL) or from the diagonal bounds
static int split_f16s(cudaStream_t s, int m, int k, const float *P, long ldp, const F16Panel &o, long ldk,
                      const float *d = nullptr, int r0 = 0, const float *f = nullptr)
{
    if (m <= 0 || k <= 0) return GB300_OK;
    if (!d)
        gb300_count_launch(), panel_row_scale_kernel<<<(m + 31) / 32, dim3(32, 8), 0, s>>>(m, k, P, ldp, o.rk, o.rs);
    dim3 g((m + 31) / 32, (unsigned)((ldk + 31) / 32));
    gb300_count_launch(), split_f16s_kmajor_kernel<<<g, dim3(32, 8), 0, s>>>(m, k, P, ldp, o.rk, o.rs, d ? 1 : 0, d, r0, f,
                                                                           o.h, o.l, ldk);
    return gb300_last_launch_status();
}

// rows [r, ...) of a split panel
static F16Panel rows_of(const F16Panel &p, long r, long ldk)
{
    return {p.h + r * ldk, p.l + r * ldk, p.rk + r, p.rs + r};
}

// One operand of the update: BF16 hi / lo, or the scaled FP16 split
// (hi = h, lo = l, rk = the row scale exponents).
struct TcOperand {
    const void *hi, *lo;
    const float *rs;
};

// max_grid > 0 caps the persistent grid (CTAs, one per SM): the trailing
// update that runs beside the next panel leaves that panel's SMs free.
// f16s: both operands are scaled FP16 panels.  [t0, t1) (t1 < 0: to the end)
// restricts the launch to a range of the update's tiles, in the order
// tcu_tile_coords gives them (lower: column by column from the diagonal).
static int tc_update_op(cudaStream_t s, int m, int n, int K, const TcOperand &A, long lda, const TcOperand &B,
                        long ldb, int nterms, int lower, float *C, long ldc, int *d_err, int store, int max_grid,
                        bool f16s, int t0 = 0, int t1 = -1, bool b_lower = false)
{
    if (m <= 0 || n <= 0 || K <= 0) return GB300_OK;
    if ((nterms != 1 && nterms != 3) || (nterms == 3 && (!A.lo || !B.lo)) || (lower && m != n) || !d_err ||
        (f16s && (!A.rs || !B.rs)))
        return GB300_EINVAL;
    CUtensorMap ta_hi, ta_lo, tb_hi, tb_lo;
    int rc;
    if ((rc = make_kmajor_map(&ta_hi, A.hi, m, K, lda, TCU_BM))) return rc;
    if ((rc = make_kmajor_map(&tb_hi, B.hi, n, K, ldb, TCU_BN))) return rc;
    if (nterms == 3) {
        if ((rc = make_kmajor_map(&ta_lo, A.lo, m, K, lda, TCU_BM))) return rc;
        if ((rc = make_kmajor_map(&tb_lo, B.lo, n, K, ldb, TCU_BN))) return rc;
    } else {
        ta_lo = ta_hi;
        tb_lo = tb_hi;
    }
    TcUpdateArgs a;
    a.f16s = f16s ? 1 : 0;
    a.rs_a = f16s ? A.rs : nullptr;
    a.rs_b = f16s ? B.rs : nullptr;
    a.rs_b_vec = f16s && ((uintptr_t)B.rs & 15) == 0;
    a.C = C;
    a.ldc = ldc;
    a.m = m;
    a.n = n;
    a.K = K;
    a.nterms = nterms;
    a.lower = lower;
    a.store = store;
    a.b_lower = b_lower ? 1 : 0;
    a.tiles_m = (m + TCU_BM - 1) / TCU_BM;
    a.tiles_n = (n + TCU_BN - 1) / TCU_BN;
    if (lower) {
        long cnt = 0;
        for (int tn = 0; 2 * tn < a.tiles_m; ++tn) cnt += a.tiles_m - 2 * tn;
        a.num_tiles = (int)cnt;
    } else {
        a.num_tiles = a.tiles_m * a.tiles_n;
    }
    a.tile_begin = std::max(0, std::min(t0, a.num_tiles));
    a.tile_end = t1 < 0 ? a.num_tiles : std::max(a.tile_begin, std::min(t1, a.num_tiles));
    if (a.tile_end <= a.tile_begin) return GB300_OK;
    a.err = d_err;
    a.wait_budget_ns = 2000000000ull;  // 2 s per wait: far above any legitimate stall
    if (int rc = gb300_func_dyn_smem((const void *)tc_update_kernel, TCU_SMEM)) return rc;
    const int ntl = a.tile_end - a.tile_begin;
    const int grid = std::min(ntl, max_grid > 0 ? std::min(max_grid, num_sms()) : num_sms());
    gb300_count_launch(), tc_update_kernel<<<grid, TCU_THREADS, TCU_SMEM, s>>>(ta_hi, ta_lo, tb_hi, tb_lo, a);
    return gb300_last_launch_status();
}

// BF16 operands (the public C-ABI update)
int tc_update(cudaStream_t s, int m, int n, int K, const void *a_hi, const void *a_lo, long lda, const void *b_hi,
              const void *b_lo, long ldb, int nterms, int lower, float *C, long ldc, int *d_err, int store = 0,
              int max_grid = 0)
{
    return tc_update_op(s, m, n, K, {a_hi, a_lo, nullptr}, lda, {b_hi, b_lo, nullptr}, ldb, nterms,
                        lower, C, ldc, d_err, store, max_grid, false);
}

// scaled FP16 panels (the factorisation)
static int tc_update_f16s(cudaStream_t s, int m, int n, int K, const F16Panel &A, long lda, const F16Panel &B,
                          long ldb, int nterms, int lower, float *C, long ldc, int *d_err, int store = 0,
                          int max_grid = 0, int t0 = 0, int t1 = -1, bool b_lower = false)
{
    return tc_update_op(s, m, n, K, {A.h, A.l, A.rs}, lda, {B.h, B.l, B.rs}, ldb, nterms, lower, C, ldc,
                        d_err, store, max_grid, true, t0, t1, b_lower);
}



// Workspace of potrf_tc for order n and tile nb (ldk = nb rounded up to 64):
// two split panels (scaled FP16 h, l: n x ldk each, and n row scales; step
// k's panel is read by its trailing update while step k+1's is written), the
// inverse of the diagonal tile (ldk x ldk FP32) and its split, the diagonal of
// the matrix and its maximum per column tile (the panels' row bounds), the
// doubling scratch of the triangular inverse (ldk x ldk FP32) and the
// diagonal-tile kernel's barrier counter.
struct TcWs {
    F16Panel pan[2], inv;
    float *d, *dtile;
    float *linv, *scratch;
    unsigned *bar;  // grid-barrier counter of the diagonal-tile kernel
};
static size_t tc_ws_layout(int n, int nb, void *base, TcWs *w)
{
    const size_t ldk = ((size_t)(nb > 0 ? nb : 1) + 63) / 64 * 64;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t panel = al((size_t)n * ldk * 2), rsn = scale_bytes(n);
    const size_t inv = ldk * ldk, invh = al(inv * 2), rsk = scale_bytes(ldk);
    const size_t ntiles = nb > 0 ? ((size_t)n + nb - 1) / nb : 1;
    const size_t off_inv = 2 * (2 * panel + 2 * rsn);
    const size_t off_d = off_inv + 2 * invh + 2 * rsk;
    const size_t off_linv = off_d + rsn + al(ntiles * 4);
    if (w && base) {
        char *b = (char *)base;
        for (int i = 0; i < 2; ++i) {
            char *p = b + i * (2 * panel + 2 * rsn);
            w->pan[i] = {(__half *)p, (__half *)(p + panel), (int *)(p + 2 * panel), (float *)(p + 2 * panel + rsn)};
        }
        char *q = b + off_inv;
        w->inv = {(__half *)q, (__half *)(q + invh), (int *)(q + 2 * invh), (float *)(q + 2 * invh + rsk)};
        w->d = (float *)(b + off_d);
        w->dtile = (float *)(b + off_d + rsn);
        w->linv = (float *)(b + off_linv);
        w->scratch = w->linv + inv;
        w->bar = (unsigned *)(w->scratch + inv);
    }
    return off_linv + 2 * inv * 4 + 256;
}

static_assert(DC_MAXN == GB300_DIAG_TILE_MAX, "one limit for the diagonal-tile kernel");

// Factor the FP32 diagonal tile (n <= DC_MAXN) in place and, when `invert`,
// write its lower-triangular inverse to Linv (ld ldi): one cooperative launch
// of diag_coop_kernel, the grid sized to the widest phase and to what can be
// resident at once.
static int diag_factor_inverse(cudaStream_t s, int n, float *A, long lda, float *Linv, long ldi, float *T,
                               unsigned *bar, int *info, int info_base, int *err, bool invert, int max_sms = 0)
{
    static const int occ = [] {
        int o = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, diag_coop_kernel, DC_T, 0) != cudaSuccess) {
            cudaGetLastError();
            o = 1;
        }
        return o;
    }();
    // widest phase: block rows + inverse combines (A), tile updates +
    // inverse products (B), the last row's products
    const int nblk = (n + DC_B - 1) / DC_B;
    int work = 1;
    for (int k = 0; k < nblk; ++k) {
        const int m = nblk - k - 1;
        work = std::max(work, nblk - k + (invert && k >= 2 ? k - 1 : 0));
        if (m > 0) work = std::max(work, m * (m + 1) / 2 + (invert && k >= 1 ? k * (k + 1) / 2 : 0));
    }
    if (invert) work = std::max(work, nblk * (nblk - 1) / 2);
    const int sms = max_sms > 0 ? std::min(max_sms, num_sms()) : num_sms();
    const int grid = std::max(1, std::min(work, sms * std::max(occ, 1)));
    if (invert) cudaMemset2DAsync(Linv, ldi * sizeof(float), 0, n * sizeof(float), n, s);
    cudaMemsetAsync(bar, 0, sizeof(unsigned), s);
    DiagCoopArgs a;
    a.n = n;
    a.A = A;
    a.lda = lda;
    a.Linv = Linv;
    a.ldi = ldi;
    a.T = T;
    a.info = info;
    a.info_base = info_base;
    a.bar = bar;
    a.err = err;
    a.invert = invert ? 1 : 0;
    void *args[] = {&a};
    gb300_count_launch();
    return gb300_record_cuda_error(
        cudaLaunchCooperativeKernel((const void *)diag_coop_kernel, dim3(grid), dim3(DC_T), args, 0, s));
}

// A high-priority stream and a fork / join event pair per host thread and
// device for the trailing updates that run beside the next panel.  The
// priority lets the update's CTAs take their SMs before the panel's kernels
// spread over the GPU.
struct LookaheadStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~LookaheadStream()
    {
        if (s) cudaStreamDestroy(s);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
    }
};

static LookaheadStream *lookahead_stream()
{
    thread_local LookaheadStream ls[16];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return nullptr;
    LookaheadStream &x = ls[dev];
    if (!x.s) {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (cudaStreamCreateWithPriority(&x.s, cudaStreamNonBlocking, greatest) != cudaSuccess ||
            cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    return &x;
}

// SMs the panel of step k+1 keeps while step k's trailing update runs on the
// others.  GB300_LOOKAHEAD_SMS fixes the count (0 runs the steps one after the
// other).  Otherwise the autotuned schedule for the tile size
// (starpu_gb300_dense_autotune, stored beside the perfmodels) gives either a
// fixed count or the parameters of the per-step model; without one the model
// runs on the defaults below.  The model balances the update's 3 m2^2 kb
// flops on the remaining SMs, at the split-precision tensor rate of this
// kernel (default 1.45 PFLOP/s on the whole GPU), against the panel's
// latency-bound diagonal tile (default about 0.75 ms) plus its 6 m2 kb^2
// TRSM flops and the panel splits, which together run at a fraction of that
// rate per SM (default GB300_PANEL_RATE or 0.4: the per-step timeline of the
// n = 32768 solve gave 2.02 ms for a 27648-row panel on 38 SMs).
namespace {
// set by the autotuner for its trials: a fixed count (>= 0), or -1 for the
// model with the parameters below (rate <= 0: the defaults).  Per host
// thread: the trials' factorisations run on the autotuning thread, and a
// factorisation another thread runs meanwhile keeps its own schedule.
thread_local int g_la_trial = -2;
thread_local double g_trial_rate = 0, g_trial_tdiag = 0, g_trial_panel = 0;
} // namespace

static int lookahead_sms(int m2, int kb)
{
    // read once (function-local statics initialise thread-safely)
    static const int fixed = [] {
        const char *e = getenv("GB300_LOOKAHEAD_SMS");
        return e && *e ? std::max(0, atoi(e)) : -1;
    }();
    static const double panel_rate_env = [] {
        const char *r = getenv("GB300_PANEL_RATE");
        return (r && *r && atof(r) > 0.0) ? atof(r) : 0.4;
    }();
    const int S = num_sms();
    if (fixed >= 0) return fixed >= S ? 0 : fixed;
    double rate = 1.45e15, t_diag = 0.75e-3, panel_rate = panel_rate_env;
    const int trial = g_la_trial;
    if (trial >= 0) return trial >= S ? 0 : trial;
    if (trial == -1) {
        if (g_trial_rate > 0) rate = g_trial_rate, t_diag = g_trial_tdiag, panel_rate = g_trial_panel;
    } else {
        DenseTuning t;
        if (dense_tuning(kb, &t)) {
            if (t.lookahead_sms >= 0) return t.lookahead_sms >= S ? 0 : t.lookahead_sms;
            rate = t.update_tflops * 1e12, t_diag = t.t_diag_us * 1e-6, panel_rate = t.panel_rate;
        }
    }
    if (S < 32 || m2 <= 0) return 0;
    const double R = rate / S;
    const double f_upd = 3.0 * m2 * (double)m2 * kb, f_trsm = 6.0 * m2 * (double)kb * kb / panel_rate;
    // below about a quarter of the GPU the diagonal-tile kernel itself slows down
    int best = S / 4;
    double best_t = 1e30;
    for (int L = S / 4; L <= S - 16; L += 8) {
        const double t = std::max(f_upd / (R * (S - L)), t_diag + f_trsm / (R * L));
        if (t < best_t) {
            best_t = t;
            best = L;
        }
    }
    return best;
}

// Panel of the step at column k0 (width kb), in two parts.  panel_diag: the
// FP32 POTRF of the diagonal tile (SIMT, one cooperative launch) and its
// inverse, split for the tensor cores.  panel_solve: the panel TRSM
// P <- P L_kk^-T  as one split-precision product P * Linv^T (store form,
// always 3 products), with P split before and after.  sms > 0 keeps their
// kernels to that many SMs' worth of CTAs.
static int panel_diag(cudaStream_t s, int n, float *A, long lda, int k0, int kb, int nb, const TcWs &w,
                      float *linv_band, int *d_info, int *d_err, int sms)
{
    const long ldk = ((long)nb + 63) / 64 * 64;
    float *Akk = A + k0 + (long)k0 * lda;
    const int m = n - k0 - kb;
    const int slot = gb300_prof_begin(s, GB300_PROF_PANEL);
    int rc = 0;
    // the inverse of the diagonal tile: step k's own block of the band when
    // the caller keeps them all, else the one reused buffer
    float *linv = linv_band ? linv_band + (size_t)(k0 / nb) * ldk * ldk : w.linv;
    if (kb <= DC_MAXN) {
        rc = diag_factor_inverse(s, kb, Akk, lda, linv, ldk, w.scratch, w.bar, d_info, k0, d_err, m > 0 || linv_band,
                                 sms);
    } else {
        potrf_tiled<float>(s, kb, Akk, lda, small_w<float>::value, d_info, k0);
        if (m > 0) trtri_lower<float>(s, kb, Akk, lda, linv, ldk, w.scratch);
    }
    // the inverse split from its row maxima (its elements have no bound from A)
    if (!rc && m > 0) rc = split_f16s(s, kb, kb, linv, ldk, w.inv, ldk);
    gb300_prof_end(s, slot, (double)kb * kb * kb / 3.0, 4.0 * kb * kb);
    return rc;
}

static int panel_solve(cudaStream_t s, int n, float *A, long lda, int k0, int kb, int nb, int np, const TcWs &w,
                       const F16Panel &pan, int *d_err, int sms, bool bounds = true)
{
    const long ldk = ((long)nb + 63) / 64 * 64;
    const int m = n - k0 - kb;
    if (m <= 0) return GB300_OK;
    const int slot = gb300_prof_begin(s, GB300_PROF_PANEL);
    float *P = A + (k0 + kb) + (long)k0 * lda;
    // the panel before its solve bounded by sqrt(d_r max d over the tile's
    // columns), the solved panel by sqrt(d_r) (without the bounds -- the first
    // panel, before the diagonal is saved -- both from their row maxima)
    const float *d = bounds ? w.d : nullptr;
    int rc = split_f16s(s, m, kb, P, lda, pan, ldk, d, k0 + kb, w.dtile + k0 / nb);
    // the inverse is lower triangular: a tile of columns n0 .. n0 + 255 needs k <= n0 + 255 only
    if (!rc) rc = tc_update_f16s(s, m, kb, kb, pan, ldk, w.inv, ldk, 3, 0, P, lda, d_err, 1, sms, 0, -1, true);
    if (!rc) rc = split_f16s(s, m, kb, P, lda, pan, ldk, d, k0 + kb, nullptr);
    // algorithmic work: TRSM m kb^2; bytes: the panel read and written, its split written twice
    gb300_prof_end(s, slot, (double)m * kb * kb, 8.0 * m * kb + 4.0 * m * ldk * np);
    return rc;
}

// Tiled right-looking Cholesky of an FP32 matrix on the tensor cores
// (split-precision products when nterms == 3) with a lookahead of one panel.
// After step k's panel, its rank-kb update is applied first to the next
// column block (its lower diagonal tile and the rectangle below), then step
// k+1's panel -- which needs nothing else -- runs on a few SMs while the rest
// of step k's update (the trailing triangle beyond the next tile) runs on the
// other SMs, from a high-priority stream.  The two write disjoint parts of A
// and read different panel buffers; the streams join before step k+1's
// update.  The diagonal-tile factorisation, latency-bound on a few SMs, thus
// hides behind the trailing update.  (Measured and not kept: factoring only
// the diagonal tile beside the first tiles of the trailing update and
// running the panel's solve and the rest of the update on the whole GPU --
// 75.9 ms per solve at n = 32768 against 70.7: the diagonal tile slows down
// beside other kernels, and the early steps lose the overlap of the solve.)
// `side(s)`, when given, is called once, from the loop, when the step whose
// trailing triangle first has at most `side_rows` rows has been enqueued: the
// caller starts work that only needs the GPU's idle resources there (the
// steps from then on are bound by their latency-bound diagonal tiles).
// `on_panel(s, k0, kb)`, when given, is called after each panel whose
// column block [k0, k0 + kb) has rows below its diagonal tile has been
// enqueued: that block of the factor is final from then on.  `ready`, when
// given, is an event the first update waits for: the first panel reads only
// the first column block, the rest of A may still be being written.
// One split panel per step for TcArrival::panel_store: h and l (n x ldk) and
// the row scales, step after step.
static size_t arrival_panel_bytes(int n, int nb)
{
    const size_t ldk = ((size_t)(nb > 0 ? nb : 1) + 63) / 64 * 64;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return 2 * al((size_t)n * ldk * 2) + 2 * scale_bytes(n);
}

size_t tc_arrival_store_bytes(int n, int nb)
{
    if (n <= 0 || nb <= 0) return 0;
    return ((size_t)n + nb - 1) / nb * arrival_panel_bytes(n, nb);
}

static F16Panel arrival_panel(void *store, int n, int nb, int step)
{
    const size_t ldk = ((size_t)nb + 63) / 64 * 64;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t panel = al((size_t)n * ldk * 2), rsn = scale_bytes(n);
    char *p = (char *)store + (size_t)step * arrival_panel_bytes(n, nb);
    return {(__half *)p, (__half *)(p + panel), (int *)(p + 2 * panel), (float *)(p + 2 * panel + rsn)};
}

int potrf_tc(cudaStream_t s, int n, float *A, long lda, int nb, int nterms, void *work, int *d_info, int *d_err,
             float *linv_band, const std::function<void(cudaStream_t)> &side, int side_rows,
             const std::function<void(cudaStream_t, int, int)> &on_panel, cudaEvent_t ready, const TcArrival *arr)
{
    bool side_done = !side;
    const long ldk = ((long)nb + 63) / 64 * 64;
    TcWs w;
    tc_ws_layout(n, nb, work, &w);
    const int np = nterms == 3 ? 2 : 1;  // split panel arrays an update reads: h, l
    // a step has a trailing triangle beyond its next column block only when n > 2 nb
    LookaheadStream *la = n > 2 * nb ? lookahead_stream() : nullptr;
    // the split panel of step k: two buffers in turn, or one per step when
    // the columns arrive over time (the late columns replay every step)
    auto panel_of = [&](int step) -> F16Panel {
        return arr ? arrival_panel(arr->panel_store, n, nb, step) : w.pan[step & 1];
    };
    // arriving columns: superblocks [0, included) are in the update region,
    // which ends at column avail
    int included = 0;
    long avail = n;
    int rc = 0;
    auto include_below = [&](long col_limit, cudaStream_t st, int steps_done, int max_grid) {
        while (!rc && included < arr->nsb && arr->start[included] < col_limit) {
            const int c0 = arr->start[included], c1 = arr->start[included + 1];
            cudaStreamWaitEvent(st, arr->ready[included], 0);
            // the updates of steps 0 .. steps_done - 1 on the new columns (rows >= c0),
            // in step order: the lower square of the superblock and the rectangle below
            for (int i = 0; i < steps_done && !rc; ++i) {
                const F16Panel pi = panel_of(i);
                const long r0 = (long)(i + 1) * nb;  // the panel's first row
                const int kbi = std::min(nb, n - i * nb);
                const int slot = gb300_prof_begin(st, GB300_PROF_TC_UPDATE);
                rc = tc_update_f16s(st, c1 - c0, c1 - c0, kbi, rows_of(pi, c0 - r0, ldk), ldk, rows_of(pi, c0 - r0, ldk),
                                    ldk, nterms, 1, A + c0 + (long)c0 * lda, lda, d_err, 0, max_grid);
                if (!rc && n > c1)
                    rc = tc_update_f16s(st, n - c1, c1 - c0, kbi, rows_of(pi, c1 - r0, ldk), ldk,
                                        rows_of(pi, c0 - r0, ldk), ldk, nterms, 0, A + c1 + (long)c0 * lda, lda, d_err,
                                        0, max_grid);
                const double w1 = (double)(c1 - c0);
                gb300_prof_end(st, slot, (double)nterms * kbi * (w1 * (w1 + 1.0) + 2.0 * (n - c1) * w1),
                               8.0 * (w1 * (w1 + 1.0) / 2.0 + (double)(n - c1) * w1) + 2.0 * (n - c0) * ldk * np);
            }
            ++included;
        }
        avail = included < arr->nsb ? arr->start[included] : n;
    };
    const int D = arr ? std::max(0, arr->lookahead_blocks) : 0;
    if (arr) include_below(std::min<long>(n, (long)(2 + D) * nb), s, 0, 0);
    if (!rc) rc = panel_diag(s, n, A, lda, 0, std::min(nb, n), nb, w, linv_band, d_info, d_err, 0);
    if (!rc) rc = panel_solve(s, n, A, lda, 0, std::min(nb, n), nb, np, w, panel_of(0), d_err, 0, false);
    if (ready) cudaStreamWaitEvent(s, ready, 0);
    // the diagonal of the matrix (rows past the first tile, which no step has
    // touched yet) and its maxima per column tile: the later panels' row bounds
    if (!rc && n > nb) {
        const int ntiles = (n + nb - 1) / nb;
        gb300_count_launch(), diag_bounds_kernel<<<ntiles, 256, 0, s>>>(n, A, lda, nb, w.d, w.dtile,
                                                                        arr ? arr->diag : nullptr);
        rc = gb300_last_launch_status();
    }
    if (!rc && on_panel && n > nb) on_panel(s, 0, nb);
    int step = 0;
    for (int k0 = 0; k0 < n && !rc; k0 += nb, ++step) {
        const int kb = std::min(nb, n - k0);
        const int m = n - k0 - kb;
        if (m <= 0) break;
        const F16Panel pan = panel_of(step);
        const int kb1 = std::min(nb, m);  // width of the next column block
        const int m2 = m - kb1;           // rows and columns beyond it
        float *C11 = A + (k0 + kb) + (long)(k0 + kb) * lda;
        // the next column block: its diagonal tile (lower) and the rectangle below
        int slot = gb300_prof_begin(s, GB300_PROF_TC_UPDATE);
        rc = tc_update_f16s(s, kb1, kb1, kb, pan, ldk, pan, ldk, nterms, 1, C11, lda, d_err);
        if (!rc && m2 > 0)
            rc = tc_update_f16s(s, m2, kb1, kb, rows_of(pan, kb1, ldk), ldk, pan, ldk, nterms, 0, C11 + kb1, lda, d_err);
        // algorithmic work: the lower triangle of the kb1 tile and the m2 x kb1
        // rectangle, per term; bytes: C read + written in FP32, the panels read
        gb300_prof_end(s, slot, (double)nterms * kb * ((double)kb1 * (kb1 + 1.0) + 2.0 * m2 * kb1),
                       8.0 * ((double)kb1 * (kb1 + 1.0) / 2.0 + (double)m2 * kb1) + 2.0 * m * ldk * np);
        if (rc) break;
        float *C22 = C11 + kb1 + (long)kb1 * lda;
        const F16Panel pan2 = rows_of(pan, kb1, ldk);
        const F16Panel next = panel_of(step + 1);
        // the trailing update of this step: the lower triangle of the columns
        // [k0 + kb + kb1, avail) and, when columns are still to arrive, the
        // rectangle below it (avail = n: the whole trailing triangle)
        auto trailing = [&](cudaStream_t st, int max_grid) {
            if (arr) include_below(std::min<long>(n, (long)(step + 3 + D) * nb), st, step, max_grid);
            const int ms = (int)(avail - (k0 + kb + kb1));  // columns of the region
            if (rc || ms <= 0) return;
            const double f2 = (double)nterms * kb * ((double)ms * (ms + 1.0) + 2.0 * (m2 - ms) * ms);
            const double b2 = 8.0 * ((double)ms * (ms + 1.0) / 2.0 + (double)(m2 - ms) * ms) + 2.0 * m2 * ldk * np;
            const int slot2 = gb300_prof_begin(st, GB300_PROF_TC_UPDATE);
            if (max_grid > 0) gb300_prof_set_share(slot2, (double)max_grid / num_sms());
            rc = tc_update_f16s(st, ms, ms, kb, pan2, ldk, pan2, ldk, nterms, 1, C22, lda, d_err, 0, max_grid);
            if (!rc && m2 > ms)
                rc = tc_update_f16s(st, m2 - ms, ms, kb, rows_of(pan2, ms, ldk), ldk, pan2, ldk, nterms, 0, C22 + ms,
                                    lda, d_err, 0, max_grid);
            gb300_prof_end(st, slot2, f2, b2);
        };
        const int la_sms = lookahead_sms(m2, kb);
        if (m2 > 0 && la && la_sms > 0) {
            cudaEventRecord(la->fork, s);
            cudaStreamWaitEvent(la->s, la->fork, 0);
            trailing(la->s, num_sms() - la_sms);
            cudaEventRecord(la->join, la->s);
            if (!rc) rc = panel_diag(s, n, A, lda, k0 + kb, kb1, nb, w, linv_band, d_info, d_err, la_sms);
            if (!rc) rc = panel_solve(s, n, A, lda, k0 + kb, kb1, nb, np, w, next, d_err, la_sms);
            if (!rc && on_panel) on_panel(s, k0 + kb, kb1);
            cudaStreamWaitEvent(s, la->join, 0);  // joined before step k+1's update
        } else {
            if (m2 > 0) trailing(s, 0);
            else if (arr) include_below(n, s, step, 0);
            if (!rc) rc = panel_diag(s, n, A, lda, k0 + kb, kb1, nb, w, linv_band, d_info, d_err, 0);
            if (!rc) rc = panel_solve(s, n, A, lda, k0 + kb, kb1, nb, np, w, next, d_err, 0);
            if (!rc && on_panel && m2 > 0) on_panel(s, k0 + kb, kb1);
        }
        if (!side_done && m2 <= side_rows) {
            side(s);
            side_done = true;
        }
    }
    if (!side_done) side(s);
    if (rc) return rc;
    return gb300_last_launch_status();
}

// ---- residual partials on the tensor cores (sliced fixed-point products) ----

static long rtc_ldk(int n) { return ((long)n + 63) / 64 * 64; }

size_t residual_tc_a_bytes(int n) { return n > 0 ? (size_t)8 * n * rtc_ldk(n) * 2 : 0; }

// The 8 digit slices of the symmetric A (lower triangle read), once per
// matrix, scaled by 2^alpha with max |A_ij| < 2^alpha (amax_bits: that max as
// FP64 bits).  rowsum (optional): the per-tile row sums for the norm.
int residual_tc_slice_a(cudaStream_t s, int n, const double *A, long lda, const unsigned long long *amax_bits,
                        void *slices, float *rowsum)
{
    if (n <= 0) return GB300_OK;
    const long ldk = rtc_ldk(n);
    // the kernel writes every column below round8(n); only the padding beyond it needs zeros
    const long kw = ((long)n + 7) / 8 * 8;
    if (ldk > kw)
        cudaMemset2DAsync((uint16_t *)slices + kw, ldk * 2, 0, (ldk - kw) * 2, (size_t)8 * n, s);
    const unsigned nt = (unsigned)((n + 63) / 64);
    gb300_count_launch(), rtc_a_slices_kernel<<<dim3(nt, nt), 256, 0, s>>>(n, A, lda, amax_bits, (uint16_t *)slices,
                                                                           ldk, rowsum);
    return gb300_last_launch_status();
}

size_t residual_tc_xs_bytes(int n, int nrhs)
{
    const long groups = (nrhs + 15) / 16;
    return (size_t)groups * RTC_XROWS * rtc_ldk(n) * 2;
}

// K chunk of the tensor-core residual: a multiple of the exact accumulation
// block, with enough work items (128-row block x chunk x group of 16) for a
// few per SM, and at most max_chunks chunks (the partials buffer).
int residual_tc_kchunk(int n, int nrhs, int max_chunks)
{
    const long items = (long)((n + RTC_BM - 1) / RTC_BM) * ((nrhs + 15) / 16);
    long nk = (4L * num_sms() + items - 1) / items;
    nk = std::max(1L, std::min<long>(max_chunks, nk));
    long kc = ((n + nk - 1) / nk + RTC_KBLK - 1) / RTC_KBLK * RTC_KBLK;
    return (int)std::max<long>(kc, RTC_KBLK);
}

// P_z = -(A X) over the K chunks z of length kchunk, with the slices of the
// symmetric A from residual_tc_slice_a.  sx: ilogb(max |x_j|) per column
// (device), amax_bits: max |A_ij| (device, the slices' scale).  xs:
// residual_tc_xs_bytes(n, nrhs) bytes of scratch.
int residual_tc(cudaStream_t s, int n, int nrhs, const void *a_slices, const double *X, long ldx, const int *sx,
                const unsigned long long *amax_bits, int kchunk, void *xs, double *partials, int *d_err)
{
    if (n <= 0 || nrhs <= 0) return GB300_OK;
    if (kchunk % RTC_KBLK || !d_err) return GB300_EINVAL;
    const long ldk = rtc_ldk(n);
    const int groups = (nrhs + 15) / 16;
    uint16_t *Xs = (uint16_t *)xs;
    cudaMemsetAsync(xs, 0, residual_tc_xs_bytes(n, nrhs), s);
    for (int g = 0; g < groups; ++g) {
        const int nc = std::min(16, nrhs - 16 * g);
        gb300_count_launch(), rtc_x_slices_kernel<<<dim3((unsigned)((ldk + 255) / 256), 16), 256, 0, s>>>(
            n, nc, X + (long)g * 16 * ldx, ldx, sx + 16 * g, Xs + (long)g * RTC_XROWS * ldk, ldk);
    }
    CUtensorMap tm, tma;
    int rc = make_kmajor_map(&tm, xs, groups * RTC_XROWS, (int)ldk, ldk, RTC_XROWS);
    if (!rc) rc = make_kmajor_map(&tma, a_slices, 8 * n, (int)ldk, ldk, RTC_BM);
    if (rc) return rc;
    ResidualTcArgs a;
    a.n = n;
    a.nrhs = nrhs;
    a.amax_bits = amax_bits;
    a.sx = sx;
    a.kchunk = kchunk;
    a.nblocks = (n + RTC_BM - 1) / RTC_BM;
    a.nchunks = (n + kchunk - 1) / kchunk;
    a.ngroups = groups;
    a.nitems = a.nblocks * a.nchunks * a.ngroups;
    a.P = partials;
    a.err = d_err;
    a.wait_budget_ns = 2000000000ull;  // 2 s per wait: far above any legitimate stall
    if (int rc2 = gb300_func_dyn_smem((const void *)residual_tc_kernel, RTC_SMEM)) return rc2;
    const int grid = std::min(a.nitems, num_sms());
    gb300_count_launch(), residual_tc_kernel<<<grid, RTC_THREADS, RTC_SMEM, s>>>(tma, tm, a);
    return gb300_last_launch_status();
}

} // namespace gb300

using namespace gb300;

extern "C" {

int starpu_gb300_split_bf16(void *stream, int m, int k, const float *P, int ldp, void *hi, void *lo, int ldk)
{
    if (m < 0 || k < 0 || ldp < (m > 1 ? m : 1) || ldk < k) return GB300_EINVAL;
    return split_bf16((cudaStream_t)stream, m, k, P, ldp, hi, lo, ldk);
}

int starpu_gb300_tc_update(void *stream, int m, int n, int k, const void *a_hi, const void *a_lo, int lda,
                           const void *b_hi, const void *b_lo, int ldb, int nterms, int lower, float *C, int ldc,
                           int *d_err)
{
    if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) || lda < k || ldb < k) return GB300_EINVAL;
    return tc_update((cudaStream_t)stream, m, n, k, a_hi, a_lo, lda, b_hi, b_lo, ldb, nterms, lower, C, ldc, d_err);
}

size_t starpu_gb300_spotrf_tc_workspace(int n, int nb) { return tc_ws_layout(n < 0 ? 0 : n, nb, nullptr, nullptr); }

int starpu_gb300_spotrf_tc(void *stream, int n, float *A, int lda, int nb, int nterms, void *work, size_t lwork,
                           int *d_info, int *d_err)
{
    if (n < 0 || lda < (n > 1 ? n : 1) || nb <= 0 || (nterms != 1 && nterms != 3) || !d_err) return GB300_EINVAL;
    if (lwork < starpu_gb300_spotrf_tc_workspace(n, nb) || !work) return GB300_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (d_info) cudaMemsetAsync(d_info, 0, sizeof(int), s);
    if (!n) return GB300_OK;
    return potrf_tc(s, n, A, lda, nb, nterms, work, d_info, d_err, nullptr, {}, 0, {}, nullptr);
}

// ---- tensor-core tile update for the codelets -----------------------------
//
// Workspace: the row-scaled FP16 splits of A (m rows) and B (n rows) for
// m, n, k <= nmax: h and l (K-major, row stride round64(k)) and the row
// exponents of each operand.
static size_t tile_tc_operand_bytes(int rows, long ldk)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return 2 * al((size_t)rows * ldk * 2) + 2 * scale_bytes(rows);
}

static F16Panel tile_tc_operand(void *base, int rows, long ldk)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    char *p = (char *)base;
    const size_t half = al((size_t)rows * ldk * 2);
    return {(__half *)p, (__half *)(p + half), (int *)(p + 2 * half), (float *)(p + 2 * half + scale_bytes(rows))};
}

size_t starpu_gb300_tile_tc_workspace(int nmax)
{
    if (nmax <= 0) return 0;
    const long ldk = ((long)nmax + 63) / 64 * 64;
    return 2 * tile_tc_operand_bytes(nmax, ldk);
}

int starpu_gb300_tile_tc_prepare(void)
{
    return gb300_func_dyn_smem((const void *)tc_update_kernel, TCU_SMEM);
}

int starpu_gb300_sgemm_nt_tile_tc(void *stream, int m, int n, int k, const float *A, int lda, const float *B,
                                  int ldb, float *C, int ldc, int lower, void *work, size_t lwork, int *d_err)
{
    if (m < 0 || n < 0 || k < 0 || lda < (m > 1 ? m : 1) || ldb < (n > 1 ? n : 1) || ldc < (m > 1 ? m : 1) ||
        (lower && m != n) || !d_err || !work)
        return GB300_EINVAL;
    const int nmax = std::max(m, std::max(n, k));
    if (lwork < starpu_gb300_tile_tc_workspace(nmax)) return GB300_EINVAL;
    if (!m || !n || !k) return GB300_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const long ldk = ((long)k + 63) / 64 * 64;
    const F16Panel pa = tile_tc_operand(work, m, ldk);
    int rc = split_f16s(s, m, k, A, lda, pa, ldk);
    F16Panel pb = pa;
    if (!rc && !(B == A && n == m && ldb == lda)) {
        pb = tile_tc_operand((char *)work + tile_tc_operand_bytes(m, ldk), n, ldk);
        rc = split_f16s(s, n, k, B, ldb, pb, ldk);
    }
    if (!rc) rc = tc_update_f16s(s, m, n, k, pa, ldk, pb, ldk, 3, lower ? 1 : 0, C, ldc, d_err);
    return rc;
}

// A x A FP32 matrix 1/(1+i+j) + n delta_ij (the tuning input: SPD, and the
// factorisation's time does not depend on the values)
__global__ void fill_hilbert_f32_kernel(int n, float *A, long lda)
{
    const long total = (long)n * n;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        A[i + (long)j * lda] = 1.0f / (1.0f + i + j) + (i == j ? (float)n : 0.0f);
    }
}

int starpu_gb300_dense_autotune(int n, int nb, int reps)
{
    if (nb < 64 || nb > DC_MAXN || n < 3 * nb) return GB300_EINVAL;
    if (reps <= 0) reps = 2;
    const int S = num_sms();
    const int L = std::max(1, S / 4);
    const long ldk = ((long)nb + 63) / 64 * 64;
    const size_t lw = tc_ws_layout(n, nb, nullptr, nullptr);
    float *A0 = nullptr, *A = nullptr;
    void *work = nullptr;
    int *flags = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = gb300_record_cuda_error(cudaMalloc(&A0, sizeof(float) * (size_t)n * n));
    if (!rc) rc = gb300_record_cuda_error(cudaMalloc(&A, sizeof(float) * (size_t)n * n));
    if (!rc) rc = gb300_record_cuda_error(cudaMalloc(&work, lw));
    if (!rc) rc = gb300_record_cuda_error(cudaMalloc(&flags, 2 * sizeof(int)));
    if (!rc) rc = gb300_record_cuda_error(cudaMemset(flags, 0, 2 * sizeof(int)));
    if (!rc) rc = gb300_record_cuda_error(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    if (!rc) rc = gb300_record_cuda_error(cudaEventCreate(&e0));
    if (!rc) rc = gb300_record_cuda_error(cudaEventCreate(&e1));
    DenseTuning best;
    best.nb = nb;
    best.n = n;
    auto timed = [&](const std::function<int()> &fn, double *ms_out) -> int {
        double tot = 0;
        for (int r = 0; r <= reps; ++r) {
            int rc2 = gb300_record_cuda_error(cudaEventRecord(e0, s));
            if (!rc2) rc2 = fn();
            if (!rc2) rc2 = gb300_record_cuda_error(cudaEventRecord(e1, s));
            if (!rc2) rc2 = gb300_record_cuda_error(cudaEventSynchronize(e1));
            if (rc2) return rc2;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) tot += ms;  // the first run is a warm-up
        }
        *ms_out = tot / reps;
        return GB300_OK;
    };
    if (!rc) {
        gb300_count_launch(), fill_hilbert_f32_kernel<<<1024, 256, 0, s>>>(n, A0, n);
        rc = gb300_last_launch_status();
    }
    TcWs w;
    tc_ws_layout(n, nb, work, &w);
    if (!rc) rc = gb300_record_cuda_error(cudaMemsetAsync(work, 0, lw, s));
    int *d_info = flags, *d_err = flags + 1;
    // 1. the diagonal tile (factor + inverse) on a quarter of the SMs
    double t_diag_ms = 0;
    if (!rc)
        rc = timed([&] {
            cudaMemcpy2DAsync(A, sizeof(float) * n, A0, sizeof(float) * n, sizeof(float) * nb, nb,
                              cudaMemcpyDeviceToDevice, s);
            return diag_factor_inverse(s, nb, A, n, w.linv, ldk, w.scratch, w.bar, d_info, 0, d_err, true, L);
        }, &t_diag_ms);
    // 2. the trailing update (lower m x m, K = nb, 3 products) on the whole GPU
    const int m = std::min(n - nb, 8192);
    double t_upd_ms = 0, t_panel_ms = 0;
    if (!rc)
        rc = timed([&] { return tc_update_f16s(s, m, m, nb, w.pan[0], ldk, w.pan[0], ldk, 3, 1, A, n, d_err); },
                   &t_upd_ms);
    // 3. the panel solve (store form m x nb, K = nb) on the same quarter
    if (!rc)
        rc = timed([&] { return tc_update_f16s(s, m, nb, nb, w.pan[0], ldk, w.inv, ldk, 3, 0, A, n, d_err, 1, L); },
                   &t_panel_ms);
    if (!rc) {
        best.t_diag_us = t_diag_ms * 1e3;
        const double rate = 3.0 * nb * (double)m * (m + 1.0) / (t_upd_ms * 1e-3);
        best.update_tflops = rate / 1e12;
        best.panel_rate = (6.0 * m * (double)nb * nb / (t_panel_ms * 1e-3)) / (rate * L / S);
    }
    // 4. whole factorisations: the model on these parameters, and fixed splits
    const int cands[5] = {-1, S / 4, S / 3, S / 2, 0};
    best.step_ms = INFINITY;
    for (int c = 0; c < 5 && !rc; ++c) {
        g_trial_rate = best.update_tflops * 1e12;
        g_trial_tdiag = best.t_diag_us * 1e-6;
        g_trial_panel = best.panel_rate;
        g_la_trial = cands[c];
        double ms = 0;
        rc = timed([&] {
            cudaMemcpyAsync(A, A0, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, s);
            return potrf_tc(s, n, A, n, nb, 3, work, d_info, d_err, nullptr, {}, 0, {}, nullptr);
        }, &ms);
        g_la_trial = -2;
        if (!rc && ms < best.step_ms) {
            best.step_ms = ms;
            best.lookahead_sms = cands[c];
        }
    }
    int hflags[2] = {0, 0};
    if (!rc) rc = gb300_record_cuda_error(cudaMemcpy(hflags, flags, sizeof hflags, cudaMemcpyDeviceToHost));
    if (!rc && (hflags[0] || hflags[1])) {
        gb300_set_error("starpu_gb300_dense_autotune: the tuning factorisation failed");
        rc = GB300_EINVAL;
    }
    if (s) cudaStreamSynchronize(s);
    cudaFree(A0);
    cudaFree(A);
    cudaFree(work);
    cudaFree(flags);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (rc) return rc;
    return dense_tuning_store(best);
}

int starpu_gb300_dense_get_tuning(int nb, int *lookahead_sms, double *t_diag_us, double *update_tflops,
                                  double *panel_rate, double *step_ms)
{
    DenseTuning t;
    if (!dense_tuning(nb, &t)) return 0;
    if (lookahead_sms) *lookahead_sms = t.lookahead_sms;
    if (t_diag_us) *t_diag_us = t.t_diag_us;
    if (update_tflops) *update_tflops = t.update_tflops;
    if (panel_rate) *panel_rate = t.panel_rate;
    if (step_ms) *step_ms = t.step_ms;
    return 1;
}

} // extern "C"
