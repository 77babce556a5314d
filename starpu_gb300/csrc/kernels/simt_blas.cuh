// SIMT (CUDA-core) dense kernels for the tiled Cholesky path, FP32 and FP64.
//
// These are the building blocks that the tile codelets and the whole-matrix
// drivers compose.  They replace, for the plain (non-tensor-core) precisions,
// the vendor calls the reference codelets make on the CUDA worker stream:
//   cublasSgemm(N,T)      examples/cholesky/cholesky_kernels.c:98
//   cublasSsyrk(L,N)      examples/cholesky/cholesky_kernels.c:177
//   cublasStrsm(R,L,T,N)  examples/cholesky/cholesky_kernels.c:258
//   cusolverDnSpotrf(L)   examples/cholesky/cholesky_kernels.c:354
// All matrices are column-major with an explicit leading dimension, exactly
// like the StarPU matrix interface (nx rows contiguous, ld >= nx).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

namespace gb300 {

// ---------------------------------------------------------------------------
// GEMM:  C[m x n] = beta*C + alpha * op(A)[m x k] * op(B)[k x n]
//   TA=false: op(A)(i,p) = A[i + p*lda]     TA=true: op(A)(i,p) = A[p + i*lda]
//   TB=false: op(B)(p,j) = B[p + j*ldb]     TB=true: op(B)(p,j) = B[j + p*ldb]
// LOWER (requires m == n, BM == BN): only blocks on/below the diagonal are
// launched (triangular grid) and only elements with i >= j are written.  This
// is the SYRK "L" update and the whole-trailing-matrix update.
// Each thread owns a TM x TN register tile split in two halves along both
// axes (rows h*BM/2 + tr*TM/2 + v) so shared-memory reads are vectorised and
// bank-conflict free, and global C accesses stay coalesced.
// ---------------------------------------------------------------------------
template <typename T> struct vec2_of;
template <> struct vec2_of<float> { typedef float2 type; };
template <> struct vec2_of<double> { typedef double2 type; };

// K split (kchunk > 0): blockIdx.z takes the K range [z*kchunk, (z+1)*kchunk)
// and writes its partial product to C + z*cstride (beta applies to each
// partial); a separate pass reduces the partials in a fixed order, so the
// result does not depend on scheduling.
// Batch (kchunk < 0): blockIdx.z is the problem index; its A, B and C start
// at A + z*astride, B + z*bstride, C + z*cstride.
template <typename T, bool TA, bool TB, int BM, int BN, int BK, int TM, int TN, bool LOWER>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_simt_kernel(int m, int n, int k, T alpha, const T *__restrict__ A, long lda,
                 const T *__restrict__ B, long ldb, T beta, T *__restrict__ C, long ldc, int kchunk = 0,
                 long cstride = 0, long astride = 0, long bstride = 0)
{
    if (kchunk > 0) {
        const int kz = blockIdx.z * kchunk;
        k = min(kchunk, k - kz);
        A += TA ? (long)kz : (long)kz * lda;
        B += TB ? (long)kz * ldb : (long)kz;
        C += (long)blockIdx.z * cstride;
    } else if (kchunk < 0) {
        A += (long)blockIdx.z * astride;
        B += (long)blockIdx.z * bstride;
        C += (long)blockIdx.z * cstride;
    }
    constexpr int RG = BM / TM;            // row groups
    constexpr int CG = BN / TN;            // column groups
    constexpr int NT = RG * CG;
    constexpr int PADA = 16 / sizeof(T);   // keeps rows 16B aligned, breaks bank aliasing
    constexpr int LDA_S = BM + PADA;
    constexpr int LDB_S = BN + PADA;
    constexpr int LA = (BM * BK + NT - 1) / NT;
    constexpr int LB = (BN * BK + NT - 1) / NT;
    static_assert(TM % 2 == 0 || TM == 1, "TM even");
    __shared__ __align__(16) T As[2][BK][LDA_S];
    __shared__ __align__(16) T Bs[2][BK][LDB_S];

    int bi, bj;
    if (LOWER) {
        // triangular block index t -> (bi >= bj)
        long t = blockIdx.x;
        long r = (long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
        while ((r + 1) * (r + 2) / 2 <= t) ++r;
        while (r * (r + 1) / 2 > t) --r;
        bi = (int)r;
        bj = (int)(t - r * (r + 1) / 2);
    } else {
        bi = blockIdx.x;
        bj = blockIdx.y;
    }
    const int m0 = bi * BM, n0 = bj * BN;
    const int tid = threadIdx.x;
    const int tr = tid % RG, tc = tid / RG;

    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

    T ra[LA], rb[LB];
    auto load_a = [&](int k0) {
#pragma unroll
        for (int l = 0; l < LA; ++l) {
            int idx = tid + l * NT;
            int i, p;
            if (!TA) { i = idx % BM; p = idx / BM; } else { p = idx % BK; i = idx / BK; }
            T v = T(0);
            if (idx < BM * BK && m0 + i < m && k0 + p < k)
                v = TA ? A[(long)(k0 + p) + (long)(m0 + i) * lda] : A[(long)(m0 + i) + (long)(k0 + p) * lda];
            ra[l] = v;
        }
    };
    auto load_b = [&](int k0) {
#pragma unroll
        for (int l = 0; l < LB; ++l) {
            int idx = tid + l * NT;
            int j, p;
            if (TB) { j = idx % BN; p = idx / BN; } else { p = idx % BK; j = idx / BK; }
            T v = T(0);
            if (idx < BN * BK && n0 + j < n && k0 + p < k)
                v = TB ? B[(long)(n0 + j) + (long)(k0 + p) * ldb] : B[(long)(k0 + p) + (long)(n0 + j) * ldb];
            rb[l] = v;
        }
    };
    auto store_ab = [&](int buf) {
#pragma unroll
        for (int l = 0; l < LA; ++l) {
            int idx = tid + l * NT;
            if (idx < BM * BK) {
                int i, p;
                if (!TA) { i = idx % BM; p = idx / BM; } else { p = idx % BK; i = idx / BK; }
                As[buf][p][i] = ra[l];
            }
        }
#pragma unroll
        for (int l = 0; l < LB; ++l) {
            int idx = tid + l * NT;
            if (idx < BN * BK) {
                int j, p;
                if (TB) { j = idx % BN; p = idx / BN; } else { p = idx % BK; j = idx / BK; }
                Bs[buf][p][j] = rb[l];
            }
        }
    };

    const int nk = (k + BK - 1) / BK;
    if (nk > 0) {
        load_a(0);
        load_b(0);
        store_ab(0);
    }
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        const int cur = kt & 1;
        if (kt + 1 < nk) { load_a((kt + 1) * BK); load_b((kt + 1) * BK); }
#pragma unroll
        for (int p = 0; p < BK; ++p) {
            T a[TM], b[TN];
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int v = 0; v < TM / 2; ++v) a[h * (TM / 2) + v] = As[cur][p][h * (BM / 2) + tr * (TM / 2) + v];
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int v = 0; v < TN / 2; ++v) b[h * (TN / 2) + v] = Bs[cur][p][h * (BN / 2) + tc * (TN / 2) + v];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        if (kt + 1 < nk) store_ab(cur ^ 1);
        __syncthreads();
    }

#pragma unroll
    for (int jj = 0; jj < TN; ++jj) {
        const int j = n0 + (jj / (TN / 2)) * (BN / 2) + tc * (TN / 2) + (jj % (TN / 2));
        if (j >= n) continue;
#pragma unroll
        for (int ii = 0; ii < TM; ++ii) {
            const int i = m0 + (ii / (TM / 2)) * (BM / 2) + tr * (TM / 2) + (ii % (TM / 2));
            if (i >= m) continue;
            if (LOWER && i < j) continue;
            T *c = &C[(long)i + (long)j * ldc];
            T old = (beta == T(0)) ? T(0) : beta * (*c);
            *c = fma(alpha, acc[ii][jj], old);
        }
    }
}

// ---------------------------------------------------------------------------
// Unblocked Cholesky of one n x n (n <= NMAX) diagonal block, lower, held in
// registers.  Same arithmetic as the reference CPU codelet loop
// (examples/cholesky/cholesky_kernels.c:329-342): lambda = sqrt(a_zz),
// scale the column by 1/lambda, rank-1 update of the trailing lower part.
// A non-positive (or NaN) pivot records info = info_base + z + 1 (LAPACK
// convention, first failure wins) in *info; the kernel never traps.
// ---------------------------------------------------------------------------
template <typename T, int NMAX>
__global__ void __launch_bounds__(256) potf2_small_kernel(int n, T *__restrict__ A, long lda, int *info, int info_base)
{
    // 256 threads as NMAX rows x CL column lanes; thread (ti, tc) keeps row ti,
    // columns tc, tc + CL, ... in registers.  The step loop is unrolled so
    // that column z lives in a fixed register of its owners; the owners
    // publish column z through a double-buffered shared vector (one barrier
    // per step), every thread scales its two factors by 1/sqrt(a_zz) itself.
    constexpr int CL = 256 / NMAX, NC = NMAX / CL;
    __shared__ T col[2][NMAX];
    const int tid = threadIdx.x;
    const int ti = tid % NMAX, tc = tid / NMAX;
    T a[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        const int c = tc + q * CL;
        a[q] = (ti < n && c <= ti) ? A[(long)ti + (long)c * lda] : T(0);
    }
    bool bad = false;
#pragma unroll
    for (int z = 0; z < NMAX; ++z) {
        if (z >= n) break;
        T *cz = col[z & 1];
        if (tc == z % CL) cz[ti] = a[z / CL];  // owners of column z publish it (rows < z hold 0)
        __syncthreads();
        const T d = cz[z];
        if (!(d > T(0)) && !bad) {
            bad = true;
            if (tid == 0 && info) atomicCAS(info, 0, info_base + z + 1);
        }
        const T lzz = sqrt(d);
        const T inv = T(1) / lzz;
        const T li = cz[ti] * inv;
        if (tc == z % CL) a[z / CL] = (ti == z) ? lzz : (ti > z ? li : a[z / CL]);
        if (ti > z) {
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const int c = tc + q * CL;
                if (c > z && c <= ti) a[q] = fma(-li, cz[c] * inv, a[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        const int c = tc + q * CL;
        if (ti < n && c <= ti) A[(long)ti + (long)c * lda] = a[q];
    }
}

// ---------------------------------------------------------------------------
// B[m x w] <- B * L^{-T}, L w x w lower non-unit (w <= W): the right-side
// TRSM of the panel (cublasStrsm(R,L,T,N), cholesky_kernels.c:258) for one
// column block.  Every row of B is an independent forward substitution; one
// thread owns one row in registers.  Column-oriented order like reference
// BLAS strsm: x_j *= 1/L_jj, then x_c -= L_cj * x_j for c > j.
// ---------------------------------------------------------------------------
template <typename T, int W, bool FULL>
__global__ void __launch_bounds__(128) trsm_rltn_small_kernel(int m, int w, const T *__restrict__ L, long ldl,
                                                              T *__restrict__ B, long ldb)
{
    __shared__ T Ls[W][W + 1];
    __shared__ T invd[W];
    const int tid = threadIdx.x;
    const int ww = FULL ? W : w;
    for (int idx = tid; idx < W * W; idx += blockDim.x) {
        int i = idx % W, j = idx / W;
        Ls[i][j] = (i < ww && j < ww && i >= j) ? L[(long)i + (long)j * ldl] : T(0);
    }
    __syncthreads();
    for (int j = tid; j < W; j += blockDim.x) invd[j] = (j < ww) ? T(1) / Ls[j][j] : T(0);
    __syncthreads();
    const long r = (long)blockIdx.x * blockDim.x + tid;
    if (r >= m) return;
    T x[W];
#pragma unroll
    for (int c = 0; c < W; ++c) x[c] = (FULL || c < ww) ? B[r + (long)c * ldb] : T(0);
#pragma unroll
    for (int j = 0; j < W; ++j) {
        x[j] *= invd[j];
#pragma unroll
        for (int c = j + 1; c < W; ++c) x[c] = fma(-Ls[c][j], x[j], x[c]);
    }
#pragma unroll
    for (int c = 0; c < W; ++c)
        if (FULL || c < ww) B[r + (long)c * ldb] = x[c];
}

// ---------------------------------------------------------------------------
// Left-side small triangular solves on a w x nrhs block (w <= W), one thread
// per right-hand side.  Used by the blocked POTRS (forward L y = b, backward
// L^T x = y), mirroring LAPACK dpotrs (min-dgels/base/SRC/dpotrs.c): two
// triangular sweeps with the Cholesky factor.
// ---------------------------------------------------------------------------
template <typename T, int W, bool TRANS>
__global__ void __launch_bounds__(64) trsm_left_small_kernel(int w, int nrhs, const T *__restrict__ L, long ldl,
                                                             T *__restrict__ B, long ldb)
{
    __shared__ T Ls[W][W + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < W * W; idx += blockDim.x) {
        int i = idx % W, j = idx / W;
        Ls[i][j] = (i < w && j < w && i >= j) ? L[(long)i + (long)j * ldl] : T(i == j ? 1 : 0);
    }
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + tid;
    if (c >= nrhs) return;
    T x[W];
#pragma unroll
    for (int i = 0; i < W; ++i) x[i] = (i < w) ? B[(long)i + (long)c * ldb] : T(0);
    if (!TRANS) {
#pragma unroll
        for (int j = 0; j < W; ++j) {
            x[j] = x[j] / Ls[j][j];
#pragma unroll
            for (int i = j + 1; i < W; ++i) x[i] = fma(-Ls[i][j], x[j], x[i]);
        }
    } else {
#pragma unroll
        for (int j = W - 1; j >= 0; --j) {
            x[j] = x[j] / Ls[j][j];
#pragma unroll
            for (int i = 0; i < j; ++i) x[i] = fma(-Ls[j][i], x[j], x[i]);
        }
    }
#pragma unroll
    for (int i = 0; i < W; ++i)
        if (i < w) B[(long)i + (long)c * ldb] = x[i];
}

// ---------------------------------------------------------------------------
// Diagonal-block solve of the blocked POTRS with wide blocks (w <= W, W up
// to 128): L_ii (w x w) and 16 right-hand-side columns of the block are
// staged in shared memory; each column is owned by 8 consecutive lanes that
// compute one row at a time as a dot product split 8 ways and reduced with
// shuffles, so rows advance with warp-level synchronisation only.
//   TRANS = false: y_r = (b_r - sum_{c<r} L_rc y_c) / L_rr,  r = 0..w-1
//   TRANS = true : x_r = (y_r - sum_{c>r} L_cr x_c) / L_rr,  r = w-1..0
// Launch: ceil(nrhs / 16) CTAs of 128 threads, dynamic shared memory
// (W * (W + 1) + W * 16) * sizeof(T).
// ---------------------------------------------------------------------------
template <typename T, int W, bool TRANS>
__global__ void __launch_bounds__(128) trsv_block_kernel(int w, int nrhs, const T *__restrict__ L, long ldl,
                                                         T *__restrict__ B, long ldb)
{
    extern __shared__ __align__(16) unsigned char trsv_smem[];
    T *Ls = (T *)trsv_smem;            // [W][W+1], Ls[r * (W+1) + c] = L(r, c)
    T *Ys = Ls + W * (W + 1);          // [16][W]
    const int tid = threadIdx.x;
    const int col0 = blockIdx.x * 16;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        Ls[r * (W + 1) + c] = (r >= c) ? L[(long)r + (long)c * ldl] : T(0);
    }
    for (int idx = tid; idx < 16 * w; idx += blockDim.x) {
        const int r = idx % w, j = idx / w;
        Ys[j * W + r] = (col0 + j < nrhs) ? B[(long)r + (long)(col0 + j) * ldb] : T(0);
    }
    __syncthreads();
    const int j = tid >> 3;      // right-hand side owned by this group of 8 lanes
    const int l8 = tid & 7;
    T *y = Ys + j * W;
    const unsigned gmask = 0xFFu << ((tid & 31) & ~7);
    for (int s = 0; s < w; ++s) {
        const int r = TRANS ? (w - 1 - s) : s;
        T acc = T(0);
        if (!TRANS) {
            for (int c = l8; c < r; c += 8) acc = fma(Ls[r * (W + 1) + c], y[c], acc);
        } else {
            for (int c = r + 1 + l8; c < w; c += 8) acc = fma(Ls[c * (W + 1) + r], y[c], acc);
        }
        acc += __shfl_xor_sync(gmask, acc, 1);
        acc += __shfl_xor_sync(gmask, acc, 2);
        acc += __shfl_xor_sync(gmask, acc, 4);
        if (l8 == 0) y[r] = (y[r] - acc) / Ls[r * (W + 1) + r];
        __syncwarp(gmask);
    }
    __syncthreads();
    for (int idx = tid; idx < 16 * w; idx += blockDim.x) {
        const int r = idx % w, jj = idx / w;
        if (col0 + jj < nrhs) B[(long)r + (long)(col0 + jj) * ldb] = Ys[jj * W + r];
    }
}

// ---------------------------------------------------------------------------
// Elementwise helpers.
// ---------------------------------------------------------------------------
template <typename TO, typename TI>
__global__ void convert_lower_kernel(int n, const TI *__restrict__ in, long ldi, TO *__restrict__ out, long ldo, int lower_only)
{
    const long j = blockIdx.y;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (lower_only && i < j) continue;
        out[i + j * ldo] = (TO)in[i + j * ldi];
    }
}

template <typename TO, typename TI>
__global__ void convert_rect_kernel(int m, int n, const TI *__restrict__ in, long ldi, TO *__restrict__ out, long ldo)
{
    const long j = blockIdx.y;
    if (j >= n) return;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x)
        out[i + j * ldo] = (TO)in[i + j * ldi];
}

template <typename T>
__global__ void zero_upper_kernel(int n, T *__restrict__ A, long lda)
{
    const long j = blockIdx.y;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < j && i < n; i += (long)gridDim.x * blockDim.x)
        A[i + j * lda] = T(0);
}

} // namespace gb300
