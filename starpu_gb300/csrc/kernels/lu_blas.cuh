// SIMT kernels of the tiled LU factorisation (examples/lu): the factor form
// of the reference codelets, A = L U with L lower non-unit and U unit upper
// (the CPU GETRF loop of examples/lu/xlu_kernels.c:369-380 keeps the pivot
// in L and scales the pivot row), and its threshold pivoting: a step whose
// pivot is smaller than the threshold in magnitude takes the largest entry of
// its row and swaps whole columns (xlu_kernels.c:516-545).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace gb300 {

// 1 / d rounded to T the way the reference forms its scale factor: in double,
// then converted (the BLAS SCAL takes a T alpha)
template <typename T> __device__ __forceinline__ T lu_recip(T d) { return (T)(1.0 / (double)d); }

// ---------------------------------------------------------------------------
// Unblocked LU of one n x n (n <= NMAX) diagonal block, held in registers:
// 256 threads as NMAX rows x CL column lanes, thread (ti, tc) keeps row ti,
// columns tc, tc + CL, ...  Step z: the owners of column z and of row z
// publish them through double-buffered shared vectors (one barrier per step);
// every thread scales its copy of row z by 1/a_zz and applies the rank-1
// update to its elements.  A zero pivot records info = info_base + z + 1
// (first wins, no trap).  thr > 0: the first step whose pivot has magnitude
// below thr is recorded (atomicMin of info_base + z into *d_first), for the
// caller's pivoting fallback.
// ---------------------------------------------------------------------------
template <typename T, int NMAX>
__global__ void __launch_bounds__(256) getf2_small_kernel(int n, T *__restrict__ A, long lda, T thr, int *d_first,
                                                          int *info, int info_base)
{
    constexpr int CL = 256 / NMAX, NC = NMAX / CL;
    __shared__ T col[2][NMAX], row[2][NMAX];
    const int tid = threadIdx.x;
    const int ti = tid % NMAX, tc = tid / NMAX;
    T a[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        const int c = tc + q * CL;
        a[q] = (ti < n && c < n) ? A[(long)ti + (long)c * lda] : T(0);
    }
    bool flagged = false;
#pragma unroll
    for (int z = 0; z < NMAX; ++z) {
        if (z >= n) break;
        T *cz = col[z & 1], *rz = row[z & 1];
        if (tc == z % CL) cz[ti] = a[z / CL];
        if (ti == z) {
#pragma unroll
            for (int q = 0; q < NC; ++q) rz[tc + q * CL] = a[q];
        }
        __syncthreads();
        const T d = cz[z];
        if (tid == 0) {
            if (d == T(0) && info) atomicCAS(info, 0, info_base + z + 1);
            if (thr > T(0) && !flagged && !(fabs((double)d) >= (double)thr) && d_first) {
                atomicMin(d_first, info_base + z);
                flagged = true;
            }
        }
        const T inv = lu_recip(d);
        if (ti == z) {
#pragma unroll
            for (int q = 0; q < NC; ++q)
                if (tc + q * CL > z) a[q] = a[q] * inv;
        } else if (ti > z) {
            const T l = cz[ti];
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const int c = tc + q * CL;
                if (c > z) a[q] = fma(-l, rz[c] * inv, a[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        const int c = tc + q * CL;
        if (ti < n && c < n) A[(long)ti + (long)c * lda] = a[q];
    }
}

// ---------------------------------------------------------------------------
// B[m x w] <- B * U^{-1}, U w x w unit upper (w <= W): the right-side TRSM of
// the LU's block column (cublasStrsm(R, U, N, U), xlu_kernels.c:281-289).
// One thread per row of B, column-oriented like reference BLAS strsm.
// FULL (w == W) keeps every index static, which keeps x[] in registers.
// ---------------------------------------------------------------------------
template <typename T, int W, bool FULL>
__global__ void __launch_bounds__(128) trsm_runu_small_kernel(int m, int w, const T *__restrict__ U, long ldu,
                                                              T *__restrict__ B, long ldb)
{
    __shared__ T Us[W][W + 1];
    const int tid = threadIdx.x;
    const int ww = FULL ? W : w;
    for (int idx = tid; idx < W * W; idx += blockDim.x) {
        const int i = idx % W, j = idx / W;
        Us[i][j] = (i < ww && j < ww && i < j) ? U[(long)i + (long)j * ldu] : T(0);
    }
    __syncthreads();
    const long r = (long)blockIdx.x * blockDim.x + tid;
    if (r >= m) return;
    T x[W];
#pragma unroll
    for (int c = 0; c < W; ++c) x[c] = (FULL || c < ww) ? B[r + (long)c * ldb] : T(0);
#pragma unroll
    for (int j = 0; j < W; ++j) {
#pragma unroll
        for (int c = j + 1; c < W; ++c) x[c] = fma(-Us[j][c], x[j], x[c]);
    }
#pragma unroll
    for (int c = 0; c < W; ++c)
        if (FULL || c < ww) B[r + (long)c * ldb] = x[c];
}

// ---------------------------------------------------------------------------
// Exact unblocked threshold-pivoting LU of one n x n tile in global memory
// (the reference GETRF_PIVOT loop, xlu_kernels.c:516-545, with the pivot
// index of its CUDA branch), run by one CTA of 1024 threads.  It does
// nothing unless *d_first < n: the blocked factorisation that ran first met a
// pivot below the threshold, so the tile was restored from its copy and is
// factored again here with pivoting.  ipiv[z] = the column swapped with z at
// step z (z itself when the step pivoted in place), -1 when it did not pivot.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(1024) getrf_pivot_unblocked_kernel(int n, T *__restrict__ A, long lda, T thr,
                                                                     const int *d_first, int *ipiv, int *info)
{
    if (*d_first >= n) return;
    __shared__ double sval[32];
    __shared__ int sidx[32];
    __shared__ int s_p;
    __shared__ T s_piv;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int z = 0; z < n; ++z) {
        T *az = A + (long)z * lda;  // column z
        if (tid == 0) s_piv = az[z];
        __syncthreads();
        if (!(fabs((double)s_piv) >= (double)thr)) {
            // largest |a_zj|, j >= z (row z), first index on ties
            double best = -1.0;
            int bi = n;
            for (int j = z + tid; j < n; j += nt) {
                const double v = fabs((double)A[(long)z + (long)j * lda]);
                if (v > best) best = v, bi = j;
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_down_sync(0xffffffffu, best, o);
                const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) best = ov, bi = oi;
            }
            if ((tid & 31) == 0) sval[tid >> 5] = best, sidx[tid >> 5] = bi;
            __syncthreads();
            if (tid == 0) {
                double b = sval[0];
                int p = sidx[0];
                for (int w = 1; w < nt / 32; ++w)
                    if (sval[w] > b || (sval[w] == b && sidx[w] < p)) b = sval[w], p = sidx[w];
                s_p = p < n ? p : z;
                ipiv[z] = s_p;
            }
            __syncthreads();
            const int p = s_p;
            if (p != z) {
                T *ap = A + (long)p * lda;
                for (int i = tid; i < n; i += nt) {
                    const T t = az[i];
                    az[i] = ap[i];
                    ap[i] = t;
                }
            }
            __syncthreads();
            if (tid == 0) s_piv = az[z];
        } else if (tid == 0) {
            ipiv[z] = -1;
        }
        __syncthreads();
        const T d = s_piv;
        if (tid == 0 && d == T(0) && info) atomicCAS(info, 0, z + 1);
        const T inv = lu_recip(d);
        for (int j = z + 1 + tid; j < n; j += nt) A[(long)z + (long)j * lda] *= inv;
        __syncthreads();
        // rank-1 update of the trailing block: a_ij -= a_iz * a_zj
        const int m = n - z - 1;
        for (long e = tid; e < (long)m * m; e += nt) {
            const int i = z + 1 + (int)(e % m), j = z + 1 + (int)(e / m);
            A[(long)i + (long)j * lda] = fma(-az[i], A[(long)z + (long)j * lda], A[(long)i + (long)j * lda]);
        }
        __syncthreads();
    }
}

// When a step of the blocked factorisation needed a pivot (*d_first < n):
// put the tile back from its copy (ld n) and clear the status word, so the
// pivoting factorisation starts from the input.
template <typename T>
__global__ void restore_if_flagged_kernel(int n, const T *__restrict__ copy, T *__restrict__ A, long lda,
                                          const int *d_first, int *info)
{
    if (*d_first >= n) return;
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 0 && info) *info = 0;
    if (e < (long)n * n) A[(e % n) + (e / n) * lda] = copy[e];
}

__global__ void lu_set_int_kernel(int *p, int v) { *p = v; }

// ---------------------------------------------------------------------------
// Column swaps of one tile in the order given (the reference PIVOT codelet,
// xlu_kernels.c:686-693): swap columns pairs[s].x and pairs[s].y for s = 0,
// 1, ...  One thread per row applies the whole sequence to its row.
// ---------------------------------------------------------------------------
constexpr int LU_SWAP_MAX = 1024;
struct LuSwapList {
    int count;
    int2 pairs[LU_SWAP_MAX];
};

template <typename T>
__global__ void __launch_bounds__(256) swap_columns_kernel(int m, T *__restrict__ A, long lda, const LuSwapList list)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int s = 0; s < list.count; ++s) {
        const int2 p = list.pairs[s];
        T *x = A + i + (long)p.x * lda, *y = A + i + (long)p.y * lda;
        const T t = *x;
        *x = *y;
        *y = t;
    }
}

} // namespace gb300
