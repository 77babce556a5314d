// Double-float building blocks of the residuals on the FP32 pipe: the
// power-of-two scale of a column, the split of a scaled FP64 value into two
// FP32 parts by bit operations, and the error-free multiply-accumulate of
// two such pairs into a running (high, low) sum.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace gb300 {

// exponent e with v * 2^-e in [1, 2) (0 for v == 0 or non-finite v)
__device__ __forceinline__ int df_scale_exp(double v)
{
    if (!(v > 0.0) || !isfinite(v)) return 0;
    return ilogb(v);
}

// a * 2^-ea as (hi, lo) FP32, by bit manipulation.  Requires |a| * 2^-ea < 2
// (ea from an upper bound of |a|); non-finite a gives a non-finite hi.
__device__ __forceinline__ float2 df_split_scaled(double a, int ea)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(a);
    const int e = (int)((u >> 52) & 0x7FF);
    const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
    if (e == 0x7FF) return make_float2(__int_as_float((int)(sign | 0x7FC00000u)), 0.0f);
    const int fe = e - 1023 - ea + 127;  // biased FP32 exponent of a * 2^-ea
    if (e == 0 || fe <= 0) return make_float2(0.0f, 0.0f);
    if (fe >= 255) return make_float2(__int_as_float((int)(sign | 0x7F800000u)), 0.0f);
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    const float hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)(m >> 29));
    float lo = 0.0f;
    if (fe >= 53) {
        // the 29 dropped bits, weight 2^(fe - 127 - 52), rounded to 24 bits
        const float r = __uint2float_rn((unsigned)(m & 0x1FFFFFFFu));
        lo = __uint_as_float(sign | __float_as_uint(__fmul_rn(r, __uint_as_float((unsigned)(fe - 52) << 23))));
    }
    return make_float2(hi, lo);
}

// (sh, sl) += (ah + al) * (xh + xl); intrinsics keep the compiler from
// contracting the error-free transformations into FMAs
__device__ __forceinline__ void df_mac(float &sh, float &sl, float ah, float al, float xh, float xl)
{
    const float p = __fmul_rn(ah, xh);
    float e = __fmaf_rn(ah, xh, -p);
    e = __fmaf_rn(ah, xl, e);
    e = __fmaf_rn(al, xh, e);
    const float t = __fadd_rn(sh, p);
    const float z = __fsub_rn(t, sh);
    const float d = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
    sl = __fadd_rn(sl, __fadd_rn(d, e));
    sh = t;
}

} // namespace gb300
