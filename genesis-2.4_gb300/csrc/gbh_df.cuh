// gbh_df.cuh -- double-float arithmetic on FP32 instructions, and exact
// float <-> double conversions on the integer pipe.
//
// A df value is an unevaluated sum hi + lo of two floats with |lo| <=
// ulp(hi)/2, carrying about 48 significand bits. The primitives are the
// error-free transformations of Dekker (1971) and Knuth (TAOCP vol. 2,
// 4.2.2): TwoSum, FastTwoSum and TwoProd via fused multiply-add, composed as
// in the double-double literature (Hida, Li, Bailey 2001, "sloppy" add).
//
// On GB300 the FP64 pipe runs about 1.6 DFMA per SM per clock while FP32 runs
// ~113 FFMA, and the F2F conversions between float and double cost as much
// as two DFMAs, so the mixed-precision step keeps gate and table arithmetic
// in df and converts with integer bit manipulation instead of F2F.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbh {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_make(float h, float l) { df r; r.hi = h; r.lo = l; return r; }

__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return df_make(s, e);
}

__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = a + b;
    return df_make(s, b - (s - a));
}

__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = a * b;
    return df_make(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ df df_add(df x, df y)
{
    df s = two_sum(x.hi, y.hi);
    s.lo += x.lo + y.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_add_f(df x, float y)
{
    df s = two_sum(x.hi, y);
    s.lo += x.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_neg(df x) { return df_make(-x.hi, -x.lo); }

__device__ __forceinline__ df df_mul(df x, df y)
{
    df p = two_prod(x.hi, y.hi);
    p.lo = __fmaf_rn(x.hi, y.lo, p.lo);
    p.lo = __fmaf_rn(x.lo, y.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ df df_mul_f(df x, float y)
{
    df p = two_prod(x.hi, y);
    p.lo = __fmaf_rn(x.lo, y, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// x / y: one float quotient, its df remainder, one correction
__device__ __forceinline__ df df_div(df x, df y)
{
    const float r = rcp_approx(y.hi);
    const float q1 = x.hi * r;
    df p = two_prod(q1, y.hi);
    p.lo = __fmaf_rn(q1, y.lo, p.lo);
    const float rem = ((x.hi - p.hi) - p.lo) + x.lo;
    const float q2 = rem * r;
    return fast_two_sum(q1, q2);
}

// ---- exact conversions on the integer pipe --------------------------------
// float -> double (normal floats and zero; denormals flush to signed zero)
__device__ __forceinline__ double f2d_bits(float f)
{
    const uint32_t u = __float_as_uint(f);
    const uint32_t sign = u & 0x80000000u;
    const uint32_t e = (u >> 23) & 0xffu;
    const uint32_t m = u & 0x7fffffu;
    const uint32_t hi = (e == 0u) ? sign : (sign | ((e + 896u) << 20) | (m >> 3));
    const uint32_t lo = (e == 0u) ? 0u : (m << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// double -> float truncated toward zero (exact when the double already has at
// most 24 significant bits; values below the float normal range flush to 0)
__device__ __forceinline__ float d2f_trunc_bits(double d)
{
    const uint32_t hi = (uint32_t)__double2hiint(d);
    const uint32_t lo = (uint32_t)__double2loint(d);
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t bits = (e <= 0) ? sign : (e >= 255 ? (sign | 0x7f800000u) : (sign | ((uint32_t)e << 23) | m));
    return __uint_as_float(bits);
}

// double -> df on the integer pipe: hi = d truncated to 24 significant bits,
// lo = the next 24 bits of the significand, truncated (|d - hi - lo| <
// 2^-47 |d|); no FP64 instruction. Values whose hi or lo falls outside the
// float normal range lose that part (flush to signed zero).
__device__ __forceinline__ df d2df(double d)
{
    const uint32_t h = (uint32_t)__double2hiint(d);
    const uint32_t l = (uint32_t)__double2loint(d);
    const float fh = d2f_trunc_bits(d);
    const uint32_t r = l & 0x1fffffffu;
    const int e = (int)((h >> 20) & 0x7ffu);
    const int p = 31 - __clz((int)r);
    const int fe = p + e - 948;
    uint32_t lo = 0u;
    if (r != 0u && fe > 0 && e - 896 > 0 && e - 896 < 255) {
        const uint32_t m = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
        lo = (h & 0x80000000u) | ((uint32_t)fe << 23) | (m & 0x7fffffu);
    }
    return df_make(fh, __uint_as_float(lo));
}

// df -> double: exact conversions, one FP64 add
__device__ __forceinline__ double df2d(df x) { return f2d_bits(x.hi) + f2d_bits(x.lo); }

// reciprocal of a normal double to ~46 bits: the mantissa m in [1,2) gets a
// float seed (MUFU), the seed is rescaled by the exponent on the integer
// pipe, then one Newton step in FP64 (two DFMA). Valid for any finite d with
// 2^-1021 < |d| < 2^1021.
__device__ __forceinline__ double rcp_newton(double d)
{
    const int hi = __double2hiint(d), lo = __double2loint(d);
    const int e = (hi >> 20) & 0x7ff;
    const double m = __hiloint2double((hi & 0x800fffff) | 0x3ff00000, lo);
    const double s = f2d_bits(rcp_approx(d2f_trunc_bits(m)));
    const double r = __hiloint2double(__double2hiint(s) + ((1023 - e) << 20), __double2loint(s));
    const double err = fma(-d, r, 1.0);
    return fma(r, err, r);
}


}  // namespace gbh
