// Double-float arithmetic: a value is an unevaluated pair hi + lo of FP32
// numbers (|lo| <= ulp(hi) / 2), about 46-48 significant bits.  On GB300 the
// FP64 pipe issues a small fraction of the FP32 rate (a DFMA costs the pipe
// time of dozens of FMAs), so recurrences that need more than FP32 but far
// less than the full FP64 range run faster in pairs of FP32 operations.
//
// The error-free transforms are the classical ones (Knuth's two-sum,
// Dekker's fast two-sum, and the FMA two-product); the arithmetic below is
// the "sloppy" double-float addition and the FMA product of the
// double-double literature (e.g. Hida, Li and Bailey's QD library and Joldes,
// Muller and Popescu's analysis): relative error a few units of 2^-48 of the
// operands for a sum, of the result for a product.  Every FP32 operation is
// written with the _rn intrinsics so that the compiler cannot contract a
// product and a sum into one FMA, which would break the transforms.
#pragma once
#include <cuda_runtime.h>

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo) { return df{hi, lo}; }

// s + e = a + b exactly
__device__ __forceinline__ df df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df{s, e};
}

// s + e = a + b exactly when |a| >= |b| (or a = 0)
__device__ __forceinline__ df df_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df df_add(df a, df b)
{
    const df s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_mul(df a, df b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}

__device__ __forceinline__ df df_mul_f(df a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return df_fast_two_sum(p, e);
}

// a * b + c with one rounding of the pair's parts (the product's error term
// and both low parts are gathered before the final normalisation)
__device__ __forceinline__ df df_fma(df a, df b, df c)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const df s = df_two_sum(p, c.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

// 1 / a: the approximate FP32 reciprocal (rcp.approx, relative error below
// 2^-22) refined by one Newton step carried in pairs: r = 1 - a y is formed
// with FMAs (its rounding is second order), y' = y + y r; relative error
// about 2^-44 and below.  a is a normal FP32 number of either sign.
__device__ __forceinline__ df df_rcp(df a)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(a.hi));
    float r = fmaf(-a.hi, y, 1.0f);
    r = fmaf(-a.lo, y, r);
    return df_fast_two_sum(y, __fmul_rn(y, r));
}

// FP64 -> pair (FP64 instructions: for per-instance constants, not loops)
__device__ __forceinline__ df df_from_f64(double d)
{
    const float hi = __double2float_rn(d);
    return df{hi, __double2float_rn(d - (double)hi)};
}

struct cdf {
    df re, im;
};

__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return cdf{df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ cdf cdf_mul_f(cdf a, float b) { return cdf{df_mul_f(a.re, b), df_mul_f(a.im, b)}; }
