// Double-float ("float-float") arithmetic for FP32-mode phase generation.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the FP32 path
// evaluates the large SAR phase arguments (1e4-1e5 rad, needing ~1e-9
// relative accuracy) as unevaluated sums hi + lo of two floats (~48-bit
// significand).  The operations are the classic error-free transformations:
// Knuth's TwoSum, TwoProd via a fused multiply-add, and Newton-corrected
// division / square root (Dekker 1971; Hida, Li & Bailey's double-double
// algorithms restated for float pairs).
#pragma once

#include <cuda_runtime.h>

namespace s1g {

struct df {
    float hi, lo;
};

__host__ __device__ __forceinline__ df df_make(float h, float l) {
    df r;
    r.hi = h;
    r.lo = l;
    return r;
}

// Split an FP64 value into a float pair (host-side table preparation, or a
// single FP64 op on the device per row / column).
__host__ __device__ __forceinline__ df df_from(double x) {
    const float h = (float)x;
    return df_make(h, (float)(x - (double)h));
}

__host__ __device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

#ifdef __CUDACC__
__device__ __forceinline__ df quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return df_make(s, e);
}

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df_make(s, e);
}

__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return df_make(p, e);
}

__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_neg(df a) { return df_make(-a.hi, -a.lo); }

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_add_f(df a, float b) {
    df s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_mul(df a, df b) {
    df p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return quick_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ df df_mul_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return quick_two_sum(p.hi, p.lo);
}

// Hardware reciprocal (rcp.approx, relative error ~2^-23): the quotient
// digits below are corrected by exact remainders, so their rounding does not
// reach the result.
__device__ __forceinline__ float df_rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// a / b by long division: three float quotient digits, each from the exact
// remainder of the previous ones (relative error ~2^-48).
__device__ __forceinline__ df df_div(df a, df b) {
    const float rb = df_rcp_approx(b.hi);
    const float q1 = a.hi * rb;
    df r = df_sub(a, df_mul_f(b, q1));
    const float q2 = r.hi * rb;
    r = df_sub(r, df_mul_f(b, q2));
    const float q3 = r.hi * rb;
    df q = quick_two_sum(q1, q2);
    return df_add_f(q, q3);
}
// sqrt(a): the correctly rounded float root, then one Newton step
// s + (a - s^2) / (2 s) with the exact residual (relative error ~2^-47).
__device__ __forceinline__ df df_sqrt(df a) {
    if (a.hi <= 0.0f) return df_make(0.0f, 0.0f);
    const float s = __fsqrt_rn(a.hi);
    const df s2 = two_prod(s, s);
    const df r = df_sub(a, s2);
    const float corr = r.hi * (0.5f * df_rcp_approx(s));
    return quick_two_sum(s, corr);
}
// 2*pi as a float pair and its reciprocal.
__device__ __forceinline__ df df_two_pi() { return df_make(6.28318548202514648f, -1.74845553e-7f); }

// Reduce a phase (|x| up to ~1e6 rad) to a float in about [-pi, pi].
__device__ __forceinline__ float df_wrap(df x) {
    const float k = rintf(x.hi * 0.159154943091895336f);
    const df tp = df_two_pi();
    df r = df_sub(x, df_add(two_prod(k, tp.hi), df_make(0.0f, k * tp.lo)));
    return r.hi + r.lo;
}
#endif

}  // namespace s1g
