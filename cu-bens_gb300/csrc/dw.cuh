// Double-word ("double-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits. GB300's FP32 pipe issues 64 times more
// operations per clock than its FP64 pipe, so a band LDL^T whose accuracy
// needs more than FP32 (the 1.58M-equation DKT panel: an FP32 factor's error
// in the smooth modes exceeds one) runs several times faster in this form
// than in native FP64.
//
// The building blocks are the error-free transformations of Knuth (two-sum)
// and Dekker (two-product through a fused multiply-add), as collected in
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44 (2017). Every
// operation uses the _rn intrinsics so that the compiler neither contracts
// nor reorders the compensated sums.
#pragma once

#include <cuda_runtime.h>

namespace cb {

struct dw {
    float hi, lo;
};

// a + b = s + e exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a + b = s + e exactly when the exponent of a is at least that of b (Dekker)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dw dw_from_double(double x)
{
    const float h = __double2float_rn(x);
    return dw{h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double dw_to_double(dw a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dw dw_add(dw a, dw b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    dw r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ dw dw_neg(dw a) { return dw{-a.hi, -a.lo}; }

__device__ __forceinline__ dw dw_sub(dw a, dw b) { return dw_add(a, dw_neg(b)); }

// a * b: the exact product of the high parts (FMA) plus the cross terms
__device__ __forceinline__ dw dw_mul(dw a, dw b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    dw r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}

// 1 / d: the FP32 reciprocal refined by one Newton step in double-word form
__device__ __forceinline__ dw dw_recip(dw d)
{
    const float r = __frcp_rn(d.hi);
    // t = 1 - d r, formed with the exact product of the high parts
    float t = __fmaf_rn(-d.hi, r, 1.0f);
    t = __fmaf_rn(-d.lo, r, t);
    dw out;
    fast_two_sum(r, __fmul_rn(r, t), out.hi, out.lo);
    return out;
}

// Accumulator of a sum of products, renormalised once at the end: the high
// parts add by two-sum into (s, c), the rounding errors and cross terms into c.
struct dw_acc {
    float s, c;
};

__device__ __forceinline__ void acc_zero(dw_acc &a)
{
    a.s = 0.0f;
    a.c = 0.0f;
}

// a += x * y. Every operation is a fused multiply-add: a sum u + v is formed
// as fma(u, 1, v) and a difference u - v as fma(v, -1, u), which round
// exactly as the add does, so the products, Knuth's two-sum and the error
// terms all issue as FFMA.
__device__ __forceinline__ void acc_fma(dw_acc &a, dw x, dw y)
{
    const float p = __fmaf_rn(x.hi, y.hi, -0.0f);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    const float s = __fmaf_rn(a.s, 1.0f, p);
    const float bb = __fmaf_rn(a.s, -1.0f, s);   // s - a.s
    const float t1 = __fmaf_rn(bb, -1.0f, s);    // s - bb
    const float t2 = __fmaf_rn(t1, -1.0f, a.s);  // a.s - t1
    const float t3 = __fmaf_rn(bb, -1.0f, p);    // p - bb
    const float t = __fmaf_rn(t2, 1.0f, t3);
    a.s = s;
    a.c = __fmaf_rn(a.c, 1.0f, __fmaf_rn(t, 1.0f, e));
}

__device__ __forceinline__ dw acc_value(const dw_acc &a)
{
    dw r;
    fast_two_sum(a.s, a.c, r.hi, r.lo);
    return r;
}

}  // namespace cb
