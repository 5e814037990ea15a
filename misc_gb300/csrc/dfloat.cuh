// Double-float arithmetic on the FP32 pipe (device code).
//
// GB300 executes FP64 instructions at about 1/64 of its FP32 rate, so the FP64 element kernels
// carry their bulk arithmetic as unevaluated sums x = hi + lo of two floats (about 48
// significant bits, relative error near 2^-47 per operation) and use FP64 only to deliver the
// final values.  The building blocks are the error-free transformations of Knuth (two-sum) and
// of the fused multiply-add (two-product); every step uses the explicitly rounded intrinsics so
// the compiler cannot contract or reassociate them.
#pragma once
#include <cuda_runtime.h>

struct DF {
    float hi, lo;
};

// a + b = s.hi + s.lo exactly
__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float v = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}
// the same when |a| >= |b| (or a == 0)
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const DF s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
// multiplication by a power of two (exact)
__device__ __forceinline__ DF df_scale2(DF a, float s) { return DF{__fmul_rn(a.hi, s), __fmul_rn(a.lo, s)}; }
// 1/a: single-precision reciprocal and one Newton step r + r (1 - a r)
__device__ __forceinline__ DF df_rcp(DF a) {
    const float r = __frcp_rn(a.hi);
    const DF e = df_sub(DF{1.f, 0.f}, df_mul(a, DF{r, 0.f}));
    return df_fast_two_sum(r, __fmul_rn(r, e.hi));
}
// s += a b with a, b given as (hi, lo) parts: error-free product of the high parts, first-order
// cross terms, and a two-sum into s (renormalised once at the end by df_norm)
__device__ __forceinline__ void df_acc(DF &s, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const DF t = df_two_sum(s.hi, p);
    s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, e));
    s.hi = t.hi;
}
__device__ __forceinline__ DF df_norm(DF a) { return df_fast_two_sum(a.hi, a.lo); }
__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }
__host__ __device__ __forceinline__ DF df_from_double(double x) {
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
}
