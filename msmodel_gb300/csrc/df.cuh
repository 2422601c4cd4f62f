// df.cuh -- double-float arithmetic: a value is an unevaluated sum hi + lo of
// two FP32 numbers (about 48 significant bits), built from the error-free
// transformations of Knuth (two-sum) and Dekker (two-product via FMA), as in
// Hida, Li & Bailey, "Library for double-double and quad-double arithmetic"
// (2001), with FP32 limbs.  Every operation uses the _rn intrinsics so the
// compiler cannot contract or reassociate the compensation terms.
//
// The mixed-precision LU keeps its trailing matrix in this format: 16 bytes
// per complex entry (re.hi, re.lo, im.hi, im.lo), the FP32 pipe (64x the FP64
// rate on GB300) does the panel arithmetic, and the tensor cores do the
// trailing products.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace msg {

struct df {
    float h, l;
};

__device__ __forceinline__ df two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df{s, e};
}
__device__ __forceinline__ df quick_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.h, b.h);
    s.l = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
    return quick_two_sum(s.h, s.l);
}
__device__ __forceinline__ df df_neg(df a) { return df{-a.h, -a.l}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
    float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return quick_two_sum(p, e);
}
__device__ __forceinline__ df df_from_double(double x) {
    float h = __double2float_rn(x);
    float l = __double2float_rn(x - (double)h);
    return df{h, l};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.h + (double)a.l; }

// complex double-float, stored as float4 {re.hi, re.lo, im.hi, im.lo}
struct dfc {
    df re, im;
};
__device__ __forceinline__ dfc dfc_load(const float4* p) {
    float4 v = *p;
    return dfc{df{v.x, v.y}, df{v.z, v.w}};
}
__device__ __forceinline__ void dfc_store(float4* p, dfc a) { *p = make_float4(a.re.h, a.re.l, a.im.h, a.im.l); }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
    return dfc{df_sub(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
// c + x y + u v for double-floats, in one pass: the two leading products are
// exact by FMA (two-product), the sums of leading parts exact by two-sum, and
// every error and cross term gathers in one FP32 accumulator before a single
// renormalisation (about 27 FP32 operations against 36 for two double-float
// products and two double-float sums; the same ~2^-44 relative accuracy)
__device__ __forceinline__ df df_sum_prods(df c, df x, df y, df u, df v) {
    const float p1 = __fmul_rn(x.h, y.h), e1 = __fmaf_rn(x.h, y.h, -p1);
    const float p2 = __fmul_rn(u.h, v.h), e2 = __fmaf_rn(u.h, v.h, -p2);
    const df s = two_sum(c.h, p1);
    const df t = two_sum(s.h, p2);
    float lo = __fadd_rn(__fadd_rn(s.l, t.l), __fadd_rn(c.l, __fadd_rn(e1, e2)));
    lo = __fmaf_rn(x.h, y.l, lo);
    lo = __fmaf_rn(x.l, y.h, lo);
    lo = __fmaf_rn(u.h, v.l, lo);
    lo = __fmaf_rn(u.l, v.h, lo);
    return quick_two_sum(t.h, lo);
}

// c - a * b
__device__ __forceinline__ dfc dfc_fms(dfc c, dfc a, dfc b) {
    const df re = df_sum_prods(c.re, df_neg(a.re), b.re, a.im, b.im);
    const df im = df_sum_prods(c.im, df_neg(a.re), b.im, df_neg(a.im), b.re);
    return dfc{re, im};
}
__device__ __forceinline__ float dfc_abs1(dfc a) { return fabsf(a.re.h) + fabsf(a.im.h); }
__device__ __forceinline__ bool dfc_is_zero(dfc a) { return a.re.h == 0.0f && a.im.h == 0.0f; }

}  // namespace msg
