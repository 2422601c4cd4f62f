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
// c - a * b
__device__ __forceinline__ dfc dfc_fms(dfc c, dfc a, dfc b) {
    df re = df_sub(df_sub(c.re, df_mul(a.re, b.re)), df_neg(df_mul(a.im, b.im)));
    df im = df_sub(df_sub(c.im, df_mul(a.re, b.im)), df_mul(a.im, b.re));
    return dfc{re, im};
}
__device__ __forceinline__ float dfc_abs1(dfc a) { return fabsf(a.re.h) + fabsf(a.im.h); }
__device__ __forceinline__ bool dfc_is_zero(dfc a) { return a.re.h == 0.0f && a.im.h == 0.0f; }

}  // namespace msg
