// green_df.cuh -- the d = 3 Foldy-Lax matrix elements for the mixed engine,
// with the transcendental work moved from the FP64 pipe (about 2 lanes per
// SM per clock on GB300) to the FP32 pipe (128 lanes) in double-float
// arithmetic.
//
//   M_ij  = -G = e^{ikr} / (4 pi r) = e^{-r Im k} (cos r Re k + i sin r Re k) / (4 pi r)
//   dM_ij = i e^{ikr} / (4 pi)
//
// FP64 computes only r, the arguments and their Cody-Waite reductions
// (3-part pi/2 and 2-part ln 2 splits in the style of fdlibm, so q * part is
// exact for |q| < 2^20); the reduced arguments (|y| <= pi/4, |t| <= ln2/2)
// go to double-float Taylor polynomials evaluated by Horner's rule:
//   sin y = y sum_{k=0}^{8} (-1)^k y^2k / (2k+1)!     (next term < 1e-19)
//   cos y = sum_{k=0}^{8} (-1)^k y^2k / (2k)!           (next term < 1e-17)
//   e^t   = sum_{k=0}^{13} t^k / k!                     (next term < 1e-17)
// Each step costs one double-float multiply and add (~2^-47 relative); the
// elements come out within a few 1e-15 of the FP64 evaluation, far inside the
// mixed path's accuracy budget (checked against CUDA's FP64 sincos/exp by
// tests/test_gpu_mixed.py through the resulting ln det).
#pragma once
#include "df.cuh"
#include "cplx.cuh"

namespace msg {

// 1/n! as double-float pairs, n = 0..18
__constant__ float c_invfact[19][2] = {
    {1.0f, 0.0f},
    {1.0f, 0.0f},
    {0.5f, 0.0f},
    {0.1666666716337204f, -4.967053879312289e-09f},
    {0.0416666679084301f, -1.2417634698280722e-09f},
    {0.008333333767950535f, -4.34617203337595e-10f},
    {0.0013888889225199819f, -3.3631094437103215e-11f},
    {0.00019841270113829523f, -2.725596874933456e-12f},
    {2.4801587642286904e-05f, -3.40699609366682e-13f},
    {2.7557318844628753e-06f, 3.793571224297229e-14f},
    {2.755731998149713e-07f, -7.575112209051195e-15f},
    {2.5052107943679403e-08f, 4.4176230446483665e-16f},
    {2.0876755879584152e-09f, 1.1082839147459852e-16f},
    {1.6059044372074283e-10f, -5.352526511562726e-18f},
    {1.147074536050896e-11f, 2.372207689231238e-19f},
    {7.647163609812713e-13f, 1.2200710471178288e-20f},
    {4.7794772561329454e-14f, 7.62544404448643e-22f},
    {2.8114573589663704e-15f, -1.0462084739763658e-22f},
    {1.5619206814541513e-16f, 1.5404471465941993e-24f},
};

__device__ __forceinline__ df invfact(int n) { return df{c_invfact[n][0], c_invfact[n][1]}; }

// sin and cos of the double-float y, |y| <= pi/4
__device__ __forceinline__ void df_sincos_small(df y, df& s, df& c) {
    const df u = df_mul(y, y);
    df ps = invfact(17), pc = invfact(16);
#pragma unroll
    for (int k = 7; k >= 0; --k) {
        const df cs = invfact(2 * k + 1), cc = invfact(2 * k);
        ps = df_add(df_mul(ps, df_neg(u)), cs);
        pc = df_add(df_mul(pc, df_neg(u)), cc);
    }
    s = df_mul(ps, y);
    c = pc;
}

// e^t for the double-float t, |t| <= ln2/2
__device__ __forceinline__ df df_exp_small(df t) {
    df p = invfact(13);
#pragma unroll
    for (int k = 12; k >= 0; --k) p = df_add(df_mul(p, t), invfact(k));
    return p;
}

// elements of M (and dM/dk if want_deriv) for one pair at distance r, as double-floats
__device__ __forceinline__ void pair_elements_df3(zc k, double r, bool want_deriv, dfc& m, dfc& dm) {
    // phase and its reduction modulo pi/2
    const double PIO2_1 = 1.57079632673412561417e+00, PIO2_2 = 6.07710050630396597660e-11,
                 PIO2_3 = 2.02226624879595063154e-21, TWO_OVER_PI = 6.36619772367581382433e-01;
    const double phi = k.re * r;
    const double qd = rint(phi * TWO_OVER_PI);
    const double yd = ((phi - qd * PIO2_1) - qd * PIO2_2) - qd * PIO2_3;
    const int quad = ((int)qd) & 3;
    // growth exponent and its reduction modulo ln 2
    const double LN2_HI = 6.93147180369123816490e-01, LN2_LO = 1.90821492927058770002e-10,
                 LOG2E = 1.44269504088896338700e+00;
    const double x = -k.im * r;
    const double nd = rint(x * LOG2E);
    const double td = (x - nd * LN2_HI) - nd * LN2_LO;
    df s, c;
    df_sincos_small(df_from_double(yd), s, c);
    // rotate by the quadrant: (sin, cos)(y + q pi/2)
    df sn, cs;
    switch (quad) {
    case 0: sn = s; cs = c; break;
    case 1: sn = c; cs = df_neg(s); break;
    case 2: sn = df_neg(s); cs = df_neg(c); break;
    default: sn = df_neg(c); cs = s; break;
    }
    df e = df_exp_small(df_from_double(td));
    const int ni = (int)nd;
    e.h = ldexpf(e.h, ni);
    e.l = ldexpf(e.l, ni);
    const df w = df_mul(e, df_from_double(1.0 / (12.566370614359172954 * r)));
    m = dfc{df_mul(w, cs), df_mul(w, sn)};
    if (want_deriv) {
        // dM = i e^{ikr} / (4 pi)
        const df w2 = df_mul(e, df_from_double(1.0 / 12.566370614359172954));
        dm = dfc{df_neg(df_mul(w2, sn)), df_mul(w2, cs)};
    }
}

// ---------------------------------------------------------------------------
// All-FP32-pipe form of the d = 3 Green function, for the wavefunction grid
// (pixels x atoms evaluations), where FP64 sqrt, division and reductions per
// pair would keep the FP64 pipe the bound.  Only the coordinates are
// converted from FP64, once per tile.
//
//   r      double-float sqrt: FP32 root plus one Newton correction
//   phase  phi = Re k * r reduced modulo pi/16 (three-float split of pi/16,
//          each product q * part exact by FMA), |y| <= pi/32; sin/cos of
//          j pi/16 from a 32-entry table, sin/cos of y by Taylor series
//          (next terms < 4e-17), combined by the addition theorem
//   growth e^{-Im k * r} reduced modulo ln2/16, 2^{j/16} from a 16-entry
//          table, e^t by Taylor series (|t| <= ln2/32, next term < 2e-18)
// Relative accuracy about 2^-44 per element (|phi| * 2^-47 absolute in the
// phase); values are FP32-range limited, so callers keep |Im k| r below 80.

__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return df{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df df_sqrt(df a) {
    if (!(a.h > 0.0f)) return df{0.0f, 0.0f};
    const float s = __fsqrt_rn(a.h);
    const df p = two_prod(s, s);
    const float e = __fadd_rn(__fsub_rn(__fsub_rn(a.h, p.h), p.l), a.l);
    return quick_two_sum(s, __fmul_rn(e, __fmul_rn(0.5f, __frcp_rn(s))));
}

__device__ __forceinline__ df df_recip(df b) {
    const float q1 = __frcp_rn(b.h);
    float r = __fmaf_rn(-b.h, q1, 1.0f);
    r = __fmaf_rn(-b.l, q1, r);
    return quick_two_sum(q1, __fmul_rn(r, q1));
}

struct Df3Tables {
    float4 sc[32];  // {sin.h, sin.l, cos.h, cos.l} of j pi/16
    float2 p2[16];  // 2^{j/16}
};

// fill by threads 0..31 of the block (FP64 sincospi / exp2 of exact arguments)
__device__ __forceinline__ void df3_tables_init(Df3Tables& t) {
    const int j = threadIdx.x;
    if (j < 32) {
        double s, c;
        sincospi(j / 16.0, &s, &c);
        const df ds = df_from_double(s), dc = df_from_double(c);
        t.sc[j] = make_float4(ds.h, ds.l, dc.h, dc.l);
    }
    if (j < 16) {
        const df p = df_from_double(exp2(j / 16.0));
        t.p2[j] = make_float2(p.h, p.l);
    }
}

// e^{i phi} for phi = kr * r
__device__ __forceinline__ void df_cis(const Df3Tables& t, df phi, df& cs, df& sn) {
    const float q = rintf(__fmul_rn(phi.h, 5.0929582f));  // 16 / pi
    df y = df_sub(phi, two_prod(q, 0.19634955f));
    y = df_sub(y, two_prod(q, -5.4639235e-09f));
    y = quick_two_sum(y.h, __fmaf_rn(-q, -2.1439056e-16f, y.l));
    const df nu = df_neg(df_mul(y, y));
    df ps = df{2.7557319e-06f, 0.0f}, pc = df{2.4801588e-05f, 0.0f};  // 1/9!, 1/8!
#pragma unroll
    for (int k = 3; k >= 0; --k) {
        ps = df_add(df_mul(ps, nu), invfact(2 * k + 1));
        pc = df_add(df_mul(pc, nu), invfact(2 * k));
    }
    const df s = df_mul(ps, y), c = pc;
    const float4 e = t.sc[((int)q) & 31];
    const df S{e.x, e.y}, C{e.z, e.w};
    sn = df_add(df_mul(S, c), df_mul(C, s));
    cs = df_sub(df_mul(C, c), df_mul(S, s));
}

// e^{x}, |x| < 80
__device__ __forceinline__ df df_exp_tab(const Df3Tables& t, df x) {
    const float q = rintf(__fmul_rn(x.h, 23.08312f));  // 16 / ln 2
    df y = df_sub(x, two_prod(q, 0.0433217f));
    y = df_sub(y, two_prod(q, -1.1904089e-10f));
    y = quick_two_sum(y.h, __fmaf_rn(-q, -5.48949e-18f, y.l));
    df p = invfact(7);
#pragma unroll
    for (int k = 6; k >= 0; --k) p = df_add(df_mul(p, y), invfact(k));
    const int qi = (int)q;
    const float2 m = t.p2[qi & 15];
    p = df_mul(p, df{m.x, m.y});
    const int sh = qi >> 4;  // floor(q / 16)
    return df{ldexpf(p.h, sh), ldexpf(p.l, sh)};
}

// M_ij = e^{ikr} / (4 pi r) and dM_ij = i e^{ikr} / (4 pi) of d = 3 from a
// double-float r, entirely on the FP32 pipe (grow: Im k != 0)
__device__ __forceinline__ void pair_elements_df3t(const Df3Tables& t, df kr, df ki, bool grow, df r,
                                                   bool want_deriv, dfc& m, dfc& dm) {
    df cs, sn;
    df_cis(t, df_mul(kr, r), cs, sn);
    const df e = grow ? df_exp_tab(t, df_neg(df_mul(ki, r))) : df{1.0f, 0.0f};
    const df fourpi{12.566371f, -3.496911e-07f};
    const df w = df_mul(e, df_recip(df_mul(fourpi, r)));
    m = dfc{df_mul(w, cs), df_mul(w, sn)};
    if (want_deriv) {
        const df w2 = df_mul(e, df{0.07957747f, 3.2103191e-09f});  // 1 / (4 pi)
        dm = dfc{df_neg(df_mul(w2, sn)), df_mul(w2, cs)};
    }
}

// a * G(k, r) of d = 3, G = -e^{ikr} / (4 pi r), accumulated into acc
__device__ __forceinline__ void df3_green_mac(const Df3Tables& t, df kr, df ki, bool grow, df r, dfc a, dfc& acc) {
    df cs, sn;
    df_cis(t, df_mul(kr, r), cs, sn);
    const df fourpi{12.566371f, -3.496911e-07f};
    df w = df_recip(df_mul(fourpi, r));
    if (grow) w = df_mul(w, df_exp_tab(t, df_neg(df_mul(ki, r))));
    // acc -= w * a * (cs + i sn)
    const df vr = df_sub(df_mul(a.re, cs), df_mul(a.im, sn));
    const df vi = df_add(df_mul(a.re, sn), df_mul(a.im, cs));
    acc.re = df_sub(acc.re, df_mul(w, vr));
    acc.im = df_sub(acc.im, df_mul(w, vi));
}

}  // namespace msg
