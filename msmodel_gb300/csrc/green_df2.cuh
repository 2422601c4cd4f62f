// green_df2.cuh -- the d = 2 Foldy-Lax matrix elements for the mixed engine in
// double-float arithmetic on the FP32 pipe (64x the FP64 rate on GB300):
//
//   M_ij  = -G_2 = K_0(z) / (2 pi),   z = -i k r
//   dM_ij = -dG_2/dk = i r K_1(z) / (2 pi)     (d/dk K_0(-ikr) = i r K_1(z))
//
// K_nu (nu = 0, 1) by the three regimes of the FP64 engine (green.cuh), chosen
// where the reference switches (green_bessel.c:208-218):
//   |z| > 16                     asymptotic series (DLMF 10.40.2), truncated at
//                                index |2z| or once |term|^2 < 1e-32;
//   Re z < 3 - (Im z)^2 / 12     ascending series (DLMF 10.31.1);
//   otherwise                    Temme's Miller scheme from his index estimate.
// The factors that depend on k alone -- sqrt(pi/2) (-ik)^(-1/2), 1/(-ik),
// ln(-ik/2) -- are formed once per matrix in FP64; per pair the FP32 pipe
// computes r (double-float square root of the double-float coordinates),
// e^{-z} = e^{-r Im k} e^{i r Re k} by the table-driven routines of
// green_df.cuh, and the loops.  Only the ascending series, a few per cent of
// the pairs (|k| r below ~6), takes ln r in FP64.
#pragma once
#include "df.cuh"
#include "cplx.cuh"
#include "green.cuh"
#include "green_df.cuh"

namespace msg {

// ------------------------------------------------------------ complex double-float helpers
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return dfc{df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return dfc{df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_scale(dfc a, df s) { return dfc{df_mul(a.re, s), df_mul(a.im, s)}; }
__device__ __forceinline__ dfc dfc_from(zc v) { return dfc{df_from_double(v.re), df_from_double(v.im)}; }
__device__ __forceinline__ float dfc_norm2f(dfc a) { return a.re.h * a.re.h + a.im.h * a.im.h; }
// 1 / b = conj(b) / |b|^2
__device__ __forceinline__ dfc dfc_recip(dfc b) {
    const df n = df_add(df_mul(b.re, b.re), df_mul(b.im, b.im));
    const df rn = df_recip(n);
    return dfc{df_mul(b.re, rn), df_neg(df_mul(b.im, rn))};
}

// ------------------------------------------------------------ coefficient tables as double-floats
struct BkTablesDf {
    float2 asym[2][BK_TAB];
    float2 ser_t[2][BK_TAB];
    float2 ser_c[2][BK_TAB];
    float2 miller[2][BK_TAB];
};
constexpr float2 split_df(double x) {
    const float h = (float)x;
    return float2{h, (float)(x - (double)h)};
}
constexpr BkTablesDf make_bk_tables_df() {
    const BkTables t = make_bk_tables();
    BkTablesDf o{};
    for (int nu = 0; nu < 2; ++nu)
        for (int k = 0; k < BK_TAB; ++k) {
            o.asym[nu][k] = split_df(t.asym[nu][k]);
            o.ser_t[nu][k] = split_df(t.ser_t[nu][k]);
            o.ser_c[nu][k] = split_df(t.ser_c[nu][k]);
            o.miller[nu][k] = split_df(t.miller[nu][k]);
        }
    return o;
}
__constant__ BkTablesDf c_bkdf = make_bk_tables_df();
__device__ __forceinline__ df tab_df(float2 v) { return df{v.x, v.y}; }

// ------------------------------------------------------------ per-matrix constants
struct Df2Item {
    df kr, ki;      // Re k, Im k
    dfc mik;        // -i k
    dfc pref;       // sqrt(pi/2) (-ik)^(-1/2)
    dfc rik;        // 1 / (-ik)
    dfc lnh;        // ln(-ik / 2)
    float kabs;     // |k|
    int grow;       // Im k != 0
};

__device__ __forceinline__ Df2Item df2_item(zc k) {
    Df2Item P;
    P.kr = df_from_double(k.re);
    P.ki = df_from_double(k.im);
    const zc mik = mk(k.im, -k.re);
    P.mik = dfc_from(mik);
    P.pref = dfc_from(sqrt(0.5 * PI) / zsqrt(mik));
    P.rik = dfc_from(zrecip(mik));
    P.lnh = dfc_from(zlog(0.5 * mik));
    P.kabs = (float)zabs(k);
    P.grow = k.im != 0.0;
    return P;
}

// K_nu regime of z = -ikr from the double-float r (0 asymptotic, 1 series, 2 Miller)
__device__ __forceinline__ int k_regime_df(const Df2Item& P, df r) {
    const float x = P.ki.h * r.h, y = -P.kr.h * r.h;
    if (x * x + y * y > 256.0f) return 0;
    if (x < 3.0f - y * y / 12.0f) return 1;
    return 2;
}

// B_nu(z) = K_nu(z) / (sqrt(pi/2z) e^-z) by the asymptotic series, for nu = 0 and
// (if both) nu = 1 in one pass over the powers of 1/(8z)
__device__ __forceinline__ void bk_asym_df(dfc iz8, int kmax, bool both, dfc& b0, dfc& b1) {
    dfc t0{df{1.0f, 0.0f}, df{0.0f, 0.0f}}, t1 = t0;
    b0 = t0;
    b1 = t0;
    bool on0 = true, on1 = both;
    for (int k = 1; k < kmax && (on0 || on1); ++k) {
        // (4 nu^2 - (2k-1)^2) / k; past the table (never reached at these |z|) in FP64
        const double o = 2.0 * k - 1.0;
        if (on0) {
            const df a = k < BK_TAB ? tab_df(c_bkdf.asym[0][k]) : df_from_double(-o * o / k);
            t0 = dfc_scale(dfc_mul(t0, iz8), a);
            b0 = dfc_add(b0, t0);
            on0 = dfc_norm2f(t0) >= 1e-32f;
        }
        if (on1) {
            const df a = k < BK_TAB ? tab_df(c_bkdf.asym[1][k]) : df_from_double((4.0 - o * o) / k);
            t1 = dfc_scale(dfc_mul(t1, iz8), a);
            b1 = dfc_add(b1, t1);
            on1 = dfc_norm2f(t1) >= 1e-32f;
        }
    }
}

// Temme's Miller scheme (bk_miller in green.cuh): the normalising sum s, so
// that B_nu(z) = 1 / s
__device__ __forceinline__ dfc bk_miller_sum_df(int nu, dfc z, int jmax) {
    const dfc one{df{1.0f, 0.0f}, df{0.0f, 0.0f}};
    dfc inv = one, s{df{0.0f, 0.0f}, df{0.0f, 0.0f}};
    for (int j = jmax; j > 0; j--) {
        const df c = j < BK_TAB ? tab_df(c_bkdf.miller[nu][j])
                                : df_from_double((double)j / ((j - nu - 0.5) * (j + nu - 0.5)));
        // ratio = c (2 (z + j) - (j + 1) inv)
        const dfc zj{df_add(z.re, df{(float)j, 0.0f}), z.im};
        const dfc a = dfc_sub(dfc_scale(zj, df{2.0f, 0.0f}), dfc_scale(inv, df{(float)(j + 1), 0.0f}));
        inv = dfc_recip(dfc_scale(a, c));
        s = dfc_add(one, dfc_mul(s, inv));
    }
    return s;
}

// K_n(z), n = 0, 1, by the ascending series; lnh = ln(z/2)
__device__ __forceinline__ dfc bk_series_df(int n, dfc z, dfc lnh) {
    const dfc h = dfc_scale(z, df{0.5f, 0.0f}), q = dfc_mul(h, h);
    constexpr float2 EUL = split_df(EULER);
    const df eul = tab_df(EUL);
    // c = ln(h) - (psi(1) + psi(n+1)) / 2, t = h^n / n!
    dfc c{df_add(lnh.re, n == 0 ? eul : df_sub(eul, df{0.5f, 0.0f})), lnh.im};
    dfc t = n == 0 ? dfc{df{1.0f, 0.0f}, df{0.0f, 0.0f}} : h;
    dfc sum = dfc_mul(c, t);
    for (int k = 1; k < 50; k++) {
        t = dfc_scale(dfc_mul(t, q), tab_df(c_bkdf.ser_t[n][k]));
        c.re = df_sub(c.re, tab_df(c_bkdf.ser_c[n][k]));
        const dfc add = dfc_mul(c, t);
        sum = dfc_add(sum, add);
        if (dfc_norm2f(add) < 1e-32f * dfc_norm2f(sum)) break;
    }
    if (n == 0) return dfc{df_neg(sum.re), df_neg(sum.im)};
    return dfc_add(dfc_recip(dfc_scale(h, df{2.0f, 0.0f})), sum);  // 1/(2h) + sum
}

// M_ij = K_0(z)/(2 pi) and, if want_deriv, dM_ij = i r K_1(z)/(2 pi), for a pair at
// the double-float distance r in regime reg (k_regime_df)
__device__ __forceinline__ void pair_elements_df2(const Df3Tables& tab, const Df2Item& P, df r, int reg,
                                                  bool want_deriv, dfc& m, dfc& dm) {
    constexpr float2 INV2PI = split_df(1.0 / TWOPI);
    const df inv2pi = tab_df(INV2PI);
    const dfc z = dfc_scale(P.mik, r);
    dfc k0, k1;
    if (reg == 1) {
        const dfc lnh{df_add(P.lnh.re, df_from_double(log((double)r.h + (double)r.l))), P.lnh.im};
        k0 = bk_series_df(0, z, lnh);
        if (want_deriv) k1 = bk_series_df(1, z, lnh);
    } else {
        // sqrt(pi/2z) e^{-z} = pref r^(-1/2) e^{i k r}
        df cs, sn;
        df_cis(tab, df_mul(P.kr, r), cs, sn);
        const df e = P.grow ? df_exp_tab(tab, df_neg(df_mul(P.ki, r))) : df{1.0f, 0.0f};
        const dfc w = dfc_scale(dfc_mul(P.pref, dfc{cs, sn}), df_mul(e, df_recip(df_sqrt(r))));
        if (reg == 0) {
            const dfc iz8 = dfc_scale(P.rik, df_recip(df_mul(r, df{8.0f, 0.0f})));
            const int kmax = (int)floorf(2.0f * P.kabs * r.h);
            dfc b0, b1;
            bk_asym_df(iz8, kmax, want_deriv, b0, b1);
            k0 = dfc_mul(w, b0);
            if (want_deriv) k1 = dfc_mul(w, b1);
        } else {
            // Temme's start index from |z| and Re z (FP32 suffices: a different index
            // changes the result by the scheme's own truncation, ~1e-16)
            const float zr = z.re.h, za = P.kabs * r.h;
            const float x = zr + 36.841361f;
            const int jmax = (int)floorf(x * x / (4.0f * (zr + za)));
            k0 = dfc_mul(w, dfc_recip(bk_miller_sum_df(0, z, jmax)));
            if (want_deriv) k1 = dfc_mul(w, dfc_recip(bk_miller_sum_df(1, z, jmax)));
        }
    }
    m = dfc_scale(k0, inv2pi);
    if (want_deriv) {
        const dfc v = dfc_scale(k1, df_mul(r, inv2pi));
        dm = dfc{df_neg(v.im), v.re};  // i v
    }
}

}  // namespace msg
