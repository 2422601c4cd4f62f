// green.cuh -- device FP64 special functions of the Foldy-Lax matrix.
//
//   G_d(k, r)  outgoing free Green function (reference src/core/green_bessel.c:280)
//   dG/dk      = (k / 2pi) G_{d-2}          (green_bessel.c:311)
//   K_nu(z)    modified Bessel function of the second kind, integer and
//              half-integer order, by three regimes chosen exactly where the
//              reference switches (green_bessel.c:208-218): the asymptotic
//              series for |z| > 16, the ascending series (DLMF 10.31.1) inside
//              the parabola Re z < 3 - (Im z)^2/12, and Temme's (1975) Miller
//              scheme elsewhere.
//   F(k)^-1    inverse single-atom amplitude, four models
//              (src/core/scattering_model_util.c:101-169).
//
// Everything is FP64: the phase k r and the Bessel functions at complex k
// need it.
#pragma once
#include "cplx.cuh"
#include "msgpu.h"

#define MSG_D __device__ __forceinline__

namespace msg {

constexpr double PI = 3.1415926535897932385;
constexpr double TWOPI = 6.2831853071795864769;
constexpr double FOURPI = 12.566370614359172954;
constexpr double SQRTPI = 1.7724538509055160273;
constexpr double EULER = 0.5772156649015328606;
constexpr double LN_EPS = -36.841361487904730944;  // ln(1e-16)

MSG_HD double uball_surface(int d) {
    if (d == 0) return 0.0;
    double s = (d % 2 == 0) ? TWOPI : 2.0;
    for (int m = d; m > 2;) { m -= 2; s *= TWOPI / m; }
    return s;
}

// Scalar coefficients of the K_nu loops for nu = 0, 1 (the orders the
// Foldy-Lax matrix and its k-derivative need), computed at compile time by the
// same double operations the loops would do; the FP64 pipe (1/64 of the FP32
// rate on GB300) then spends no division per iteration on them.
constexpr int BK_TAB = 128;
struct BkTables {
    double asym[2][BK_TAB];    // (4 nu^2 - (2k-1)^2) / k
    double ser_t[2][BK_TAB];   // 1 / (k (nu + k))
    double ser_c[2][BK_TAB];   // (1/k + 1/(nu + k)) / 2
    double miller[2][BK_TAB];  // j / ((j - nu - 1/2)(j + nu - 1/2))
};
constexpr BkTables make_bk_tables() {
    BkTables t{};
    for (int nu = 0; nu < 2; ++nu)
        for (int k = 1; k < BK_TAB; ++k) {
            const double o = 2.0 * k - 1.0, fn = 4.0 * nu * nu;
            t.asym[nu][k] = (fn - o * o) / k;
            t.ser_t[nu][k] = 1.0 / ((double)k * (nu + k));
            t.ser_c[nu][k] = 0.5 * (1.0 / k + 1.0 / (nu + k));
            t.miller[nu][k] = (double)k / ((k - nu - 0.5) * (k + nu - 0.5));
        }
    return t;
}
__constant__ BkTables c_bk = make_bk_tables();

// B_nu(z) = K_nu(z) / (sqrt(pi/2z) e^-z), asymptotic series (DLMF 10.40.2)
// truncated at the smallest term (index |2z|) or once |term| < 1e-16.
MSG_D zc bk_asym(int nu, zc z) {
    zc sum = mk(1.0), term = mk(1.0);
    int kmax = (int)floor(2.0 * zabs(z));
    double fn = 4.0 * nu * nu;
    zc iz8 = 1.0 / (8.0 * z);
    for (int k = 1; k < kmax; k++) {
        double o = 2.0 * k - 1.0;
        term = term * iz8 * ((nu < 2 && k < BK_TAB) ? c_bk.asym[nu][k] : (fn - o * o) / k);
        sum += term;
        if (zabs2(term) < 1e-32) break;
    }
    return sum;
}

// K_n(z), integer n >= 0, ascending series (DLMF 10.31.1):
//   1/2 (z/2)^-n sum_{k<n} (n-k-1)!/k! (-z^2/4)^k
//   + (-1)^(n+1) sum_k [ln(z/2) - (psi(k+1)+psi(n+k+1))/2] (z/2)^(n+2k) / (k!(n+k)!)
MSG_D zc bk_series(int n, zc z) {
    zc h = 0.5 * z, q = h * h;
    zc fin = mk(0.0);
    if (n > 0) {
        double fact = 1.0;
        for (int j = 2; j < n; j++) fact *= j;
        zc pw = mk(1.0), acc = mk(0.0);
        for (int k = 0; k < n; k++) {
            acc += fact * pw;
            pw = pw * (-q);
            if (k + 1 < n) fact = fact / (n - k - 1) / (k + 1);
        }
        zc hn = h;
        for (int j = 1; j < n; j++) hn = hn * h;
        fin = 0.5 * (acc / hn);
    }
    double psin = -EULER;
    for (int j = 1; j <= n; j++) psin += 1.0 / j;
    zc c = zlog(h) - 0.5 * (-EULER + psin);
    double nfact = 1.0;
    for (int j = 2; j <= n; j++) nfact *= j;
    zc t = mk(1.0 / nfact);
    for (int j = 0; j < n; j++) t = t * h;
    zc sum = c * t;
    const bool tab = n < 2;
    for (int k = 1; k < 50; k++) {
        t = t * q * (tab ? c_bk.ser_t[n][k] : 1.0 / ((double)k * (n + k)));
        c = c - (tab ? c_bk.ser_c[n][k] : 0.5 * (1.0 / k + 1.0 / (n + k)));
        zc add = c * t;
        sum += add;
        if (zabs2(add) < 1e-32 * zabs2(sum)) break;
    }
    return (n % 2 == 0) ? fin - sum : fin + sum;
}

// B_nu(z) by Temme's Miller scheme.  w_j = (nu+1/2)_j (1/2-nu)_j / j!
// U(nu+1/2+j, 2nu+1, 2z) obeys ((j-1/2)^2-nu^2)/j w_{j-1} = 2(j+z) w_j -
// (j+1) w_{j+1} and sum_j w_j = (2z)^-(nu+1/2), hence B_nu = w_0 / sum_j w_j.
// The backward ratio recurrence starts at Temme's estimate of the index.
MSG_D zc bk_miller(int nu, zc z) {
    double x = z.re + (-LN_EPS);
    int jmax = (int)floor(x * x / (4.0 * (z.re + zabs(z))));
    zc ratio = mk(1.0), s = mk(0.0);
    zc inv = mk(1.0);  // 1 / ratio: one complex reciprocal per step serves both quotients
    for (int j = jmax; j > 0; j--) {
        const double c = (nu < 2 && j < BK_TAB) ? c_bk.miller[nu][j] : (double)j / ((j - nu - 0.5) * (j + nu - 0.5));
        ratio = c * (2.0 * (z + (double)j) - (double)(j + 1) * inv);
        inv = zrecip(ratio);
        s = 1.0 + s * inv;
    }
    return 1.0 / s;
}

MSG_D zc bessel_k_int(int nu, zc z) {
    double x = z.re, y = z.im;
    if (x * x + y * y > 256.0) return zsqrt(0.5 * PI / z) * zexp(-z) * bk_asym(nu, z);
    if (x < 3.0 - y * y / 12.0) return bk_series(nu, z);
    return zsqrt(0.5 * PI / z) * zexp(-z) * bk_miller(nu, z);
}

// K_{twonu/2}(z); half-integer orders by the terminating expansion (DLMF 10.49.12),
// integer orders >= 2 by forward recurrence from K_0, K_1.
MSG_D zc bessel_k(int twonu, zc z) {
    if (twonu < 0) twonu = -twonu;
    if (twonu == 0 || twonu == 2) return bessel_k_int(twonu / 2, z);
    if (twonu % 2 == 0) {
        zc km = bessel_k_int(0, z), k = bessel_k_int(1, z), kp = mk(0.0);
        for (int m = 1; m < twonu / 2; m++) { kp = km + (2.0 * m) * k / z; km = k; k = kp; }
        return kp;
    }
    int m = (twonu + 1) / 2;
    zc sum = mk(1.0), term = mk(1.0);
    for (int i = 1; i < m; i++) { term = term * ((double)(m - i) * (m + i - 1) / i) / (2.0 * z); sum += term; }
    return zsqrt(PI / (2.0 * z)) * zexp(-z) * sum;
}

// G_d(k, r): d=1 e^{ikr}/(2ik); d=3 -e^{ikr}/(4 pi r); d=2 -K_0(-ikr)/(2pi);
// otherwise -(-ik/(2 pi r))^{(d-2)/2} K_{(d-2)/2}(-ikr) / (2pi).
MSG_D zc free_green(int d, zc k, double r) {
    zc ik = mk(-k.im, k.re);
    if (d == 3) return -(zexp(ik * r) / (FOURPI * r));
    if (d == 2) return -(bessel_k_int(0, -(ik * r)) / TWOPI);
    if (d == 1) return zexp(ik * r) / (2.0 * ik);
    return -(zpow(-ik / (TWOPI * r), (d - 2.0) / 2.0) * bessel_k(d - 2, -(ik * r)) / TWOPI);
}

MSG_D zc dk_free_green(int d, zc k, double r) { return (k / TWOPI) * free_green(d - 2, k, r); }

// regularized 0F1(;a;z) power series (reference green_bessel.c:254)
MSG_D zc hyp0f1(double a, zc z) {
    zc t = mk(1.0);
    if (a < 1.0 && fmod(a, 1.0) == 0.0) { t = zpow(z, 1.0 - a); a = 2.0 - a; }
    t = t / tgamma(a);
    zc s = t;
    for (int i = 1; i <= 50; i++) {
        t = t * z / (i * a);
        s += t;
        a += 1.0;
        if (zabs(t) < 1e-16 * zabs(s)) break;
    }
    return s;
}

// I_d(k, r) = -Im G continued to complex k (reference green_bessel.c:298)
MSG_D zc free_green_imag(int d, zc k, double r) {
    if (zabs(k) * r < 3.0) {
        zc x = k * r;
        return 0.25 * zpow(k / (2.0 * SQRTPI), d - 2.0) * hyp0f1(d / 2.0, -(x * x) / 4.0);
    }
    double sg = (k.re < 0 && d % 2 == 0) ? -1.0 : 1.0;
    zc diff = free_green(d, -k, r) - free_green(d, k, r);
    return sg * (diff / mk(0.0, 2.0));
}

// F(k)^-1 for the model (reference scattering_model_util.c:101-169)
MSG_D zc invf(const msgpu_model& m, int d, zc k) {
    switch (m.type) {
    case MSGPU_MAXIMUM: {
        zc i0 = (uball_surface(d) / (8.0 * PI)) * zpow(k / TWOPI, d - 2.0);
        return mk(-i0.im, i0.re);
    }
    case MSGPU_HARDSPHERE: {
        double a = m.p[0];
        zc i0 = (uball_surface(d) / (8.0 * PI)) * zpow(k / TWOPI, d - 2.0);
        return -(i0 * free_green(d, k, a) / free_green_imag(d, k, a));
    }
    case MSGPU_SOFTSPHERE: {
        double a = m.p[0];
        if (d == 2) return zlog(mk(0.0, 1.0) / (a * k)) / TWOPI;
        double pre = (d % 2 == 0) ? 0.25 : a / 2.0, fr = TWOPI * a * a;
        for (int m2 = d; m2 > 2;) { m2 -= 2; pre /= fr * m2; }
        zc w = zpow(a * k, d - 2.0);
        return pre * (1.0 + mk(-w.im, w.re));
    }
    case MSGPU_RESONANT: {
        zc i0 = (uball_surface(d) / (8.0 * PI)) * zpow(k / TWOPI, d - 2.0);
        return i0 * (mk(0.0, 1.0) - (k - m.p[0]) / m.p[1]);
    }
    default:
        return mk(0.0);
    }
}

// diagonal of dM/dk: central difference with step 1e-4 (reference ms_matrix_util.c:69-70)
MSG_D zc dk_invf(const msgpu_model& m, int d, zc k) {
    const double h = 1e-4;
    return (invf(m, d, k + h) - invf(m, d, k - h)) / (2.0 * h);
}

MSG_D double atom_distance(int d, const double* __restrict__ pos, int i, int j) {
    double r2 = 0.0;
    for (int c = 0; c < d; c++) {
        double t = pos[i * d + c] - pos[j * d + c];
        r2 += t * t;
    }
    return sqrt(r2);
}

}  // namespace msg
