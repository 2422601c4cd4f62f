// cplx.cuh -- FP64 complex arithmetic for device (and host) code.
//
// Layout is two doubles {re, im}, the same as C99 `double _Complex` and
// LAPACK COMPLEX*16, so matrices cross the C ABI without conversion.
// Transcendentals are built on CUDA's double-precision exp, log, sincos,
// atan2, hypot and sqrt (called, not re-implemented).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define MSG_HD __host__ __device__ __forceinline__

struct zc {
    double re, im;
};

MSG_HD zc mk(double r, double i = 0.0) { return zc{r, i}; }
MSG_HD zc operator+(zc a, zc b) { return zc{a.re + b.re, a.im + b.im}; }
MSG_HD zc operator-(zc a, zc b) { return zc{a.re - b.re, a.im - b.im}; }
MSG_HD zc operator-(zc a) { return zc{-a.re, -a.im}; }
MSG_HD zc operator*(zc a, zc b) { return zc{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
MSG_HD zc operator*(double s, zc a) { return zc{s * a.re, s * a.im}; }
MSG_HD zc operator*(zc a, double s) { return zc{s * a.re, s * a.im}; }
MSG_HD zc operator/(zc a, double s) { return zc{a.re / s, a.im / s}; }
MSG_HD zc operator+(zc a, double s) { return zc{a.re + s, a.im}; }
MSG_HD zc operator-(zc a, double s) { return zc{a.re - s, a.im}; }
MSG_HD zc operator+(double s, zc a) { return zc{a.re + s, a.im}; }
MSG_HD zc operator-(double s, zc a) { return zc{s - a.re, -a.im}; }
MSG_HD zc& operator+=(zc& a, zc b) { a.re += b.re; a.im += b.im; return a; }
MSG_HD zc& operator-=(zc& a, zc b) { a.re -= b.re; a.im -= b.im; return a; }
MSG_HD zc& operator*=(zc& a, zc b) { a = a * b; return a; }
MSG_HD bool is_zero(zc a) { return a.re == 0.0 && a.im == 0.0; }
MSG_HD double abs1(zc a) { return fabs(a.re) + fabs(a.im); }  // LAPACK dcabs1
MSG_HD double zabs(zc a) { return hypot(a.re, a.im); }
MSG_HD zc conjz(zc a) { return zc{a.re, -a.im}; }

// Smith's algorithm: a / b without premature overflow.
MSG_HD zc operator/(zc a, zc b) {
    if (fabs(b.re) >= fabs(b.im)) {
        double r = b.im / b.re, den = b.re + b.im * r;
        return zc{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
    } else {
        double r = b.re / b.im, den = b.re * r + b.im;
        return zc{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
    }
}
MSG_HD zc operator/(double s, zc b) { return zc{s, 0.0} / b; }
// 1 / b with Smith's scaling in two real divisions (the quotient above takes three)
MSG_HD zc zrecip(zc b) {
    if (fabs(b.re) >= fabs(b.im)) {
        const double r = b.im / b.re, d = 1.0 / (b.re + b.im * r);
        return zc{d, -r * d};
    }
    const double r = b.re / b.im, d = 1.0 / (b.re * r + b.im);
    return zc{r * d, -d};
}
MSG_HD zc& operator/=(zc& a, zc b) { a = a / b; return a; }

MSG_HD zc zexp(zc z) {
    double s, c, e = exp(z.re);
    sincos(z.im, &s, &c);
    return zc{e * c, e * s};
}
MSG_HD zc zlog(zc z) { return zc{log(hypot(z.re, z.im)), atan2(z.im, z.re)}; }
// principal square root
MSG_HD zc zsqrt(zc z) {
    if (z.re == 0.0 && z.im == 0.0) return zc{0.0, z.im};
    double t = sqrt(0.5 * (fabs(z.re) + hypot(z.re, z.im)));
    if (z.re >= 0.0) return zc{t, z.im / (2.0 * t)};
    return zc{fabs(z.im) / (2.0 * t), copysign(t, z.im)};
}
// z^p for real p, principal branch: exp(p log z); 0^p = 0 for p > 0, 1 for p = 0
MSG_HD zc zpow(zc z, double p) {
    if (p == 0.0) return zc{1.0, 0.0};
    if (z.re == 0.0 && z.im == 0.0) return zc{0.0, 0.0};
    return zexp(p * zlog(z));
}
MSG_HD double zabs2(zc a) { return a.re * a.re + a.im * a.im; }
