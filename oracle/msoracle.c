/*
 * msoracle.c -- CPU oracle (test infrastructure, never shipped or called by
 * the product).  A restatement, in this project's own code, of the reference
 * algorithms of MSModel v1.0.0 on the Foldy-Lax hot path.  Citations are to
 * files of the reference project (src/core/...).
 *
 * Parity is pinned two ways: (1) against the golden vectors the reference's
 * own tests hold (src/test/test_ms_matrix.c, src/test/test_green_bessel_data.h,
 * Mathematica values), and (2) against the reference itself compiled from its
 * sources into oracle/_ref (see oracle/build_oracle.py).
 */
#define _GNU_SOURCE
#include "msoracle.h"
#include <complex.h>
#include <dlfcn.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

static const double O_PI = 3.1415926535897932385;
static const double O_TWOPI = 6.2831853071795864769;
static const double O_FOURPI = 12.566370614359172954;
static const double O_SQRTPI = 1.7724538509055160273;
static const double O_EULER = 0.5772156649015328606;

static inline cplx ld2(const double* p) { return p[0] + I * p[1]; }
static inline void st2(double* p, cplx z) { p[0] = creal(z); p[1] = cimag(z); }

/* ------------------------------------------------------------------------
 * LAPACK (the reference links -llapack, Makefile:31; here the OpenBLAS that
 * scipy bundles is loaded at run time).
 * ---------------------------------------------------------------------- */
typedef void (*zgetrf_t)(int*, int*, cplx*, int*, int*, int*);
typedef void (*zgetrs_t)(char*, int*, int*, cplx*, int*, int*, cplx*, int*, int*);
typedef void (*zgels_t)(char*, int*, int*, int*, cplx*, int*, cplx*, int*, cplx*, int*, int*);
typedef void (*setnt_t)(int);
typedef char* (*getcfg_t)(void);
static zgetrf_t p_zgetrf;
static zgetrs_t p_zgetrs;
static zgels_t p_zgels;
static getcfg_t p_getcfg;

int orc_set_lapack(const char* path) {
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return 1;
    p_zgetrf = (zgetrf_t)dlsym(h, "scipy_zgetrf_");
    p_zgetrs = (zgetrs_t)dlsym(h, "scipy_zgetrs_");
    p_zgels = (zgels_t)dlsym(h, "scipy_zgels_");
    p_getcfg = (getcfg_t)dlsym(h, "scipy_openblas_get_config");
    setnt_t setnt = (setnt_t)dlsym(h, "scipy_openblas_set_num_threads");
    if (setnt) setnt(1); /* one LAPACK thread per caller, as the reference runs it */
    return (p_zgetrf && p_zgetrs && p_zgels) ? 0 : 2;
}
int orc_have_lapack(void) { return p_zgetrf != NULL; }
const char* orc_lapack_config(void) { return p_getcfg ? p_getcfg() : "oracle-restated zgetf2"; }

/* ------------------------------------------------------------------------
 * RNG: Numerical Recipes "Ran" (src/core/nru_random.c:24-39 next_state /
 * random_double, :63 init_random).  State = {u, v, w, seed}.
 * ---------------------------------------------------------------------- */
uint64_t orc_rng_next(uint64_t* s) {
    uint64_t u = s[0], v = s[1], w = s[2];
    u = u * 2862933555777941757ULL + 7046029254386353087ULL;
    v ^= v >> 17; v ^= v << 31; v ^= v >> 8;
    w = 4294957665ULL * (w & 0xffffffffULL) + (w >> 32);
    uint64_t x = u ^ (u << 21);
    x ^= x >> 35; x ^= x << 4;
    s[0] = u; s[1] = v; s[2] = w;
    return (x + v) ^ w;
}
double orc_rng_double(uint64_t* s) { return 5.42101086242752217E-20 * (double)orc_rng_next(s); }
void orc_rng_init(uint64_t* s, uint64_t seed) {
    s[3] = seed;
    s[1] = 4101842887655102017ULL;
    s[2] = 1;
    s[0] = seed ^ s[1];
    orc_rng_next(s);
    s[1] = s[0];
    orc_rng_next(s);
    s[2] = s[1];
    orc_rng_next(s);
}
/* normal deviate by ratio of uniforms (nru_random.c:48) */
static double rng_normal(uint64_t* s) {
    double u, v, x, y, q;
    for (;;) {
        u = orc_rng_double(s);
        v = 1.7156 * (orc_rng_double(s) - 0.5);
        x = u - 0.449871;
        y = fabs(v) + 0.386595;
        q = x * x + y * (0.19600 * y - 0.25472 * x);
        if (!(q > 0.27597 && (q > 0.27846 || v * v > -4. * u * u * log(u)))) break;
    }
    return v / u;
}

/* unit d-ball volume / surface (src/core/green_bessel.c:41, :63) */
double orc_uball_volume(int d) {
    if (d == 0) return 1.;
    double v = (d % 2 == 0) ? O_PI : 2.;
    for (int m = d; m > 2; m -= 2) v *= O_TWOPI / m;
    return v;
}
double orc_uball_surface(int d) {
    if (d == 0) return 0.;
    double s = (d % 2 == 0) ? O_TWOPI : 2.;
    for (int m = d; m > 2;) { m -= 2; s *= O_TWOPI / m; }
    return s;
}

/* Seeded scatterers, atom-major pos[i*d + c] (src/core/medium_util.c:95-193). */
void orc_fill_medium(int d, int n, int shape, double ratio, uint64_t seed, double* pos) {
    uint64_t st[4];
    orc_rng_init(st, seed);
    if (d == 1 && shape == ORC_BALL) shape = ORC_CUBE; /* medium_util.c:57 */
    int ntot = n * d;
    if (shape == ORC_CUBE) {
        double s = pow(n, 1. / d);
        for (int l = 0; l < ntot; l++) pos[l] = s * orc_rng_double(st);
    } else if (shape == ORC_BALL) {
        double rad = pow(n / orc_uball_volume(d), 1. / d);
        double r2 = rad * rad;
        for (int i = 0; i < n; i++) {
            double nrm;
            do {
                nrm = 0.;
                for (int c = 0; c < d; c++) {
                    double x = rad * (2 * orc_rng_double(st) - 1);
                    pos[i * d + c] = x;
                    nrm += x * x;
                }
            } while (nrm > r2);
        }
    } else if (shape == ORC_LATTICE) {
        int s = (int)ceil(pow(n, 1. / d));
        for (int i = 0; i < n; i++) {
            int v = i;
            for (int c = 0; c < d; c++) { pos[i * d + c] = v % s; v /= s; }
        }
    } else {
        double sig = pow(n, 1. / d) / 2.506628274631000502;
        for (int l = 0; l < ntot; l++) pos[l] = sig * rng_normal(st);
    }
    if (ratio != 1. && d != 1) {
        double f2 = pow(ratio, -1. / d), f1 = ratio * f2;
        for (int l = 0; l < ntot; l++) pos[l] *= (l % d == 0) ? f1 : f2;
    }
}

static double dist(int d, const double* a, const double* b) {
    double r2 = 0.;
    for (int c = 0; c < d; c++) { double t = a[c] - b[c]; r2 += t * t; }
    return sqrt(r2);
}

/* ------------------------------------------------------------------------
 * Modified Bessel K_nu(z), integer nu >= 0.  Region choice as in
 * src/core/green_bessel.c:208-218: |z|>16 asymptotic, inside the parabola
 * Re z < 3 - (Im z)^2/12 the power series, otherwise Temme's Miller scheme.
 * ---------------------------------------------------------------------- */

/* B_nu(z) = K_nu(z) / (sqrt(pi/2z) e^-z) by the asymptotic series (DLMF
 * 10.40.2), truncated at the smallest term, |2z| (green_bessel.c:106). */
static cplx bk_asym(int nu, cplx z) {
    cplx sum = 1., term = 1.;
    int kmax = (int)floor(cabs(2. * z));
    double fn = 4. * nu * nu;
    for (int k = 1; k < kmax; k++) {
        double o = 2. * k - 1.;
        term *= (fn - o * o) / (8. * k * z);
        sum += term;
        if (creal(term) * creal(term) + cimag(term) * cimag(term) < 1e-32) break;
    }
    return sum;
}

/* K_n(z) by the ascending series (DLMF 10.31.1), green_bessel.c:125. */
static cplx bk_series(int n, cplx z) {
    cplx h = 0.5 * z, q = h * h;
    cplx fin = 0.;
    if (n > 0) {
        /* 1/2 (z/2)^-n sum_{k<n} (n-k-1)!/k! (-z^2/4)^k */
        double fact = 1.;
        for (int j = 2; j < n; j++) fact *= j;          /* (n-1)! */
        cplx pw = 1., acc = 0.;
        for (int k = 0; k < n; k++) {
            acc += fact * pw;
            pw *= -q;
            if (k + 1 < n) fact = fact / (n - k - 1) / (k + 1); /* (n-k-2)!/(k+1)! */
        }
        fin = 0.5 * acc / cpow(h, n);
    }
    /* (-1)^(n+1) sum_k [ln(z/2) - (psi(k+1)+psi(n+k+1))/2] (z/2)^(n+2k)/(k!(n+k)!) */
    double psin = -O_EULER;
    for (int j = 1; j <= n; j++) psin += 1. / j;
    cplx c = clog(h) - 0.5 * (-O_EULER + psin);
    double nfact = 1.;
    for (int j = 2; j <= n; j++) nfact *= j;
    cplx t = (n > 0 ? cpow(h, n) : 1.) / nfact;
    cplx sum = c * t;
    for (int k = 1; k < 50; k++) {
        t *= q / ((double)k * (n + k));
        c -= 0.5 * (1. / k + 1. / (n + k));
        cplx add = c * t;
        sum += add;
        if (creal(add) * creal(add) + cimag(add) * cimag(add) <
            1e-32 * (creal(sum) * creal(sum) + cimag(sum) * cimag(sum)))
            break;
    }
    return fin + ((n % 2 == 0) ? -sum : sum);
}

/* B_nu(z) by Temme's (1975) Miller scheme on w_j = (nu+1/2)_j (1/2-nu)_j / j!
 * U(nu+1/2+j, 2nu+1, 2z), which obeys
 *   ((j-1/2)^2-nu^2)/j w_{j-1} - 2(j+z) w_j + (j+1) w_{j+1} = 0
 * and sum_j w_j = (2z)^-(nu+1/2), so that B_nu = w_0 / sum_j w_j.
 * Start index from Temme's estimate (green_bessel.c:187). */
static cplx bk_miller(int nu, cplx z) {
    int jmax = (int)floor((creal(z) + 36.841361487904730944) * (creal(z) + 36.841361487904730944) /
                          (4. * (creal(z) + cabs(z))));
    cplx ratio = 1., s = 0.; /* ratio = w_{j-1}/w_j ; s = sum_{i>=j} w_i / w_{j-1} */
    for (int j = jmax; j > 0; j--) {
        double c = (double)j / ((j - nu - 0.5) * (j + nu - 0.5));
        ratio = c * (2. * (z + j) - (j + 1) / ratio);
        s = 1. + s / ratio;
    }
    return 1. / s;
}

static cplx bessel_k_int(int nu, cplx z) {
    double x = creal(z), y = cimag(z);
    if (x * x + y * y > 256.) return csqrt(0.5 * O_PI / z) * cexp(-z) * bk_asym(nu, z);
    if (x < 3. - y * y / 12.) return bk_series(nu, z);
    return csqrt(0.5 * O_PI / z) * cexp(-z) * bk_miller(nu, z);
}

/* K_nu for nu = twonu/2 integer or half integer (green_bessel.c:224).
 * Half-integer orders use the terminating expansion (DLMF 10.49.12). */
static cplx bessel_k(int twonu, cplx z) {
    if (twonu < 0) twonu = -twonu;
    if (twonu == 0 || twonu == 2) return bessel_k_int(twonu / 2, z);
    if (twonu % 2 == 0) {
        cplx km = bessel_k_int(0, z), k = bessel_k_int(1, z), kp = 0.;
        for (int m = 1; m < twonu / 2; m++) { kp = km + (2. * m) * k / z; km = k; k = kp; }
        return kp;
    }
    int m = (twonu + 1) / 2; /* nu + 1/2 */
    cplx sum = 1., term = 1.;
    for (int i = 1; i < m; i++) { term *= (double)(m - i) * (m + i - 1) / (2. * z * i); sum += term; }
    return csqrt(O_PI / (2. * z)) * cexp(-z) * sum;
}
void orc_bessel_k(int twonu, const double* z, double* out) { st2(out, bessel_k(twonu, ld2(z))); }

/* Outgoing free Green function G_d(k, r) (green_bessel.c:280). */
static cplx free_green(int d, cplx k, double r) {
    cplx ik = I * k;
    if (d == 1) return cexp(ik * r) / (2. * ik);
    if (d == 3) return -cexp(ik * r) / (O_FOURPI * r);
    if (d == 2) return -bessel_k_int(0, -ik * r) / O_TWOPI;
    return -cpow(-ik / (O_TWOPI * r), (d - 2.) / 2.) * bessel_k(d - 2, -ik * r) / O_TWOPI;
}
/* dG/dk = (k/2pi) G_{d-2} (green_bessel.c:311). */
static cplx dk_free_green(int d, cplx k, double r) { return (k / O_TWOPI) * free_green(d - 2, k, r); }

/* Regularized 0F1(;a;z) by its power series (green_bessel.c:254). */
static cplx hyp0f1(double a, cplx z) {
    cplx t = 1.;
    if (a < 1. && fmod(a, 1.) == 0.) { t = cpow(z, 1. - a); a = 2. - a; }
    t /= tgamma(a);
    cplx s = t;
    for (int i = 1; i <= 50; i++) {
        t *= z / (i * a);
        s += t;
        a += 1.;
        if (cabs(t) < 1e-16 * cabs(s)) break;
    }
    return s;
}
/* I_d(k,r) = -Im G continued to complex k (green_bessel.c:298). */
static cplx free_green_imag(int d, cplx k, double r) {
    if (cabs(k) * r < 3.) {
        cplx x = k * r;
        return 0.25 * cpow(k / (2. * O_SQRTPI), d - 2.) * hyp0f1(d / 2., -x * x / 4.);
    }
    int sg = (creal(k) < 0 && d % 2 == 0) ? -1 : 1;
    return sg * (free_green(d, -k, r) - free_green(d, k, r)) / (2. * I);
}

void orc_free_green(int d, const double* k, double r, double* out) { st2(out, free_green(d, ld2(k), r)); }
void orc_dk_free_green(int d, const double* k, double r, double* out) { st2(out, dk_free_green(d, ld2(k), r)); }
void orc_free_green_imag(int d, const double* k, double r, double* out) { st2(out, free_green_imag(d, ld2(k), r)); }
void orc_hyp0f1(double a, const double* z, double* out) { st2(out, hyp0f1(a, ld2(z))); }

/* Inverse single-atom amplitude F(k)^-1 (src/core/scattering_model_util.c:101-169). */
static cplx invf(const orc_model* m, int d, cplx k) {
    switch (m->type) {
    case ORC_MAXIMUM: {
        cplx i0 = orc_uball_surface(d) * cpow(k / O_TWOPI, d - 2) / (8 * O_PI);
        return I * i0;
    }
    case ORC_HARDSPHERE: {
        double a = m->p[0];
        cplx i0 = orc_uball_surface(d) * cpow(k / O_TWOPI, d - 2) / (8 * O_PI);
        return -i0 * free_green(d, k, a) / free_green_imag(d, k, a);
    }
    case ORC_SOFTSPHERE: {
        double a = m->p[0];
        if (d == 2) return clog(I / (a * k)) / O_TWOPI;
        double pre = (d % 2 == 0) ? 0.25 : a / 2, fr = O_TWOPI * a * a;
        for (int m2 = d; m2 > 2;) { m2 -= 2; pre /= fr * m2; }
        return pre * (1. + I * cpow(a * k, d - 2));
    }
    case ORC_RESONANT: {
        cplx i0 = orc_uball_surface(d) * cpow(k / O_TWOPI, d - 2) / (8 * O_PI);
        return i0 * (I - (k - m->p[0]) / m->p[1]);
    }
    default:
        return 0.;
    }
}
void orc_invf(const orc_model* m, int d, const double* k, double* out) { st2(out, invf(m, d, ld2(k))); }

/* ------------------------------------------------------------------------
 * Matrices (src/core/ms_matrix_util.c:32-44 build_ms_matrix, :68-81
 * build_dk_ms_matrix): column-major, symmetric fill, F^-1 on the diagonal,
 * central difference with step 1e-4 for the diagonal of dM/dk.
 * ---------------------------------------------------------------------- */
static void build_m(int d, int n, const double* pos, const orc_model* m, cplx k, cplx* a) {
    cplx dg = invf(m, d, k);
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < j; i++) {
            cplx e = -free_green(d, k, dist(d, pos + i * d, pos + j * d));
            a[i + (size_t)j * n] = e;
            a[j + (size_t)i * n] = e;
        }
        a[(size_t)(n + 1) * j] = dg;
    }
}
static void build_dm(int d, int n, const double* pos, const orc_model* m, cplx k, cplx* a) {
    const double h = 1e-4;
    cplx dg = (invf(m, d, k + h) - invf(m, d, k - h)) / (2 * h);
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < j; i++) {
            cplx e = -dk_free_green(d, k, dist(d, pos + i * d, pos + j * d));
            a[i + (size_t)j * n] = e;
            a[j + (size_t)i * n] = e;
        }
        a[(size_t)(n + 1) * j] = dg;
    }
}
void orc_build_ms_matrix(int d, int n, const double* pos, const orc_model* m, const double* k, double* mat) {
    build_m(d, n, pos, m, ld2(k), (cplx*)mat);
}
void orc_build_dk_ms_matrix(int d, int n, const double* pos, const orc_model* m, const double* k, double* mat) {
    build_dm(d, n, pos, m, ld2(k), (cplx*)mat);
}

/* LAPACK zgetf2 restated: right-looking, pivot = first max of |re|+|im|
 * (IZAMAX), 1-based ipiv, info = first exactly-zero pivot. */
static int lu_restated(int n, cplx* a, int* ipiv) {
    int info = 0;
    for (int j = 0; j < n; j++) {
        int p = j;
        double best = -1.;
        for (int i = j; i < n; i++) {
            cplx v = a[i + (size_t)j * n];
            double m1 = fabs(creal(v)) + fabs(cimag(v));
            if (m1 > best) { best = m1; p = i; }
        }
        ipiv[j] = p + 1;
        cplx piv = a[p + (size_t)j * n];
        if (piv != 0.) {
            if (p != j)
                for (int c = 0; c < n; c++) {
                    cplx t = a[j + (size_t)c * n];
                    a[j + (size_t)c * n] = a[p + (size_t)c * n];
                    a[p + (size_t)c * n] = t;
                }
            if (cabs(piv) >= DBL_MIN) {
                cplx r = 1. / piv;
                for (int i = j + 1; i < n; i++) a[i + (size_t)j * n] *= r;
            } else {
                for (int i = j + 1; i < n; i++) a[i + (size_t)j * n] /= piv;
            }
        } else if (info == 0) {
            info = j + 1;
        }
        for (int c = j + 1; c < n; c++) {
            cplx u = a[j + (size_t)c * n];
            if (u == 0.) continue;
            for (int i = j + 1; i < n; i++) a[i + (size_t)c * n] -= a[i + (size_t)j * n] * u;
        }
    }
    return info;
}
int orc_lu(int n, double* mat, int* ipiv, int use_lapack) {
    int info = 0;
    if (use_lapack && p_zgetrf) { p_zgetrf(&n, &n, (cplx*)mat, &n, ipiv, &info); return info; }
    return lu_restated(n, (cplx*)mat, ipiv);
}
/* zgetrs restated for nrhs columns */
static void lu_solve(int n, const cplx* a, const int* ipiv, int nrhs, cplx* b, int use_lapack) {
    if (use_lapack && p_zgetrs) {
        int info, ld = n;
        char tr = 'N';
        p_zgetrs(&tr, &n, &nrhs, (cplx*)a, &ld, (int*)ipiv, b, &ld, &info);
        return;
    }
    for (int c = 0; c < nrhs; c++) {
        cplx* x = b + (size_t)c * n;
        for (int i = 0; i < n; i++) {
            int p = ipiv[i] - 1;
            if (p != i) { cplx t = x[i]; x[i] = x[p]; x[p] = t; }
        }
        for (int j = 0; j < n; j++) {
            cplx xj = x[j];
            if (xj != 0.)
                for (int i = j + 1; i < n; i++) x[i] -= xj * a[i + (size_t)j * n];
        }
        for (int j = n - 1; j >= 0; j--) {
            if (x[j] != 0.) {
                x[j] /= a[j + (size_t)j * n];
                cplx xj = x[j];
                for (int i = 0; i < j; i++) x[i] -= xj * a[i + (size_t)j * n];
            }
        }
    }
}

/* tracelog_lu (ms_matrix_util.c:185-202): sum clog(U_ii), +i pi for an odd
 * number of interchanges, divided by n. */
static cplx tracelog(int n, cplx* a, int use_lapack, int* infop) {
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
    int info = orc_lu(n, (double*)a, ipiv, use_lapack);
    cplx tl = 0.;
    int sg = 1;
    for (int i = 0; i < n; i++) {
        tl += clog(a[i + (size_t)i * n]);
        if (ipiv[i] != i + 1) sg = -sg;
    }
    if (sg == -1) tl += I * O_PI;
    free(ipiv);
    if (infop) *infop = info;
    return tl / n;
}
int orc_tracelog_lu(int n, double* mat, int use_lapack, double* out) {
    int info;
    st2(out, tracelog(n, (cplx*)mat, use_lapack, &info));
    return info;
}

/* dk_log_det_ms (ms_matrix_util.c:242-263): tr(M^-1 dM/dk) by LU + n-RHS solve. */
static cplx dlogf(int d, int n, const double* pos, const orc_model* m, cplx k, int use_lapack, cplx* a,
                  cplx* b, int* ipiv) {
    build_m(d, n, pos, m, k, a);
    build_dm(d, n, pos, m, k, b);
    orc_lu(n, (double*)a, ipiv, use_lapack);
    lu_solve(n, a, ipiv, n, b, use_lapack);
    cplx tr = 0.;
    for (int i = 0; i < n; i++) tr += b[(size_t)(n + 1) * i];
    return tr;
}
int orc_dk_log_det(int d, int n, const double* pos, const orc_model* m, const double* k, int use_lapack,
                   double* out) {
    cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
    cplx* b = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
    st2(out, dlogf(d, n, pos, m, ld2(k), use_lapack, a, b, ipiv));
    free(a); free(b); free(ipiv);
    return 0;
}

int orc_solve(int n, double* mat, double* rhs, int use_lapack) {
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
    int info = orc_lu(n, mat, ipiv, use_lapack);
    lu_solve(n, (cplx*)mat, ipiv, 1, (cplx*)rhs, use_lapack);
    free(ipiv);
    return info;
}

/* total_cross_section (ms_matrix_util.c:344-366): -Im(conj(phi).M^-1 phi)/k */
double orc_total_cross_section(int d, int n, const double* pos, const orc_model* m, double k, int use_lapack) {
    cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
    cplx* b = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    cplx* phi = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    build_m(d, n, pos, m, k, a);
    for (int i = 0; i < n; i++) { phi[i] = cexp(I * k * pos[i * d]); b[i] = phi[i]; }
    orc_solve(n, (double*)a, (double*)b, use_lapack);
    cplx dot = 0.;
    for (int i = 0; i < n; i++) dot += conj(phi[i]) * b[i];
    free(a); free(b); free(phi);
    return -cimag(dot) / k;
}

/* ------------------------------------------------------------------------
 * Batched drivers: run_tracelog_omp (src/core/ms_core.c:96-141) and the
 * DOS-style dlogf loop (ms_core.c:476-519), one private matrix per thread.
 * ---------------------------------------------------------------------- */
void orc_tracelog_batch(int d, int n, const double* pos, const orc_model* m, int nk, const double* ks,
                        double* out, int* info, int nthreads, int use_lapack) {
#pragma omp parallel num_threads(nthreads)
    {
        cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
#pragma omp for schedule(static, 1)
        for (int l = 0; l < nk; l++) {
            int inf;
            build_m(d, n, pos, m, ld2(ks + 2 * l), a);
            st2(out + 2 * l, tracelog(n, a, use_lapack, &inf));
            if (info) info[l] = inf;
        }
        free(a);
    }
}
void orc_dlogf_batch(int d, int n, const double* pos, const orc_model* m, int nk, const double* ks,
                     double* out, int nthreads, int use_lapack) {
#pragma omp parallel num_threads(nthreads)
    {
        cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
        cplx* b = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
        int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
#pragma omp for schedule(static, 1)
        for (int l = 0; l < nk; l++) st2(out + 2 * l, dlogf(d, n, pos, m, ld2(ks + 2 * l), use_lapack, a, b, ipiv));
        free(a); free(b); free(ipiv);
    }
}

/* k-grids: get_arg_cmap (src/core/complex_map_util.c:27-31, steps :90-91),
 * get_arg_ccut (src/core/complex_cut_util.c:32-36, ntot = 3(ns+2) :75). */
void orc_kplane_args(int nx, int ny, double xmin, double xmax, double ymin, double ymax, double* ks) {
    double dx = (xmax - xmin) / (nx - 1), dy = (ymax - ymin) / (ny - 1);
    for (int l = 0; l < nx * ny; l++) {
        int ix = l % nx, iy = l / nx;
        ks[2 * l] = xmin + ix * dx;
        ks[2 * l + 1] = ymax - iy * dy;
    }
}
void orc_kcut_args(int ns, const double* zmin, const double* zmax, double* ks) {
    cplx a = ld2(zmin), b = ld2(zmax), dz = (b - a) / (ns - 1);
    for (int l = 0; l < 3 * (ns + 2); l++) {
        int il = l / 3, it = l % 3;
        st2(ks + 2 * l, ((ns - il) * a + (il - 1) * b) / (ns - 1) + I * dz * (it - 1));
    }
}

/* Halton (2,3) points from index 1 (src/core/domain_util.c:156-185);
 * dom = {xmin, xmax, ymin, ymax}. */
static double halton(int i, int b) {
    double h = 0., f = 1.;
    while (i > 0) { f /= b; h += f * (i % b); i /= b; }
    return h;
}
void orc_halton_points(const double* dom, int n, double* z) {
    for (int i = 0; i < n; i++) {
        z[2 * i] = dom[0] + (dom[1] - dom[0]) * halton(i + 1, 2);
        z[2 * i + 1] = dom[2] + (dom[3] - dom[2]) * halton(i + 1, 3);
    }
}
static int in_dom(const double* dom, cplx z) {
    return dom[0] < creal(z) && creal(z) < dom[1] && dom[2] < cimag(z) && cimag(z) < dom[3];
}

/* Least squares by Householder QR (the reference calls zgels_,
 * src/core/root_finder.c:59-68); a is m x nc column-major, b length m. */
static void cleast_squares(int m, int nc, cplx* a, cplx* b, int use_lapack) {
    if (use_lapack && p_zgels) {
        int nrhs = 1, lda = m, ldb = m, lwork = 2 * nc, info;
        char tr = 'N';
        cplx* work = (cplx*)calloc((size_t)lwork, sizeof(cplx));
        p_zgels(&tr, &m, &nc, &nrhs, a, &lda, b, &ldb, work, &lwork, &info);
        free(work);
        return;
    }
    for (int j = 0; j < nc; j++) {
        double nrm = 0.;
        for (int i = j; i < m; i++) nrm += creal(a[i + j * m] * conj(a[i + j * m]));
        nrm = sqrt(nrm);
        if (nrm == 0.) continue;
        cplx x0 = a[j + j * m];
        cplx alpha = (cabs(x0) > 0 ? -x0 / cabs(x0) : -1.) * nrm;
        a[j + j * m] -= alpha;                 /* v = x - alpha e1 */
        double vn = 0.;
        for (int i = j; i < m; i++) vn += creal(a[i + j * m] * conj(a[i + j * m]));
        for (int c = j + 1; c < nc; c++) {
            cplx s = 0.;
            for (int i = j; i < m; i++) s += conj(a[i + j * m]) * a[i + c * m];
            s = 2. * s / vn;
            for (int i = j; i < m; i++) a[i + c * m] -= s * a[i + j * m];
        }
        cplx s = 0.;
        for (int i = j; i < m; i++) s += conj(a[i + j * m]) * b[i];
        s = 2. * s / vn;
        for (int i = j; i < m; i++) b[i] -= s * a[i + j * m];
        a[j + j * m] = alpha;                  /* R_jj */
    }
    for (int j = nc - 1; j >= 0; j--) {
        cplx s = b[j];
        for (int c = j + 1; c < nc; c++) s -= a[j + c * m] * b[c];
        b[j] = s / a[j + j * m];
    }
}

static int cmp_re(const void* x, const void* y) {
    double a = creal(*(const cplx*)x), b = creal(*(const cplx*)y);
    return (a > b) - (a < b);
}

/* solve_aberth (src/core/root_finder.c:522-577) on dlogf = dk_log_det_ms
 * with the background polynomial fitted on 6*nexpsup Halton samples
 * (fit_cpoly_from_func :161, eval_cpoly :77). Gauss-Seidel sweep: root i
 * sees the already-updated roots j < i. */
int orc_solve_aberth(int d, int n, const double* pos, const orc_model* m, const double* dom, int nz, double* zz,
                     int nexpsup, int maxit, double toler, int use_lapack, int* nevals) {
    cplx* z = (cplx*)zz;
    int ne = 0;
    /* uniq_cvector (complex_vector_util.c:130) then exclude_from_domain (domain_util.c:133) */
    int size = nz > 0 ? 1 : 0;
    for (int i = 1; i < nz; i++) {
        int uniq = 1;
        for (int j = 0; j < size; j++)
            if (cabs(z[i] - z[j]) < toler * cabs(z[i]) || cabs(z[i] - z[j]) < toler) { uniq = 0; break; }
        if (uniq) { if (i != size) { cplx t = z[i]; z[i] = z[size]; z[size] = t; } size++; }
    }
    nz = size;
    size = 0;
    for (int i = 0; i < nz; i++)
        if (in_dom(dom, z[i])) { if (i != size) { cplx t = z[i]; z[i] = z[size]; z[size] = t; } size++; }
    nz = size;
    if (nz <= 1) { if (nevals) *nevals = 0; return 0; }
    cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
    cplx* b = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
    int deg = nexpsup - 1;
    cplx poly[16] = {0};
    if (nexpsup > 0) {
        int ns = 6 * nexpsup, np = deg + 1;
        double* hz = (double*)malloc(sizeof(double) * 2 * ns);
        orc_halton_points(dom, ns, hz);
        cplx* am = (cplx*)calloc((size_t)ns * np, sizeof(cplx));
        cplx* bv = (cplx*)calloc((size_t)ns, sizeof(cplx));
        for (int i = 0; i < ns; i++) {
            cplx zi = ld2(hz + 2 * i), zp = 1.;
            for (int j = 0; j < np; j++) { am[i + j * ns] = zp; zp *= zi; }
            bv[i] = dlogf(d, n, pos, m, zi, use_lapack, a, b, ipiv);
            ne++;
        }
        cleast_squares(ns, np, am, bv, use_lapack);
        for (int j = 0; j < np; j++) poly[j] = bv[j];
        free(hz); free(am); free(bv);
    }
    int* flag = (int*)calloc((size_t)nz, sizeof(int));
    for (int s = 0; s < maxit; s++) {
        for (int i = 0; i < nz; i++) {
            if (flag[i] != 0) continue;
            cplx pv = 0.;
            if (deg >= 0) { pv = poly[deg]; for (int j = deg - 1; j >= 0; j--) pv = pv * z[i] + poly[j]; }
            cplx inv = dlogf(d, n, pos, m, z[i], use_lapack, a, b, ipiv) - pv;
            ne++;
            for (int j = 0; j < nz; j++) if (j != i) inv -= 1. / (z[i] - z[j]);
            cplx dz = 1. / inv, zn = z[i] - dz;
            if (!in_dom(dom, zn)) flag[i] = -1;
            else if (cabs(dz) < toler * cabs(z[i])) flag[i] = 1;
            else z[i] = zn;
        }
        int done = 1;
        for (int i = 0; i < nz; i++) if (flag[i] == 0) { done = 0; break; }
        if (done) break;
    }
    /* filter_cvector (complex_vector_util.c:163), sort by Re (root_finder.c:575) */
    size = 0;
    for (int i = 0; i < nz; i++)
        if (flag[i] == 1) { if (i != size) { cplx t = z[i]; z[i] = z[size]; z[size] = t; } size++; }
    qsort(z, (size_t)size, sizeof(cplx), cmp_re);
    free(flag); free(a); free(b); free(ipiv);
    if (nevals) *nevals = ne;
    return size;
}

/* Wavefunction (src/core/ms_core.c:596-649 for one seed): a = M^-1 phi with
 * phi_i = exp(i k x_i) (incident_wave_util.c:73-82), psi(r) = phi(r) +
 * sum_i a_i G(k,|r-x_i|) (incident_wave_util.c:87-96) on the pixel grid of
 * get_pos_wfun (wave_function_util.c:76-81): row-major from (xmin, ymax).
 * dom = {xmin, xmax, ymin, ymax}; psi is nx*ny complex. */
int orc_wavefunction(int d, int n, const double* pos, const orc_model* m, const double* kk, int nx, int ny,
                     const double* dom, double* amp, double* psi, int nthreads, int use_lapack) {
    cplx k = ld2(kk);
    cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
    cplx* ph = (cplx*)amp;
    for (int i = 0; i < n; i++) ph[i] = cexp(I * k * pos[i * d]);
    build_m(d, n, pos, m, k, a);
    int info = orc_solve(n, (double*)a, (double*)ph, use_lapack);
    free(a);
    orc_psi_grid(d, n, pos, kk, nx, ny, dom, amp, psi, nthreads);
    return info;
}

/* eval_total_wave (incident_wave_util.c:87-96) at every pixel of the grid
 * (get_pos_wfun, wave_function_util.c:76-81) for given amplitudes amp */
void orc_psi_grid(int d, int n, const double* pos, const double* kk, int nx, int ny, const double* dom,
                  const double* amp, double* psi, int nthreads) {
    cplx k = ld2(kk);
    const cplx* ph = (const cplx*)amp;
    double dx = (dom[1] - dom[0]) / (nx - 1), dy = (dom[3] - dom[2]) / (ny - 1);
#pragma omp parallel for schedule(static, 1) num_threads(nthreads)
    for (int l = 0; l < nx * ny; l++) {
        double r[8] = {0};
        r[0] = dom[0] + (l % nx) * dx;
        r[1] = dom[3] - (l / nx) * dy;
        cplx s = 0.;
        for (int i = 0; i < n; i++) s += ph[i] * free_green(d, k, dist(d, pos + i * d, r));
        st2(psi + 2 * l, s + cexp(I * k * r[0]));
    }
}
