/*
 * ref_driver.c -- plain-pointer entry points over the reference MSModel
 * sources (compiled unmodified from src/core into oracle/_ref).  Used only to
 * pin the oracle restatement (msoracle.c) to the reference itself; test
 * infrastructure, never part of the product.  Complex values are double[2].
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <complex.h>
#include <math.h>
#include "dcomplex_type.h"
#include "medium_type.h"
#include "medium_util.h"
#include "green_bessel.h"
#include "ms_matrix_util.h"
#include "root_finder.h"
#include "complex_vector_util.h"
#include "real_vector_util.h"
#include "complex_data_type.h"
#include "complex_data_util.h"
#include "scattering_model_util.h"
#include "chistogram_type.h"
#include "chistogram_util.h"
#include "color_rule_util.h"
#include "imag_mu_histogram_type.h"
#include "imag_mu_histogram_util.h"
#include "wave_function_type.h"
#include "wave_function_util.h"
#include "incident_wave_util.h"
#include "log_cut_type.h"
#include "log_cut_util.h"
#include "wave_function_cut_type.h"
#include "wave_function_cut_util.h"
#include "diff_cross_section_type.h"
#include "diff_cross_section_util.h"
#include "complex_map_type.h"
#include "complex_map_util.h"
#include "complex_cut_type.h"
#include "complex_cut_util.h"
#include "random_function_type.h"
#include "random_function_util.h"
#include "eigenstate_list_type.h"
#include "eigenstate_list_util.h"
#include "eigenstate_util.h"

void zgesv_(int* n, int* nrhs, dcomplex* a, int* lda, int* ipiv, dcomplex* b, int* ldb, int* info);

static void make_medium(Medium* med, int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                        unsigned long seed) {
    ScatteringModel sm;
    init_scmodel(&sm, (ScatteringType)mtype, np, (double*)p);
    init_medium(med, d, n, &sm, (Shape)shape, ratio);
    del_scmodel(&sm);
    fill_medium(med, seed);
}
static void drop_medium(Medium* med) {
    del_scmodel(med->scmodel);
    del_medium(med);
}

void ref_fill(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
              double* pos) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    memcpy(pos, med.pos, sizeof(double) * (size_t)n * d);
    drop_medium(&med);
}

void ref_green(int d, const double* k, double r, double* out) {
    dcomplex g = free_green(d, k[0] + I * k[1], r);
    out[0] = creal(g); out[1] = cimag(g);
}
void ref_dk_green(int d, const double* k, double r, double* out) {
    dcomplex g = dk_free_green(d, k[0] + I * k[1], r);
    out[0] = creal(g); out[1] = cimag(g);
}
void ref_bessel_k(int twonu, const double* z, double* out) {
    dcomplex g = bessel_k(twonu, z[0] + I * z[1]);
    out[0] = creal(g); out[1] = cimag(g);
}

/* build_ms_matrix + tracelog_lu for each k (ms_core.c:124-126 loop body) */
void ref_tracelog(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
                  int nk, const double* ks, double* out) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    dcomplex* a = (dcomplex*)malloc(sizeof(dcomplex) * (size_t)n * n);
    for (int l = 0; l < nk; l++) {
        build_ms_matrix(&med, ks[2 * l] + I * ks[2 * l + 1], a);
        dcomplex t = tracelog_lu(n, a);
        out[2 * l] = creal(t); out[2 * l + 1] = cimag(t);
    }
    free(a);
    drop_medium(&med);
}

void ref_matrix(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
                const double* k, int deriv, double* mat) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    if (deriv) build_dk_ms_matrix(&med, k[0] + I * k[1], (dcomplex*)mat);
    else build_ms_matrix(&med, k[0] + I * k[1], (dcomplex*)mat);
    drop_medium(&med);
}

void ref_dlogf(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
               int nk, const double* ks, double* out) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    for (int l = 0; l < nk; l++) {
        dcomplex t = dk_log_det_ms(&med, ks[2 * l] + I * ks[2 * l + 1]);
        out[2 * l] = creal(t); out[2 * l + 1] = cimag(t);
    }
    drop_medium(&med);
}

double ref_total_cross_section(int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                               unsigned long seed, double k) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    double cs = total_cross_section(&med, k);
    drop_medium(&med);
    return cs;
}

/* find_eigenstates_serial_1 (ms_core.c:320-328): Aberth on dk_log_det_ms */
static Medium* g_med;
static dcomplex g_dlogf(dcomplex k) { return dk_log_det_ms(g_med, k); }
int ref_aberth(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
               const double* dom, int nz, double* z, int nexpsup, int maxit, double toler) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    Domain dm = {dom[0], dom[1], dom[2], dom[3]};
    g_med = &med;
    int nroot = nz;
    solve_aberth(g_dlogf, &dm, &nroot, (dcomplex*)z, nexpsup, maxit, toler, 0);
    drop_medium(&med);
    return nroot;
}

/* run_wave_function_omp body for one seed (ms_core.c:616-640), plane source */
void ref_wavefunction(int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                      unsigned long seed, const double* kk, int nx, int ny, const double* dom, double* amp,
                      double* psi) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    dcomplex k = kk[0] + I * kk[1];
    dcomplex* a = (dcomplex*)malloc(sizeof(dcomplex) * (size_t)n * n);
    dcomplex* v = (dcomplex*)amp;
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
    int nrhs = 1, info;
    for (int i = 0; i < n; i++) v[i] = cexp(I * k * med.pos[i * d]);
    build_ms_matrix(&med, k, a);
    zgesv_(&n, &nrhs, a, &n, ipiv, v, &n, &info);
    double dx = (dom[1] - dom[0]) / (nx - 1), dy = (dom[3] - dom[2]) / (ny - 1);
    double* r = (double*)calloc((size_t)d, sizeof(double));
    for (int l = 0; l < nx * ny; l++) {
        r[0] = dom[0] + (l % nx) * dx;
        r[1] = dom[3] - (l / nx) * dy;
        dcomplex s = 0.;
        for (int i = 0; i < n; i++) {
            double r2 = 0.;
            for (int c = 0; c < d; c++) { double t = med.pos[i * d + c] - r[c]; r2 += t * t; }
            s += v[i] * free_green(d, k, sqrt(r2));
        }
        s += cexp(I * k * r[0]);
        psi[2 * l] = creal(s); psi[2 * l + 1] = cimag(s);
    }
    free(r); free(a); free(ipiv);
    drop_medium(&med);
}

/* run_random_function_omp (ms_core.c:476-519) over the reference's own
 * fill_medium, total_cross_section and dk_log_det_ms: seed g+1 for sample g,
 * the k grid of get_arg_rfun (random_function_util.c:103), each bin sorted by
 * sort_vector (sort_random_function, random_function_util.c:110). */
void ref_random_function(int type, int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                         int nseed, int nbin, double xmin, double xmax, double* data) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, 1);
    for (int g = 0; g < nseed; g++) {
        fill_medium(&med, g + 1);
        for (int i = 0; i < nbin; i++) {
            double k = xmin * exp(i * log(xmax / xmin) / (nbin - 1));
            data[g + i * nseed] = type == 0 ? total_cross_section(&med, k)
                                            : -cimag(dk_log_det_ms(&med, k)) / (2 * k * 3.1415926535897932385);
        }
    }
    for (int i = 0; i < nbin; i++) sort_vector(nseed, data + i * nseed);
    drop_medium(&med);
}

/* save_cdata (complex_data_util.c:21-28) of n values into a new file */
int ref_save_cdata(int n, const double* data, const char* fname) {
    FILE* fp = fopen(fname, "w");
    if (!fp) return -1;
    ComplexData cd;
    memset(&cd, 0, sizeof cd);
    cd.ntot = n;
    cd.data = (dcomplex*)data;
    save_cdata(&cd, fp);
    fclose(fp);
    return 0;
}

/* parse_cdata (complex_data_util.c:35) of a data string back into n values */
void ref_parse_cdata(int n, const char* text, double* data) {
    ComplexData cd;
    memset(&cd, 0, sizeof cd);
    cd.ntot = n;
    cd.data = (dcomplex*)data;
    char* copy = strdup(text);
    parse_cdata(&cd, copy);
    free(copy);
}

/* traceinv (ms_matrix_util.c:319) of M(k) */
void ref_traceinv(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
                  int nk, const double* ks, double* out) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    dcomplex* a = (dcomplex*)malloc(sizeof(dcomplex) * (size_t)n * n);
    for (int l = 0; l < nk; l++) {
        build_ms_matrix(&med, ks[2 * l] + I * ks[2 * l + 1], a);
        dcomplex t = traceinv(n, a);
        out[2 * l] = creal(t); out[2 * l + 1] = cimag(t);
    }
    free(a);
    drop_medium(&med);
}

/* compute_eigenstates' step (ms_core.c:302-308): inverse_iteration of M(k)
 * from the constant unit vector, 50 steps, 1e-10; returns the convergence flag */
int ref_inverse_iteration(int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                          unsigned long seed, const double* k, double* lambda, double* vec) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    dcomplex* a = (dcomplex*)malloc(sizeof(dcomplex) * (size_t)n * n);
    build_ms_matrix(&med, k[0] + I * k[1], a);
    constant_unit_cvector(n, (dcomplex*)vec);
    dcomplex mu;
    int conv = inverse_iteration(n, a, (dcomplex*)vec, &mu, 50, 1e-10, 0);
    lambda[0] = creal(mu); lambda[1] = cimag(mu);
    free(a);
    drop_medium(&med);
    return conv;
}

/* find_eigenstates_serial_2 / _3 (ms_core.c:335-401): Muller on the smallest
 * eigenvalue (method 1; one eigenvector shared by all calls, as the reference)
 * or on 1/traceinv (method 2), then filter_cvector and uniq_cvector(1e-14) */
static int g_n;
static dcomplex *g_mat, *g_vec;
static dcomplex g_mineigval(dcomplex k) {
    dcomplex mu;
    build_ms_matrix(g_med, k, g_mat);
    inverse_iteration(g_n, g_mat, g_vec, &mu, 50, 1e-10, 0);
    return mu;
}
static dcomplex g_invtrinv(dcomplex k) {
    build_ms_matrix(g_med, k, g_mat);
    return 1. / traceinv(g_n, g_mat);
}
int ref_roots_muller(int method, int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                     unsigned long seed, const double* dom, int nz, double* z, int maxit, double toler) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    Domain dm = {dom[0], dom[1], dom[2], dom[3]};
    g_med = &med;
    g_n = n;
    g_mat = (dcomplex*)calloc((size_t)n * n, sizeof(dcomplex));
    g_vec = (dcomplex*)calloc((size_t)n, sizeof(dcomplex));
    constant_unit_cvector(n, g_vec);
    int* conv = (int*)calloc((size_t)nz, sizeof(int));
    dcomplex* kr = (dcomplex*)z;
    for (int i = 0; i < nz; i++) {
        if (method == 1) {
            conv[i] = find_root_muller(g_mineigval, &dm, &kr[i], maxit, toler, 0);
            conv[i] *= (cabs(g_mineigval(kr[i])) < sqrt(toler));
        } else {
            conv[i] = find_root_muller(g_invtrinv, &dm, &kr[i], maxit, toler, 0);
        }
    }
    int nroot = nz;
    filter_cvector(&nroot, kr, conv);
    uniq_cvector(&nroot, kr, 1e-14);
    free(conv); free(g_mat); free(g_vec);
    drop_medium(&med);
    return nroot;
}

/* eigvals (ms_matrix_util.c:147, zgeev_) of M(k) */
void ref_eigvals(int d, int n, int mtype, int np, const double* p, int shape, double ratio, unsigned long seed,
                 const double* k, double* mu) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    dcomplex* a = (dcomplex*)malloc(sizeof(dcomplex) * (size_t)n * n);
    build_ms_matrix(&med, k[0] + I * k[1], a);
    eigvals(n, a, (dcomplex*)mu);
    free(a);
    drop_medium(&med);
}

/* eigvals of the normalized MS matrix N(k) = i - G(k)/I(k,0)
 * (build_normalized_matrix, ms_matrix_util.c:50), the mu-plane task's
 * mtype=normalized */
void ref_eigvals_normalized(int d, int n, int mtype, int np, const double* p, int shape, double ratio,
                            unsigned long seed, const double* k, double* mu) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, seed);
    dcomplex* a = (dcomplex*)malloc(sizeof(dcomplex) * (size_t)n * n);
    build_normalized_matrix(&med, k[0] + I * k[1], a);
    eigvals(n, a, (dcomplex*)mu);
    free(a);
    drop_medium(&med);
}

/* save_chistogram (chistogram_util.c:414): the [muplane] section of a histogram
 * filled by fill_chist from the nz values z, with the given metadata and colour
 * rule argument (parse_colorrule's "<name> <seq|div> <ctr> [rev]"), appended to
 * fname */
void ref_save_chistogram(int nz, const double* z, int normalized_type, const double* k, int nseed, int xbin,
                         int ybin, int mbin, const char* title, const char* color, double realtime,
                         const char* fname) {
    Chistogram ch;
    memset(&ch, 0, sizeof(ch));
    init_chistogram(&ch, normalized_type ? normalized : msmatrix, k[0] + I * k[1], nseed, xbin, ybin, mbin, title);
    char arg[128];
    strncpy(arg, color, sizeof(arg) - 1);
    arg[sizeof(arg) - 1] = '\0';
    parse_colorrule(ch.colrule, arg);
    fill_chist(&ch, nz, (dcomplex*)z);
    ch.realtime = realtime;
    save_chistogram(&ch, fname);
    free(ch.colrule->data);
    del_chistogram(&ch);
}

/* fill_chist (chistogram_util.c:253) of the nz complex values z into a fresh
 * xbin x ybin histogram with an mbin marginal (init_chistogram, :31): data
 * (row-major, top row = ymax), mdata, and info = {xmin, xmax, ymin, ymax, mmin,
 * mmax, Re avg, Im avg, Re sigma, Im sigma, lost} */
void ref_chistogram(int nz, const double* z, int xbin, int ybin, int mbin, double* data, double* mdata,
                    double* info) {
    Chistogram ch;
    memset(&ch, 0, sizeof(ch));  /* domain and marginal range not set up: taken from the values */
    init_chistogram(&ch, msmatrix, 0.0, 1, xbin, ybin, mbin, "");
    const int lost = fill_chist(&ch, nz, (dcomplex*)z);
    memcpy(data, ch.data, sizeof(double) * (size_t)xbin * ybin);
    memcpy(mdata, ch.mdata, sizeof(double) * (size_t)mbin);
    const double v[11] = {ch.dom->xmin, ch.dom->xmax, ch.dom->ymin, ch.dom->ymax, ch.mmin, ch.mmax,
                          creal(ch.avgz), cimag(ch.avgz), creal(ch.sigmaz), cimag(ch.sigmaz), (double)lost};
    memcpy(info, v, sizeof(v));
    del_chistogram(&ch);
}

/* save_wfun (wave_function_util.c:228): the [wavefunction] section of an nx x ny
 * wave function with the given metadata and data, appended to fname */
void ref_save_wfun(int nx, int ny, const double* dom, const double* k, int spherical_source, int nseed,
                   unsigned long iseed, double realtime, const char* color1, const char* color2, const double* fun,
                   const double* den, const char* fname) {
    WaveFunction w;
    memset(&w, 0, sizeof(w));
    Domain dm = {dom[0], dom[1], dom[2], dom[3]};
    IncidentWave iw;
    init_iwave(&iw, spherical_source ? spherical : plane, k[0] + I * k[1]);
    init_wfun(&w, nx, ny, &dm, nseed, iseed, &iw);
    w.realtime = realtime;
    char a1[128], a2[128];
    strncpy(a1, color1, sizeof(a1) - 1);
    a1[sizeof(a1) - 1] = '\0';
    strncpy(a2, color2, sizeof(a2) - 1);
    a2[sizeof(a2) - 1] = '\0';
    parse_colorrule(w.colrule1, a1);
    parse_colorrule(w.colrule2, a2);
    memcpy(w.function, fun, sizeof(double) * (size_t)nx * ny);
    memcpy(w.density, den, sizeof(double) * (size_t)nx * ny);
    save_wfun(&w, fname);
    free(w.colrule1->data);
    free(w.colrule2->data);
    del_wfun(&w);
}

/* run_imag_mu_histogram_omp (ms_core.c:225-282) on one thread, calling the
 * reference's own steps in its order (setup_domain_ihist, free_green_imag,
 * build_ms_matrix, eigvals, tracegtwo, append_list_ihist, normalize_ihist), then
 * save_ihist (imag_mu_histogram_util.c:195) to fname; info = {xmin, xmax, avgx,
 * varx_true, varx_expc, lost} */
void ref_imag_mu(int d, int n, int mtype, int np, const double* p, int shape, double ratio, double k, int nseed,
                 int nbin, const char* title, double realtime, const char* fname, double* data, double* info) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, 1);
    ImagMuHistogram ih;
    memset(&ih, 0, sizeof(ih));
    init_ihist(&ih, nbin, nseed, k, title);
    setup_domain_ihist(&ih, &med);
    ih.avgx = creal(free_green_imag(med.d, ih.k, 0.));
    dcomplex* a = (dcomplex*)calloc((size_t)n * n, sizeof(dcomplex));
    dcomplex* mu = (dcomplex*)calloc((size_t)n, sizeof(dcomplex));
    double varx_true = 0., varx_expc = 0.;
    int lost = 0;
    for (unsigned long s = 1; s <= (unsigned long)nseed; s++) {
        fill_medium(&med, s);
        build_ms_matrix(&med, ih.k, a);
        eigvals(med.n, a, mu);
        varx_expc += 0.25 * tracegtwo(med.n, a);
        for (int i = 0; i < med.n; i++) varx_true += (cimag(mu[i]) - ih.avgx) * (cimag(mu[i]) - ih.avgx);
        lost += append_list_ihist(&ih, med.n, mu);
    }
    ih.varx_true += varx_true;
    ih.varx_expc += varx_expc;
    normalize_ihist(&ih);
    ih.varx_true /= nseed * med.n;
    ih.varx_expc /= ih.nseed;
    ih.realtime = realtime;
    save_ihist(&ih, fname);
    memcpy(data, ih.data, sizeof(double) * (size_t)nbin);
    const double v[6] = {ih.xmin, ih.xmax, ih.avgx, ih.varx_true, ih.varx_expc, (double)lost};
    memcpy(info, v, sizeof(v));
    free(ih.data);
    free(a);
    free(mu);
    drop_medium(&med);
}

/* init_logcut (log_cut_util.c:72): the mesh k[ns] of a log cut; with fname, the
 * [logkcut] section save_logcut (:122) writes for the data given */
void ref_logcut(int ns, double rek, double imkmin, double imkmax, int nseed, const char* title, double realtime,
                const double* data, double* k, const char* fname) {
    LogCut lc;
    memset(&lc, 0, sizeof(lc));
    init_logcut(&lc, ns, rek, imkmin, imkmax, nseed, title);
    memcpy(k, lc.k, sizeof(dcomplex) * (size_t)ns);
    if (fname) {
        memcpy(lc.data, data, sizeof(dcomplex) * (size_t)ns);
        lc.realtime = realtime;
        save_logcut(&lc, fname);
    }
    del_logcut(&lc);
}

/* store_data_wfcut (wave_function_cut_util.c:92-114) on bin-major samples
 * [s + i*nseed] of Re psi, Im psi and |psi|^2: out_*[3*i..3*i+2] = mean and
 * the first and third quartiles of bin i, the reference's own statistics of
 * run_wave_function_cut_omp (ms_core.c:701). */
void ref_wfcut_stats(int nseed, int nbin, const double* re, const double* im, const double* den, double* out_re,
                     double* out_im, double* out_den) {
    WaveFunctionCut wc;
    memset(&wc, 0, sizeof(wc));
    wc.nseed = nseed;
    wc.nbin = nbin;
    wc.ntot = 3 * nbin;
    wc.repsi = out_re;
    wc.impsi = out_im;
    wc.density = out_den;
    const size_t m = (size_t)nseed * nbin;
    double* a = (double*)malloc(sizeof(double) * m);
    double* b = (double*)malloc(sizeof(double) * m);
    double* c = (double*)malloc(sizeof(double) * m);
    memcpy(a, re, sizeof(double) * m);
    memcpy(b, im, sizeof(double) * m);
    memcpy(c, den, sizeof(double) * m);
    store_data_wfcut(&wc, a, b, c);
    free(a); free(b); free(c);
}

/* save_wfcut (wave_function_cut_util.c:211-226): the [wavefunction_cut] section
 * for these statistics (rows [mean, q1/4, q3/4] per bin, 3*nbin each) to fname */
void ref_save_wfcut(int nbin, double xmin, double xmax, const double* k, int spherical_source, int nseed,
                    unsigned long iseed, double realtime, const double* re, const double* im, const double* den,
                    const char* fname) {
    IncidentWave iw;
    init_iwave(&iw, spherical_source ? spherical : plane, k[0] + I * k[1]);
    WaveFunctionCut wc;
    memset(&wc, 0, sizeof(wc));
    init_wfcut(&wc, nbin, xmin, xmax, nseed, iseed, &iw);
    wc.realtime = realtime;
    memcpy(wc.repsi, re, sizeof(double) * 3 * (size_t)nbin);
    memcpy(wc.impsi, im, sizeof(double) * 3 * (size_t)nbin);
    memcpy(wc.density, den, sizeof(double) * 3 * (size_t)nbin);
    save_wfcut(&wc, fname);
    del_wfcut(&wc);
}

/* run_differential_cross_section_omp (ms_core.c:526-594) on one thread with the
 * reference's own steps in its order: per seed iseed + s, build_ms_matrix,
 * build_plane_wave (theta = 0), zgesv_, then per bin get_arg_dcs,
 * build_plane_wave, cdot_product and the prefactor; then the first nc curves,
 * sort_vector, quantile and mean_vector.  samples[s + i*nseed] before the sort;
 * data[q + i*nq], mean[i], curve[s + i*nc]; the [diff_cross_section] section
 * save_diff_cross_section writes (title, realtime given) to fname. */
void ref_diff_cross_section(int d, int n, int mtype, int np, const double* p, int shape, double ratio, double k,
                            int nseed, unsigned long iseed, int nbin, double thmin, double thmax, int nq, int nc,
                            const char* title, double realtime, const char* fname, double* samples, double* data,
                            double* mean, double* curve) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, iseed);
    DiffCrossSection dcs;
    memset(&dcs, 0, sizeof(dcs));
    char tt[80];
    strncpy(tt, title, sizeof(tt) - 1);
    tt[sizeof(tt) - 1] = '\0';
    init_diff_cross_section(&dcs, nseed, iseed, k, nbin, nq, nc, thmin, thmax, tt);
    const double PI_ = 3.1415926535897932385;
    double prefac = pow(dcs.k / (2 * PI_), med.d - 3) / (16 * PI_ * PI_);
    double* smp = (double*)calloc((size_t)nseed * nbin, sizeof(double));
    dcomplex* m = (dcomplex*)calloc((size_t)n * n, sizeof(dcomplex));
    dcomplex* a = (dcomplex*)calloc((size_t)n, sizeof(dcomplex));
    dcomplex* b = (dcomplex*)calloc((size_t)n, sizeof(dcomplex));
    int* ipiv = (int*)calloc((size_t)n, sizeof(int));
    int nrhs = 1, info;
    for (int s = 0; s < nseed; s++) {
        fill_medium(&med, s + dcs.iseed);
        build_ms_matrix(&med, dcs.k, m);
        build_plane_wave(&med, dcs.k, 0., a);
        zgesv_(&n, &nrhs, m, &n, ipiv, a, &n, &info);
        for (int i = 0; i < nbin; i++) {
            double theta = get_arg_dcs(&dcs, i);
            build_plane_wave(&med, dcs.k, theta, b);
            dcomplex atot = cdot_product(n, b, a);
            smp[s + i * nseed] = prefac * (creal(atot) * creal(atot) + cimag(atot) * cimag(atot));
        }
    }
    memcpy(samples, smp, sizeof(double) * (size_t)nseed * nbin);
    for (int s = 0; s < dcs.nc; s++)
        for (int i = 0; i < nbin; i++) dcs.curve[s + i * dcs.nc] = smp[s + i * nseed];
    for (int i = 0; i < nbin; i++) {
        sort_vector(nseed, smp + i * nseed);
        for (int q = 0; q < dcs.nq; q++) dcs.data[q + i * dcs.nq] = quantile(nseed, smp + i * nseed, ((double)q) / (dcs.nq - 1));
        dcs.mean[i] = mean_vector(nseed, smp + i * nseed);
    }
    dcs.realtime = realtime;
    save_diff_cross_section(&dcs, fname);
    memcpy(data, dcs.data, sizeof(double) * (size_t)nbin * nq);
    memcpy(mean, dcs.mean, sizeof(double) * (size_t)nbin);
    memcpy(curve, dcs.curve, sizeof(double) * (size_t)nbin * nc);
    free(smp); free(m); free(a); free(b); free(ipiv);
    del_diff_cross_section(&dcs);
    drop_medium(&med);
}

/* The reference's writers of the [medium], [kcut], [kplane], [random_function]
 * and [eigenstate_list] sections (medium_util.c:420, complex_cut_util.c:106,
 * complex_map_util.c:236, random_function_util.c:178,
 * eigenstate_list_util.c:296) on structs its own init functions set up, with
 * the given data; each appends its section to fname. */
void ref_save_medium(int d, int n, int mtype, int np, const double* p, int shape, double ratio, const char* fname) {
    Medium med;
    make_medium(&med, d, n, mtype, np, p, shape, ratio, 1);
    save_medium(&med, fname);
    drop_medium(&med);
}

void ref_save_kcut(int ns, const double* zmin, const double* zmax, int nseed, const char* title, double realtime,
                   const double* data, const char* fname) {
    ComplexCut cc;
    memset(&cc, 0, sizeof(cc));
    init_complexcut(&cc, ns, zmin[0] + I * zmin[1], zmax[0] + I * zmax[1], nseed, title);
    memcpy(cc.data, data, sizeof(dcomplex) * (size_t)cc.ntot);
    cc.realtime = realtime;
    save_complexcut(&cc, fname);
    del_complexcut(&cc);
}

void ref_save_kplane(int nx, int ny, double xmin, double xmax, double ymin, double ymax, int nseed, const char* title,
                     double realtime, const char* color, const double* data, const char* fname) {
    ComplexMap cm;
    memset(&cm, 0, sizeof(cm));
    init_complexmap(&cm, nx, ny, xmin, xmax, ymin, ymax, nseed, title);
    char a[128];
    strncpy(a, color, sizeof(a) - 1);
    a[sizeof(a) - 1] = '\0';
    parse_colorrule(cm.colrule, a);
    memcpy(cm.data, data, sizeof(dcomplex) * (size_t)cm.ntot);
    cm.realtime = realtime;
    save_complexmap(&cm, fname);
    del_complexmap(&cm);
}

void ref_save_rfun(int type, int nseed, int nbin, double xmin, double xmax, const char* title, double realtime,
                   const double* data, const char* fname) {
    RandomFunction rf;
    memset(&rf, 0, sizeof(rf));
    char t[80];
    strncpy(t, title, sizeof(t) - 1);
    t[sizeof(t) - 1] = '\0';
    init_random_function(&rf, (RandomFunctionType)type, nseed, nbin, xmin, xmax, t);
    memcpy(rf.data, data, sizeof(double) * (size_t)rf.ntot);
    rf.realtime = realtime;
    save_random_function(&rf, fname);
    del_random_function(&rf);
}

void ref_save_eigls(int d, int n, unsigned long seed, int method, int ntarget, const double* dom, int maxit,
                    double toler, int verb, double realtime, int nstate, const double* kroot, const double* mu,
                    const double* eigv, const char* fname) {
    Medium med;
    make_medium(&med, d, n, 3, 0, NULL, 1, 1.0, seed);
    Domain dm = {dom[0], dom[1], dom[2], dom[3]};
    EigenstateList el;
    memset(&el, 0, sizeof(el));
    init_eigenstate_list(&el, &med, seed, (EigenstateMethod)method, ntarget, &dm, maxit, toler, verb);
    alloc_eigenstate_list(&el, nstate);
    for (int i = 0; i < nstate; i++) {
        el.eigtab[i]->kroot = CMPLX(kroot[2 * i], kroot[2 * i + 1]);
        el.eigtab[i]->mu = CMPLX(mu[2 * i], mu[2 * i + 1]);
        memcpy(el.eigtab[i]->eigv, eigv + 2 * (size_t)i * n, sizeof(dcomplex) * (size_t)n);
    }
    el.realtime = realtime;
    save_eigenstate_list(&el, fname);
    del_eigenstate_list(&el);
    drop_medium(&med);
}
