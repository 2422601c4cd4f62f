/*
 * dropin.c -- the reference's hot-path symbols over the GPU engine.
 *
 * Compiled as C so that `double _Complex` arguments and return values follow
 * the platform ABI exactly as the reference's callers expect.  Each function
 * keeps its reference counterpart's meaning: matrices are caller-allocated,
 * column-major n*n; LAPACK warnings are printed in the reference's words
 * (src/core/ms_matrix_util.c:188-190, :250-252, :358-360).
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "msgpu.h"
#include "msgpu_dropin.h"

static msgpu_model to_model(const msgpu_ref_scmodel* sm) {
    msgpu_model m;
    memset(&m, 0, sizeof(m));
    m.type = sm->type;
    m.np = sm->np < 2 ? sm->np : 2;
    for (int i = 0; i < m.np; i++) m.p[i] = sm->p[i];
    return m;
}

static msgpu_medium to_medium(const msgpu_ref_medium* med) {
    msgpu_medium m;
    m.d = med->d;
    m.n = med->n;
    m.pos = med->pos;
    m.model = to_model(med->scmodel);
    return m;
}

static void fail(const char* where, int e) {
    fprintf(stderr, "[ERROR] %s: GPU call failed (%d): %s\n", where, e, msgpu_last_error());
    exit(EXIT_FAILURE);
}

void build_ms_matrix(msgpu_ref_medium* med, msgpu_dcomplex k, msgpu_dcomplex* matrix) {
    msgpu_medium m = to_medium(med);
    double kk[2] = {creal(k), cimag(k)};
    int e = msgpu_build_matrix(&m, kk, 0, (double*)matrix);
    if (e) fail("build_ms_matrix", e);
}

void build_dk_ms_matrix(msgpu_ref_medium* med, msgpu_dcomplex k, msgpu_dcomplex* matrix) {
    msgpu_medium m = to_medium(med);
    double kk[2] = {creal(k), cimag(k)};
    int e = msgpu_build_matrix(&m, kk, 1, (double*)matrix);
    if (e) fail("build_dk_ms_matrix", e);
}

/* host arithmetic, as the reference: phi_i = exp(i k (cos t x_i + sin t y_i)) */
void build_plane_wave(msgpu_ref_medium* med, msgpu_dcomplex k, double theta, msgpu_dcomplex* vec) {
    const int d = med->d, n = med->n;
    theta *= 3.1415926535897932385 / 180;
    double ct = cos(theta), st = sin(theta);
    if (d == 1) {
        ct = ct > 0. ? 1. : -1.;
        for (int i = 0; i < n; i++) vec[i] = cexp(I * k * ct * med->pos[i]);
    } else {
        for (int i = 0; i < n; i++) vec[i] = cexp(I * k * (ct * med->pos[i * d] + st * med->pos[i * d + 1]));
    }
}

msgpu_dcomplex tracelog_lu(int n, msgpu_dcomplex* matrix) {
    double out[2];
    int info = 0;
    int e = msgpu_tracelog_matrix(n, (const double*)matrix, out, &info);
    if (e) fail("tracelog_lu", e);
    if (info > 0) printf("[LAPACK] Element U(%d,%d) is exactly zero, the determinant will be singular.\n", info, info);
    return out[0] + I * out[1];
}

msgpu_dcomplex dk_log_det_ms(msgpu_ref_medium* med, msgpu_dcomplex k) {
    msgpu_medium m = to_medium(med);
    double kk[2] = {creal(k), cimag(k)}, out[2];
    int st = 0;
    int e = msgpu_dk_log_det_batch(1, &m, 1, NULL, kk, out, &st, MSGPU_FP64);
    if (e) fail("dk_log_det_ms", e);
    if (st & MSGPU_S_SINGULAR) printf("[LAPACK] Element U(i,i) is exactly zero, the inverse matrix will be singular.\n");
    return out[0] + I * out[1];
}

double total_cross_section(msgpu_ref_medium* med, double k) {
    msgpu_medium m = to_medium(med);
    double kk[2] = {k, 0.0}, out[2];
    int st = 0;
    int e = msgpu_amplitude_batch(1, &m, 1, NULL, kk, out, NULL, &st, MSGPU_FP64);
    if (e) fail("total_cross_section", e);
    if (st & MSGPU_S_SINGULAR) printf("[LAPACK] Element U(i,i) is exactly zero, the solution could not be computed.\n");
    return out[0];
}

void run_tracelog_omp(msgpu_ref_medium* med, msgpu_ref_cdata* cdata, int nthread) {
    (void)nthread;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int d = med->d, n = med->n, nseed = cdata->nseed, ntot = cdata->ntot;
    msgpu_medium* media = (msgpu_medium*)calloc((size_t)nseed, sizeof(msgpu_medium));
    double* pos = (double*)malloc(sizeof(double) * (size_t)nseed * n * d);
    double* ks = (double*)malloc(sizeof(double) * 2 * (size_t)nseed * ntot);
    int* im = (int*)malloc(sizeof(int) * (size_t)nseed * ntot);
    double* out = (double*)malloc(sizeof(double) * 2 * (size_t)nseed * ntot);
    msgpu_model mdl = to_model(med->scmodel);
    for (int s = 0; s < nseed; s++) {
        double* p = pos + (size_t)s * n * d;
        int e = msgpu_fill_medium(d, n, med->shape, med->ratio, (uint64_t)(s + 1), p);
        if (e) fail("run_tracelog_omp: fill_medium", e);
        media[s].d = d;
        media[s].n = n;
        media[s].pos = p;
        media[s].model = mdl;
        for (int l = 0; l < ntot; l++) {
            msgpu_dcomplex k = cdata->get_arg(cdata, l);
            size_t it = (size_t)s * ntot + l;
            ks[2 * it] = creal(k);
            ks[2 * it + 1] = cimag(k);
            im[it] = s;
        }
    }
    int* st = (int*)calloc((size_t)nseed * ntot, sizeof(int));
    int e = msgpu_tracelog_batch(nseed, media, nseed * ntot, im, ks, out, st, MSGPU_FP64);
    if (e) fail("run_tracelog_omp", e);
    /* the reference's tracelog_lu warns once per singular matrix (ms_matrix_util.c:188-190); the
     * pivot index is not kept per item, so the warning names the matrix's point and seed instead */
    for (size_t it = 0; it < (size_t)nseed * ntot; it++)
        if (st[it] & MSGPU_S_SINGULAR)
            printf("[LAPACK] Element U(i,i) is exactly zero, the determinant will be singular (seed %d, point %d).\n",
                   (int)(it / ntot) + 1, (int)(it % ntot));
    free(st);
    /* running average over seeds in seed order (ms_core.c:127) */
    for (int s = 1; s <= nseed; s++)
        for (int l = 0; l < ntot; l++) {
            size_t it = (size_t)(s - 1) * ntot + l;
            msgpu_dcomplex t = out[2 * it] + I * out[2 * it + 1];
            cdata->data[l] = ((s - 1) * cdata->data[l] + t) / s;
        }
    /* leave the medium filled with the last seed, as the reference loop does */
    if (nseed > 0) memcpy(med->pos, pos + (size_t)(nseed - 1) * n * d, sizeof(double) * (size_t)n * d);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    cdata->realtime = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    free(media); free(pos); free(ks); free(im); free(out);
}

/* the reference's binning, resolved in the program the library is linked into */
extern int fill_chist(msgpu_ref_chist* chist, int nz, msgpu_dcomplex* z) __attribute__((weak));

void run_chistogram_omp(msgpu_ref_medium* med, msgpu_ref_chist* chist, int nthread) {
    (void)nthread;
    if (!fill_chist) {
        printf("[ERROR] run_chistogram_omp: fill_chist is not linked in, no histogram computed.\n");
        return;
    }
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int d = med->d, n = med->n, nseed = chist->nseed;
    msgpu_medium* media = (msgpu_medium*)calloc((size_t)nseed, sizeof(msgpu_medium));
    double* pos = (double*)malloc(sizeof(double) * (size_t)nseed * n * d);
    double* ks = (double*)malloc(sizeof(double) * 2 * (size_t)nseed);
    int* im = (int*)malloc(sizeof(int) * (size_t)nseed);
    int* st = (int*)calloc((size_t)nseed, sizeof(int));
    msgpu_dcomplex* mu = (msgpu_dcomplex*)malloc(sizeof(msgpu_dcomplex) * (size_t)nseed * n);
    msgpu_model mdl = to_model(med->scmodel);
    for (int s = 0; s < nseed; s++) {
        double* p = pos + (size_t)s * n * d;
        int e = msgpu_fill_medium(d, n, med->shape, med->ratio, (uint64_t)(s + 1), p);
        if (e) fail("run_chistogram_omp: fill_medium", e);
        media[s].d = d;
        media[s].n = n;
        media[s].pos = p;
        media[s].model = mdl;
        ks[2 * s] = creal(chist->k);
        ks[2 * s + 1] = cimag(chist->k);
        im[s] = s;
    }
    int e = msgpu_eigvals_batch_mtype(chist->mtype == 1 ? MSGPU_MTYPE_NORMALIZED : MSGPU_MTYPE_MSMATRIX, nseed,
                                      media, nseed, im, ks, (double*)mu, st, NULL);
    if (e) fail("run_chistogram_omp", e);
    for (int s = 0; s < nseed; s++)
        if (st[s] & MSGPU_S_NOCONV)  /* eigvals' LAPACK warning, ms_matrix_util.c:158 */
            printf("[LAPACK] The QR algorithm failed to compute all the eigenvalues (seed %d).\n", s + 1);
    const int nmu = nseed * n;
    const int lost = fill_chist(chist, nmu, mu);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    chist->realtime = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    printf("[INFO] Lost eigenvalues: %d/%d (%.2f%%)\n", lost, nmu, 100.0 * lost / nmu);
    free(media); free(pos); free(ks); free(im); free(st); free(mu);
}

extern int append_list_ihist(msgpu_ref_ihist* ihist, int nz, msgpu_dcomplex* z) __attribute__((weak));
extern void normalize_ihist(msgpu_ref_ihist* ihist) __attribute__((weak));

void run_imag_mu_histogram_omp(msgpu_ref_medium* med, msgpu_ref_ihist* ih, int nthread) {
    (void)nthread;
    if (!append_list_ihist || !normalize_ihist) {
        printf("[ERROR] run_imag_mu_histogram_omp: the reference's histogram functions are not linked in.\n");
        return;
    }
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int d = med->d, n = med->n, nseed = ih->nseed;
    msgpu_model mdl = to_model(med->scmodel);
    double kr[2] = {ih->k, 0.0}, r0 = 0.0, iz[2];
    int e = msgpu_eval_special(2, d, &mdl, 1, kr, &r0, iz);
    if (e) fail("run_imag_mu_histogram_omp: free_green_imag", e);
    ih->avgx = iz[0];
    msgpu_medium* media = (msgpu_medium*)calloc((size_t)nseed, sizeof(msgpu_medium));
    double* pos = (double*)malloc(sizeof(double) * (size_t)nseed * n * d);
    double* ks = (double*)malloc(sizeof(double) * 2 * (size_t)nseed);
    int* im = (int*)malloc(sizeof(int) * (size_t)nseed);
    int* st = (int*)calloc((size_t)nseed, sizeof(int));
    double* trg = (double*)malloc(sizeof(double) * (size_t)nseed);
    msgpu_dcomplex* mu = (msgpu_dcomplex*)malloc(sizeof(msgpu_dcomplex) * (size_t)nseed * n);
    for (int s = 0; s < nseed; s++) {
        double* p = pos + (size_t)s * n * d;
        e = msgpu_fill_medium(d, n, med->shape, med->ratio, (uint64_t)(s + 1), p);
        if (e) fail("run_imag_mu_histogram_omp: fill_medium", e);
        media[s].d = d;
        media[s].n = n;
        media[s].pos = p;
        media[s].model = mdl;
        ks[2 * s] = ih->k;
        ks[2 * s + 1] = 0.0;
        im[s] = s;
    }
    e = msgpu_eigvals_batch_mtype(MSGPU_MTYPE_MSMATRIX, nseed, media, nseed, im, ks, (double*)mu, st, trg);
    if (e) fail("run_imag_mu_histogram_omp", e);
    /* setup_domain_ihist: seed 1's smallest positive and largest Im mu, halved and doubled */
    double xmin = cimag(mu[0]), xmax = xmin;
    for (int i = 1; i < n; i++) {
        const double x = cimag(mu[i]);
        if (x < xmin && x > 0.0) xmin = x;
        if (x > xmax) xmax = x;
    }
    ih->xmin = xmin / 2.0;
    ih->xmax = 2.0 * xmax;
    memcpy(med->pos, pos, sizeof(double) * (size_t)n * d);
    double varx_true = 0.0, varx_expc = 0.0;
    int lost = 0;
    for (int s = 0; s < nseed; s++) {
        if (st[s] & MSGPU_S_NOCONV)
            printf("[LAPACK] The QR algorithm failed to compute all the eigenvalues (seed %d).\n", s + 1);
        msgpu_dcomplex* m = mu + (size_t)s * n;
        varx_expc += 0.25 * trg[s];
        for (int i = 0; i < n; i++) varx_true += (cimag(m[i]) - ih->avgx) * (cimag(m[i]) - ih->avgx);
        lost += append_list_ihist(ih, n, m);
    }
    ih->varx_true += varx_true;
    ih->varx_expc += varx_expc;
    normalize_ihist(ih);
    ih->varx_true /= (double)nseed * n;
    ih->varx_expc /= nseed;
    clock_gettime(CLOCK_MONOTONIC, &t1);
    ih->realtime = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    printf("[INFO] Lost eigenvalues: %d/%d (%.2f%%)\n", lost, nseed * n, 100.0 * lost / (nseed * n));
    free(media); free(pos); free(ks); free(im); free(st); free(trg); free(mu);
}

void run_random_function_omp(msgpu_ref_medium* med, msgpu_ref_rfun* rfun, int nthread) {
    (void)nthread;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    msgpu_model mdl = to_model(med->scmodel);
    int e = msgpu_random_function(rfun->type, med->d, med->n, med->shape, med->ratio, &mdl, rfun->nseed, rfun->nbin,
                                  rfun->xmin, rfun->xmax, rfun->data, NULL, MSGPU_FP64);
    if (e) fail("run_random_function_omp", e);
    if (rfun->nseed > 0) {
        e = msgpu_fill_medium(med->d, med->n, med->shape, med->ratio, (uint64_t)rfun->nseed, med->pos);
        if (e) fail("run_random_function_omp: fill_medium", e);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    rfun->realtime = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
}
