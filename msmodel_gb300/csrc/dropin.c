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
    return CMPLX(out[0], out[1]);
}

msgpu_dcomplex dk_log_det_ms(msgpu_ref_medium* med, msgpu_dcomplex k) {
    msgpu_medium m = to_medium(med);
    double kk[2] = {creal(k), cimag(k)}, out[2];
    int st = 0;
    int e = msgpu_dk_log_det_batch(1, &m, 1, NULL, kk, out, &st, MSGPU_FP64);
    if (e) fail("dk_log_det_ms", e);
    if (st & MSGPU_S_SINGULAR) printf("[LAPACK] Element U(i,i) is exactly zero, the inverse matrix will be singular.\n");
    return CMPLX(out[0], out[1]);
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
            msgpu_dcomplex t = CMPLX(out[2 * it], out[2 * it + 1]);
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

static double seconds_since(const struct timespec* t0) {
    struct timespec t1;
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (t1.tv_sec - t0->tv_sec) + 1e-9 * (t1.tv_nsec - t0->tv_nsec);
}

void run_wave_function_omp(msgpu_ref_medium* med, msgpu_ref_wfun* wf, int nthread) {
    (void)nthread;
    if (med->d == 1)  /* the reference's own warning, ms_core.c:597-598 */
        printf("[WARN] The wavefunction in %dD cannot be computed in the same way as in other dimensions. "
               "This may lead to strange results...\n", med->d);
    if (wf->iwave->source != 0) {
        printf("[ERROR] run_wave_function_omp: libmsgpu builds the plane incident wave only.\n");
        return;
    }
    struct timespec t0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int d = med->d, n = med->n, ns = wf->nseed, np = wf->nx * wf->ny;
    if (ns < 1 || np < 1) return;
    msgpu_model mdl = to_model(med->scmodel);
    msgpu_medium* media = (msgpu_medium*)calloc((size_t)ns, sizeof(msgpu_medium));
    double* pos = (double*)malloc(sizeof(double) * (size_t)ns * n * d);
    double* f = (double*)malloc(sizeof(double) * (size_t)np);
    double* g = (double*)malloc(sizeof(double) * (size_t)np);
    for (int s = 0; s < ns; s++) {
        double* p = pos + (size_t)s * n * d;
        int e = msgpu_fill_medium(d, n, med->shape, med->ratio, wf->iseed + (uint64_t)s, p);
        if (e) fail("run_wave_function_omp: fill_medium", e);
        media[s].d = d;
        media[s].n = n;
        media[s].pos = p;
        media[s].model = mdl;
    }
    const double k[2] = {creal(wf->iwave->k), cimag(wf->iwave->k)};
    const double dom[4] = {wf->dom->xmin, wf->dom->xmax, wf->dom->ymin, wf->dom->ymax};
    int st = msgpu_wave_function(ns, media, k, wf->nx, wf->ny, dom, f, g, NULL, NULL, MSGPU_MIXED);
    if (st < 0) fail("run_wave_function_omp", st);
    if (st & (MSGPU_S_SINGULAR | MSGPU_S_NONFINITE))
        printf("[WARN] run_wave_function_omp: a singular or non-finite solve reached the averages (status %d).\n", st);
    for (int l = 0; l < np; l++) {  /* (entry + sum over seeds)/nseed, as the sum and divide_wfun */
        wf->function[l] = wf->function[l] / ns + f[l];
        wf->density[l] = wf->density[l] / ns + g[l];
    }
    memcpy(med->pos, pos + (size_t)(ns - 1) * n * d, sizeof(double) * (size_t)n * d);
    wf->realtime = seconds_since(&t0);
    free(media); free(pos); free(f); free(g);
}

/* The roots of one realisation: every step's function values in one batched
 * GPU job; method 0 Aberth (find_eigenstates_serial_1), 1/2 Muller on the
 * smallest eigenvalue or on 1/tr M^-1 (find_eigenstates_serial_2/3). */
static void find_roots(int method, msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot) {
    struct timespec t0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int nz = *nroot;
    if (nz < 1) {
        eigls->realtime = 0.0;
        return;
    }
    msgpu_medium m = to_medium(eigls->med);
    const double dom[4] = {eigls->dom->xmin, eigls->dom->xmax, eigls->dom->ymin, eigls->dom->ymax};
    double* z0 = (double*)malloc(sizeof(double) * 2 * (size_t)nz);
    double* roots = (double*)malloc(sizeof(double) * 2 * (size_t)nz);
    for (int i = 0; i < nz; i++) {
        z0[2 * i] = creal(kroot[i]);
        z0[2 * i + 1] = cimag(kroot[i]);
    }
    int nr = 0, e;
    if (method == 0)  /* nexpsup = 4, as find_eigenstates_serial_1 passes it (ms_core.c:324) */
        e = msgpu_solve_aberth_batch(1, &m, dom, nz, z0, 4, eigls->maxit, eigls->toler, MSGPU_FP64, roots, &nr, NULL);
    else
        e = msgpu_find_roots_muller_batch(method, 1, &m, dom, nz, z0, eigls->maxit, eigls->toler, MSGPU_FP64, roots,
                                          &nr, NULL);
    if (e) fail(method == 0 ? "find_eigenstates_serial_1" : method == 1 ? "find_eigenstates_serial_2"
                                                                        : "find_eigenstates_serial_3", e);
    for (int i = 0; i < nr; i++) kroot[i] = CMPLX(roots[2 * i], roots[2 * i + 1]);
    *nroot = nr;
    if (method != 0)  /* the split into duplicates and failures is not kept */
        printf("[INFO] Found %d/%d valid roots, %d duplicates or failed.\n", nr, eigls->ntarget, nz - nr);
    eigls->realtime = seconds_since(&t0);
    free(z0); free(roots);
}

void find_eigenstates_serial_1(msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot) {
    find_roots(0, eigls, nroot, kroot);
}

void find_eigenstates_serial_2(msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot) {
    find_roots(1, eigls, nroot, kroot);
}

void find_eigenstates_serial_3(msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot) {
    find_roots(2, eigls, nroot, kroot);
}

extern void alloc_eigenstate_list(msgpu_ref_eigls* eigls, int nstate) __attribute__((weak));
extern void check_eigenstate_list(msgpu_ref_eigls* eigls) __attribute__((weak));

void compute_eigenstates(msgpu_ref_eigls* eigls, int nroot, msgpu_dcomplex* kroot, int maxit, double toler, int verb) {
    (void)verb;
    if (!alloc_eigenstate_list || !check_eigenstate_list) {
        printf("[ERROR] compute_eigenstates: the reference's eigenstate list functions are not linked in.\n");
        return;
    }
    if (maxit != 50 || toler != 1e-10) {
        printf("[ERROR] compute_eigenstates: libmsgpu runs the inverse iteration with maxit=50, toler=1e-10 only "
               "(got maxit=%d, toler=%g).\n", maxit, toler);
        return;
    }
    alloc_eigenstate_list(eigls, nroot);
    const int n = eigls->med->n, ns = eigls->nstate;
    printf("[EXEC] Computing %d states ... ", ns);
    fflush(stdout);
    if (ns > 0) {
        msgpu_medium m = to_medium(eigls->med);
        double* ks = (double*)malloc(sizeof(double) * 2 * (size_t)ns);
        double* lam = (double*)malloc(sizeof(double) * 2 * (size_t)ns);
        double* vec = (double*)malloc(sizeof(double) * 2 * (size_t)ns * n);
        int* st = (int*)calloc((size_t)ns, sizeof(int));
        for (int i = 0; i < ns; i++) {
            ks[2 * i] = creal(kroot[i]);
            ks[2 * i + 1] = cimag(kroot[i]);
        }
        int e = msgpu_inverse_iteration_batch(1, &m, ns, NULL, ks, lam, vec, st, MSGPU_FP64);
        if (e) fail("compute_eigenstates", e);
        for (int i = 0; i < ns; i++) {
            msgpu_ref_eigenstate* es = eigls->eigtab[i];
            es->kroot = kroot[i];
            es->mu = CMPLX(lam[2 * i], lam[2 * i + 1]);
            memcpy(es->eigv, vec + 2 * (size_t)i * n, sizeof(double) * 2 * (size_t)n);
            if (st[i] & MSGPU_S_SINGULAR)  /* inverse_iteration's warning, ms_matrix_util.c:284 */
                printf("[LAPACK] Element U(i,i) is exactly zero, the inverse power iteration will fail.\n");
        }
        free(ks); free(lam); free(vec); free(st);
    }
    printf("Done\n");
    check_eigenstate_list(eigls);
}

extern void store_data_wfcut(msgpu_ref_wfcut* wfcut, double* re, double* im, double* den) __attribute__((weak));

void run_wave_function_cut_omp(msgpu_ref_medium* med, msgpu_ref_wfcut* wc, int nthread) {
    (void)nthread;
    if (!store_data_wfcut) {
        printf("[ERROR] run_wave_function_cut_omp: the reference's store_data_wfcut is not linked in.\n");
        return;
    }
    if (wc->iwave->source != 0) {
        printf("[ERROR] run_wave_function_cut_omp: libmsgpu builds the plane incident wave only.\n");
        return;
    }
    struct timespec t0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int d = med->d, n = med->n, ns = wc->nseed, nb = wc->nbin;
    if (ns < 1 || nb < 2) return;
    msgpu_model mdl = to_model(med->scmodel);
    msgpu_medium* media = (msgpu_medium*)calloc((size_t)ns, sizeof(msgpu_medium));
    double* pos = (double*)malloc(sizeof(double) * (size_t)ns * n * d);
    double* psi = (double*)malloc(sizeof(double) * 2 * (size_t)ns * nb);
    double* re = (double*)malloc(sizeof(double) * (size_t)ns * nb);
    double* im = (double*)malloc(sizeof(double) * (size_t)ns * nb);
    double* den = (double*)malloc(sizeof(double) * (size_t)ns * nb);
    for (int s = 0; s < ns; s++) {
        double* p = pos + (size_t)s * n * d;
        int e = msgpu_fill_medium(d, n, med->shape, med->ratio, wc->iseed + (uint64_t)s, p);
        if (e) fail("run_wave_function_cut_omp: fill_medium", e);
        media[s].d = d;
        media[s].n = n;
        media[s].pos = p;
        media[s].model = mdl;
    }
    const double k[2] = {creal(wc->iwave->k), cimag(wc->iwave->k)};
    int st = msgpu_wave_cut(ns, media, k, nb, wc->xmin, wc->xmax, psi, NULL, MSGPU_MIXED);
    if (st < 0) fail("run_wave_function_cut_omp", st);
    if (st & (MSGPU_S_SINGULAR | MSGPU_S_NONFINITE))
        printf("[WARN] run_wave_function_cut_omp: a singular or non-finite solve reached the samples (status %d).\n",
               st);
    for (int s = 0; s < ns; s++)  /* bin-major samples, [s + i*nseed] (ms_core.c:690-692) */
        for (int i = 0; i < nb; i++) {
            const double a = psi[2 * ((size_t)s * nb + i)], b = psi[2 * ((size_t)s * nb + i) + 1];
            re[s + (size_t)i * ns] = a;
            im[s + (size_t)i * ns] = b;
            den[s + (size_t)i * ns] = a * a + b * b;
        }
    store_data_wfcut(wc, re, im, den);
    wc->realtime = seconds_since(&t0);
    free(media); free(pos); free(psi); free(re); free(im); free(den);
}

static int cmp_double(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* quantile (real_vector_util.c:121-134) of n sorted samples: linear
 * interpolation at the continuous index (n-1) q */
static double quantile_sorted(int n, const double* x, double q) {
    if (n <= 0) return NAN;
    if (n == 1 || q <= 0.) return x[0];
    if (q >= 1.) return x[n - 1];
    const double idx = (n - 1) * q;
    const int i = (int)floor(idx);
    return x[i] + (idx - i) * (x[i + 1] - x[i]);
}

void run_differential_cross_section_omp(msgpu_ref_medium* med, msgpu_ref_dcs* dcs, int nthread) {
    (void)nthread;
    if (med->d == 1)  /* the reference's own warning, ms_core.c:527-528 */
        printf("[WARN] The differential cross section in %dD cannot be computed in the same way as in other "
               "dimensions. This may lead to strange results...\n", med->d);
    struct timespec t0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    const int d = med->d, n = med->n, ns = dcs->nseed, nb = dcs->nbin;
    if (ns < 1 || nb < 2) return;
    msgpu_model mdl = to_model(med->scmodel);
    msgpu_medium* media = (msgpu_medium*)calloc((size_t)ns, sizeof(msgpu_medium));
    double* pos = (double*)malloc(sizeof(double) * (size_t)ns * n * d);
    double* smp = (double*)malloc(sizeof(double) * (size_t)ns * nb);
    for (int s = 0; s < ns; s++) {
        double* p = pos + (size_t)s * n * d;
        int e = msgpu_fill_medium(d, n, med->shape, med->ratio, dcs->iseed + (uint64_t)s, p);
        if (e) fail("run_differential_cross_section_omp: fill_medium", e);
        media[s].d = d;
        media[s].n = n;
        media[s].pos = p;
        media[s].model = mdl;
    }
    int st = msgpu_diff_cross_section(ns, media, dcs->k, nb, dcs->thmin, dcs->thmax, smp, MSGPU_MIXED);
    if (st < 0) fail("run_differential_cross_section_omp", st);
    if (st & (MSGPU_S_SINGULAR | MSGPU_S_NONFINITE))
        printf("[WARN] run_differential_cross_section_omp: a singular or non-finite solve reached the samples "
               "(status %d).\n", st);
    /* ms_core.c:572-583: sample curves of the first nc seeds (at most nseed of them:
     * the reference's loop reads past its samples beyond that), then per bin the
     * sorted samples' quantiles and mean */
    for (int s = 0; s < dcs->nc && s < ns; s++)
        for (int i = 0; i < nb; i++) dcs->curve[s + i * dcs->nc] = smp[s + (size_t)i * ns];
    for (int i = 0; i < nb; i++) {
        double* x = smp + (size_t)i * ns;
        qsort(x, (size_t)ns, sizeof(double), cmp_double);
        for (int q = 0; q < dcs->nq; q++)
            dcs->data[q + i * dcs->nq] = quantile_sorted(ns, x, ((double)q) / (dcs->nq - 1));
        double sum = 0.;
        for (int s = 0; s < ns; s++) sum += x[s];
        dcs->mean[i] = sum / ns;
    }
    dcs->realtime = seconds_since(&t0);
    free(media); free(pos); free(smp);
}
