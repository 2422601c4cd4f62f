/* Calls the task drop-ins in a program that defines none of the reference's
 * histogram, eigenstate-list and cut-statistics functions (their weak
 * references stay unresolved) and with a spherical incident wave: each must
 * print its error and return before any device work, leaving the caller's
 * structs as they were.  Prints one "done <name>" line per call for
 * tests/test_abi.py. */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "msgpu.h"
#include "msgpu_dropin.h"

int main(void) {
    double p[2] = {0.0, 0.0};
    msgpu_ref_scmodel sm;
    memset(&sm, 0, sizeof(sm));
    sm.type = MSGPU_MAXIMUM;
    sm.p = p;
    msgpu_ref_medium med;
    memset(&med, 0, sizeof(med));
    med.d = 3;
    med.n = 8;
    med.ntot = 24;
    med.shape = MSGPU_BALL;
    med.ratio = 1.0;
    med.scmodel = &sm;
    med.pos = (double*)calloc(24, sizeof(double));

    msgpu_ref_chist ch;
    memset(&ch, 0, sizeof(ch));
    ch.nseed = 2;
    run_chistogram_omp(&med, &ch, 1);
    printf("done chist\n");

    msgpu_ref_ihist ih;
    memset(&ih, 0, sizeof(ih));
    ih.nseed = 2;
    ih.k = 1.0;
    run_imag_mu_histogram_omp(&med, &ih, 1);
    printf("done ihist %g\n", ih.avgx);

    msgpu_ref_eigls el;
    memset(&el, 0, sizeof(el));
    el.med = &med;
    msgpu_dcomplex k = 1.0;
    compute_eigenstates(&el, 1, &k, 50, 1e-10, 0);
    printf("done eigls %d\n", el.nstate);

    msgpu_ref_iwave iw;
    memset(&iw, 0, sizeof(iw));
    iw.k = 1.0;
    msgpu_ref_wfcut wc;
    memset(&wc, 0, sizeof(wc));
    wc.nseed = 2;
    wc.nbin = 4;
    wc.iwave = &iw;
    run_wave_function_cut_omp(&med, &wc, 1);
    printf("done wfcut %g\n", wc.realtime);

    iw.source = 1; /* spherical */
    msgpu_ref_domain dom = {-1.0, 1.0, -1.0, 1.0};
    msgpu_ref_wfun wf;
    memset(&wf, 0, sizeof(wf));
    wf.nseed = 2;
    wf.nx = 2;
    wf.ny = 2;
    wf.iwave = &iw;
    wf.dom = &dom;
    run_wave_function_omp(&med, &wf, 1);
    printf("done wfun %g\n", wf.realtime);
    free(med.pos);
    return 0;
}
