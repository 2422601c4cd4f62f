/* Calls the symbol-compatible drop-ins exactly as the reference's C callers
 * do (double _Complex by value, Medium by pointer) and prints the results
 * for tests/test_gpu_dropin.py to compare with the oracle. */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include "msgpu.h"
#include "msgpu_dropin.h"

static msgpu_dcomplex arg_cut(void* self, int l) {
    (void)self;
    /* a kcut of 4 samples from 0.5-0.05i to 3-0.05i (get_arg_ccut order) */
    int ns = 4, il = l / 3, it = l % 3;
    msgpu_dcomplex zmin = 0.5 - 0.05 * I, zmax = 3.0 - 0.05 * I, dz = (zmax - zmin) / (ns - 1);
    return ((ns - il) * zmin + (il - 1) * zmax) / (ns - 1) + I * dz * (it - 1);
}

/* stands in for the reference's fill_chist (chistogram_util.c:253), which the
 * drop-in run_chistogram_omp calls: prints the eigenvalues it is handed */
int fill_chist(msgpu_ref_chist* chist, int nz, msgpu_dcomplex* z) {
    for (int i = 0; i < nz; i++)
        printf("chist%d %d %.17g %.17g\n", chist->mtype, i, creal(z[i]), cimag(z[i]));
    return 0;
}

/* stand in for the reference's append_list_ihist and normalize_ihist
 * (imag_mu_histogram_util.c:107,139), which the drop-in run_imag_mu_histogram_omp
 * calls: print the eigenvalues they are handed and count the normalisations */
static int n_normalize = 0;
int append_list_ihist(msgpu_ref_ihist* ih, int nz, msgpu_dcomplex* z) {
    for (int i = 0; i < nz; i++) printf("ihist %d %.17g %.17g\n", i, creal(z[i]), cimag(z[i]));
    (void)ih;
    return 0;
}
void normalize_ihist(msgpu_ref_ihist* ih) {
    (void)ih;
    n_normalize++;
}

int main(int argc, char** argv) {
    int d = 3, n = argc > 1 ? atoi(argv[1]) : 80;
    double p[2] = {0.0, 0.0};
    msgpu_ref_scmodel sm = {0};
    sm.type = MSGPU_MAXIMUM;
    sm.np = 0;
    sm.p = p;
    msgpu_ref_medium med = {0};
    med.d = d;
    med.n = n;
    med.ntot = n * d;
    med.shape = MSGPU_BALL;
    med.ratio = 1.0;
    med.scmodel = &sm;
    med.pos = (double*)malloc(sizeof(double) * n * d);
    msgpu_fill_medium(d, n, MSGPU_BALL, 1.0, 1, med.pos);
    msgpu_dcomplex* a = (msgpu_dcomplex*)malloc(sizeof(msgpu_dcomplex) * n * n);
    msgpu_dcomplex k = 1.3 - 0.07 * I;
    build_ms_matrix(&med, k, a);
    printf("M01 %.17g %.17g\n", creal(a[1 * n + 0]), cimag(a[1 * n + 0]));
    msgpu_dcomplex t = tracelog_lu(n, a);
    printf("tracelog %.17g %.17g\n", creal(t), cimag(t));
    msgpu_dcomplex g = dk_log_det_ms(&med, k);
    printf("dlogf %.17g %.17g\n", creal(g), cimag(g));
    printf("sigma %.17g\n", total_cross_section(&med, 1.3));
    msgpu_ref_cdata cd = {0};
    cd.ntot = 3 * (4 + 2);
    cd.nseed = 2;
    cd.data = (msgpu_dcomplex*)calloc(cd.ntot, sizeof(msgpu_dcomplex));
    cd.get_arg = arg_cut;
    run_tracelog_omp(&med, &cd, 4);
    for (int l = 0; l < cd.ntot; l++) printf("cut %d %.17g %.17g\n", l, creal(cd.data[l]), cimag(cd.data[l]));
    /* total cross section, seeds 1..3, 4 log-spaced bins on [0.5, 2.5] */
    msgpu_ref_rfun rf = {0};
    rf.type = 0;
    rf.nseed = 3;
    rf.nbin = 4;
    rf.ntot = rf.nseed * rf.nbin;
    rf.xmin = 0.5;
    rf.xmax = 2.5;
    rf.data = (double*)calloc(rf.ntot, sizeof(double));
    run_random_function_omp(&med, &rf, 4);
    for (int l = 0; l < rf.ntot; l++) printf("rfun %d %.17g\n", l, rf.data[l]);
    /* mu-plane histogram task, seeds 1..2 at k = 1.1, both matrix types */
    for (int mt = 0; mt < 2; mt++) {
        msgpu_ref_chist ch = {0};
        ch.mtype = mt;
        ch.k = 1.1;
        ch.nseed = 2;
        run_chistogram_omp(&med, &ch, 4);
        printf("chist_realtime %d %.17g\n", mt, ch.realtime);
    }
    /* Im mu histogram task, seeds 1..2 at k = 1.1 */
    msgpu_ref_ihist ih = {0};
    ih.k = 1.1;
    ih.nseed = 2;
    ih.nbin = 8;
    run_imag_mu_histogram_omp(&med, &ih, 4);
    printf("ihist_info %.17g %.17g %.17g %.17g %.17g %d %.17g\n", ih.xmin, ih.xmax, ih.avgx, ih.varx_true,
           ih.varx_expc, n_normalize, ih.realtime);
    printf("pos0 %.17g %.17g %.17g\n", med.pos[0], med.pos[1], med.pos[2]);
    free(a); free(med.pos); free(cd.data); free(rf.data);
    return 0;
}
