/* Calls the eigenstate and wavefunction drop-ins (find_eigenstates_serial_1/2/3,
 * compute_eigenstates, run_wave_function_omp, run_wave_function_cut_omp,
 * run_differential_cross_section_omp) the way the reference's
 * run_eigenstate_list_serial and ms_core_main call them, on cases read from
 * standard input, and prints the results for tests/test_gpu_dropin.py.
 *
 *   roots <method 0|1|2> d n seed maxit toler nz xmin xmax ymin ymax z0re z0im ...
 *   eig d n seed nk kre kim ...
 *   wave d n iseed nseed kre kim nx ny xmin xmax ymin ymax
 *   cut d n iseed nseed kre kim nbin xmin xmax
 *   dcs d n iseed nseed k nbin thmin thmax nq nc
 */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "msgpu.h"
#include "msgpu_dropin.h"

/* stand in for the reference's alloc_eigenstate_list and check_eigenstate_list
 * (eigenstate_list_util.c:61,130), which the drop-in compute_eigenstates calls */
void alloc_eigenstate_list(msgpu_ref_eigls* e, int nstate) {
    e->nstate = nstate;
    e->eigtab = (msgpu_ref_eigenstate**)calloc((size_t)nstate, sizeof(msgpu_ref_eigenstate*));
    for (int i = 0; i < nstate; i++) {
        e->eigtab[i] = (msgpu_ref_eigenstate*)calloc(1, sizeof(msgpu_ref_eigenstate));
        e->eigtab[i]->eigv = (msgpu_dcomplex*)calloc((size_t)e->med->n, sizeof(msgpu_dcomplex));
    }
}

void check_eigenstate_list(msgpu_ref_eigls* e) {
    printf("checked %d\n", e->nstate);
}

/* stands in for the reference's store_data_wfcut (wave_function_cut_util.c:92),
 * which the drop-in run_wave_function_cut_omp calls: prints the bin-major samples */
void store_data_wfcut(msgpu_ref_wfcut* wc, double* re, double* im, double* den) {
    for (int i = 0; i < wc->nbin; i++)
        for (int s = 0; s < wc->nseed; s++) {
            const size_t o = (size_t)s + (size_t)i * wc->nseed;
            printf("cut %d %d %.17g %.17g %.17g\n", s, i, re[o], im[o], den[o]);
        }
}

static msgpu_ref_scmodel sm;
static double sm_p[2];

static msgpu_ref_medium make_medium(int d, int n, unsigned long seed) {
    sm.type = MSGPU_MAXIMUM;
    sm.np = 0;
    sm.p = sm_p;
    msgpu_ref_medium med;
    memset(&med, 0, sizeof(med));
    med.d = d;
    med.n = n;
    med.ntot = n * d;
    med.shape = MSGPU_BALL;
    med.ratio = 1.0;
    med.scmodel = &sm;
    med.pos = (double*)malloc(sizeof(double) * (size_t)n * d);
    msgpu_fill_medium(d, n, MSGPU_BALL, 1.0, seed, med.pos);
    return med;
}

int main(void) {
    char cmd[16];
    while (scanf("%15s", cmd) == 1) {
        if (!strcmp(cmd, "roots")) {
            int method, d, n, maxit, nz;
            unsigned long seed;
            double toler;
            msgpu_ref_domain dom;
            if (scanf("%d %d %d %lu %d %lf %d %lf %lf %lf %lf", &method, &d, &n, &seed, &maxit, &toler, &nz, &dom.xmin,
                      &dom.xmax, &dom.ymin, &dom.ymax) != 11)
                return 2;
            msgpu_dcomplex* z = (msgpu_dcomplex*)calloc((size_t)nz, sizeof(msgpu_dcomplex));
            for (int i = 0; i < nz; i++) {
                double re, im;
                if (scanf("%lf %lf", &re, &im) != 2) return 2;
                z[i] = re + I * im;
            }
            msgpu_ref_medium med = make_medium(d, n, seed);
            msgpu_ref_eigls e;
            memset(&e, 0, sizeof(e));
            e.med = &med;
            e.seed = seed;
            e.method = method;
            e.ntarget = nz;
            e.dom = &dom;
            e.maxit = maxit;
            e.toler = toler;
            int nr = nz;
            if (method == 0) find_eigenstates_serial_1(&e, &nr, z);
            else if (method == 1) find_eigenstates_serial_2(&e, &nr, z);
            else find_eigenstates_serial_3(&e, &nr, z);
            printf("nroot %d %d %.6g\n", method, nr, e.realtime);
            for (int i = 0; i < nr; i++) printf("root %d %d %.17g %.17g\n", method, i, creal(z[i]), cimag(z[i]));
            free(z);
            free(med.pos);
        } else if (!strcmp(cmd, "eig")) {
            int d, n, nk;
            unsigned long seed;
            if (scanf("%d %d %lu %d", &d, &n, &seed, &nk) != 4) return 2;
            msgpu_dcomplex* k = (msgpu_dcomplex*)calloc((size_t)nk, sizeof(msgpu_dcomplex));
            for (int i = 0; i < nk; i++) {
                double re, im;
                if (scanf("%lf %lf", &re, &im) != 2) return 2;
                k[i] = re + I * im;
            }
            msgpu_ref_medium med = make_medium(d, n, seed);
            msgpu_ref_eigls e;
            memset(&e, 0, sizeof(e));
            e.med = &med;
            e.ntarget = nk;
            compute_eigenstates(&e, nk, k, 50, 1e-10, 0);
            for (int i = 0; i < e.nstate; i++) {
                msgpu_ref_eigenstate* s = e.eigtab[i];
                printf("state %d %.17g %.17g %.17g %.17g\n", i, creal(s->kroot), cimag(s->kroot), creal(s->mu),
                       cimag(s->mu));
                for (int j = 0; j < n; j++) printf("vec %d %d %.17g %.17g\n", i, j, creal(s->eigv[j]), cimag(s->eigv[j]));
                free(s->eigv);
                free(s);
            }
            free(e.eigtab);
            free(k);
            free(med.pos);
        } else if (!strcmp(cmd, "wave")) {
            int d, n, nseed, nx, ny;
            unsigned long iseed;
            double kre, kim;
            msgpu_ref_domain dom;
            if (scanf("%d %d %lu %d %lf %lf %d %d %lf %lf %lf %lf", &d, &n, &iseed, &nseed, &kre, &kim, &nx, &ny,
                      &dom.xmin, &dom.xmax, &dom.ymin, &dom.ymax) != 12)
                return 2;
            msgpu_ref_medium med = make_medium(d, n, 1);
            msgpu_ref_iwave iw;
            memset(&iw, 0, sizeof(iw));
            iw.source = 0;
            iw.k = kre + I * kim;
            msgpu_ref_wfun wf;
            memset(&wf, 0, sizeof(wf));
            wf.nseed = nseed;
            wf.iseed = iseed;
            wf.iwave = &iw;
            wf.nx = nx;
            wf.ny = ny;
            wf.dom = &dom;
            wf.dx = (dom.xmax - dom.xmin) / (nx - 1);
            wf.dy = (dom.ymax - dom.ymin) / (ny - 1);
            wf.function = (double*)calloc((size_t)nx * ny, sizeof(double));
            wf.density = (double*)calloc((size_t)nx * ny, sizeof(double));
            run_wave_function_omp(&med, &wf, 4);
            for (int l = 0; l < nx * ny; l++) printf("wave %d %.17g %.17g\n", l, wf.function[l], wf.density[l]);
            printf("wave_pos0 %.17g %.17g\n", med.pos[0], med.pos[1]);
            printf("wave_realtime %.6g\n", wf.realtime);
            free(wf.function);
            free(wf.density);
            free(med.pos);
        } else if (!strcmp(cmd, "cut")) {
            int d, n, nseed, nbin;
            unsigned long iseed;
            double kre, kim, xmin, xmax;
            if (scanf("%d %d %lu %d %lf %lf %d %lf %lf", &d, &n, &iseed, &nseed, &kre, &kim, &nbin, &xmin, &xmax) != 9)
                return 2;
            msgpu_ref_medium med = make_medium(d, n, 7);
            const double p0 = med.pos[0];
            msgpu_ref_iwave iw;
            memset(&iw, 0, sizeof(iw));
            iw.k = kre + I * kim;
            msgpu_ref_wfcut wc;
            memset(&wc, 0, sizeof(wc));
            wc.nseed = nseed;
            wc.iseed = iseed;
            wc.iwave = &iw;
            wc.nbin = nbin;
            wc.xmin = xmin;
            wc.xmax = xmax;
            wc.dx = (xmax - xmin) / (nbin - 1);
            wc.ntot = 3 * nbin;
            run_wave_function_cut_omp(&med, &wc, 4);
            printf("cut_med_kept %d\n", med.pos[0] == p0);
            printf("cut_realtime %.6g\n", wc.realtime);
            free(med.pos);
        } else if (!strcmp(cmd, "dcs")) {
            int d, n, nseed, nbin, nq, nc;
            unsigned long iseed;
            double k, thmin, thmax;
            if (scanf("%d %d %lu %d %lf %d %lf %lf %d %d", &d, &n, &iseed, &nseed, &k, &nbin, &thmin, &thmax, &nq,
                      &nc) != 10)
                return 2;
            msgpu_ref_medium med = make_medium(d, n, 7);
            msgpu_ref_dcs dc;
            memset(&dc, 0, sizeof(dc));
            dc.nseed = nseed;
            dc.iseed = iseed;
            dc.k = k;
            dc.thmin = thmin;
            dc.thmax = thmax;
            dc.nbin = nbin;
            dc.nq = nq;
            dc.ntot = nbin * nq;
            dc.nc = nc;
            dc.data = (double*)calloc((size_t)nbin * nq, sizeof(double));
            dc.mean = (double*)calloc((size_t)nbin, sizeof(double));
            dc.curve = (double*)calloc((size_t)nbin * nc, sizeof(double));
            run_differential_cross_section_omp(&med, &dc, 4);
            for (int l = 0; l < nbin * nq; l++) printf("dcs_data %d %d %.17g\n", d, l, dc.data[l]);
            for (int l = 0; l < nbin; l++) printf("dcs_mean %d %d %.17g\n", d, l, dc.mean[l]);
            for (int l = 0; l < nbin * nc; l++) printf("dcs_curve %d %d %.17g\n", d, l, dc.curve[l]);
            free(dc.data);
            free(dc.mean);
            free(dc.curve);
            free(med.pos);
        } else {
            return 2;
        }
        fflush(stdout);
    }
    return 0;
}
