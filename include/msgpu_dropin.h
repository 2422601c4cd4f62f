/*
 * msgpu_dropin.h -- symbol-compatible replacements for the reference's own
 * hot-path functions.  libmsgpu.so exports these names with the reference's
 * signatures, so the reference's callers (src/core/ms_core.c, root_finder.c
 * users, the tests) relink against the GPU without source changes.
 *
 * The structs below are layout-identical to the reference types they stand
 * for; only the fields the hot path reads are named meaningfully.
 */
#ifndef MSGPU_DROPIN_H
#define MSGPU_DROPIN_H
#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex msgpu_dcomplex; /* reference dcomplex, src/core/dcomplex_type.h:16 */

/* reference ScatteringModel, src/core/scattering_model_type.h:246-258 */
typedef struct msgpu_ref_scmodel {
    int type;
    int np;
    double* p;
    char dir[50];
    char name[150];
    char param_ascii[150];
    char param_latex[150];
} msgpu_ref_scmodel;

/* reference Medium, src/core/medium_type.h:42-54 */
typedef struct msgpu_ref_medium {
    int d;
    int n;
    int ntot;
    int shape;
    double ratio;
    msgpu_ref_scmodel* scmodel;
    double alpha;
    void* rnd;
    double* pos;
} msgpu_ref_medium;

/* reference ComplexData, src/core/complex_data_type.h:17-24 */
typedef struct msgpu_ref_cdata {
    int ntot;
    int nseed;
    msgpu_dcomplex* data;
    char title[80];
    double realtime;
    msgpu_dcomplex (*get_arg)(void* self, int i);
} msgpu_ref_cdata;

/* reference RandomFunction, src/core/random_function_type.h:22-33 */
typedef struct msgpu_ref_rfun {
    int type; /* 0 = crsec, 1 = dos */
    int nbin;
    int nseed;
    int ntot;
    double xmin;
    double xmax;
    double* data;
    char title[80];
    double realtime;
} msgpu_ref_rfun;

/* reference Chistogram (ComplexHistogram_s), src/core/chistogram_type.h:26-52 */
typedef struct msgpu_ref_chist {
    int mtype; /* MatrixType: 0 msmatrix, 1 normalized */
    int xbin;
    int ybin;
    int ntot;
    void* dom;
    int dom_ok;
    msgpu_dcomplex k;
    int nseed;
    msgpu_dcomplex avgz;
    msgpu_dcomplex sigmaz;
    double* data;
    void* colrule;
    double realtime;
    char title[80];
    int mbin;
    double mmin;
    double mmax;
    double* mdata;
    int mrange_ok;
} msgpu_ref_chist;

/* reference ImagMuHistogram, src/core/imag_mu_histogram_type.h:16-31 */
typedef struct msgpu_ref_ihist {
    int nseed;
    double k;
    int nbin;
    double xmin;
    double xmax;
    double* data;
    double realtime;
    char title[80];
    double avgx;
    double varx_true;
    double varx_expc;
} msgpu_ref_ihist;

/* replaces build_ms_matrix, src/core/ms_matrix_util.c:32 */
void build_ms_matrix(msgpu_ref_medium* med, msgpu_dcomplex k, msgpu_dcomplex* matrix);
/* replaces build_dk_ms_matrix, src/core/ms_matrix_util.c:68 */
void build_dk_ms_matrix(msgpu_ref_medium* med, msgpu_dcomplex k, msgpu_dcomplex* matrix);
/* replaces build_plane_wave, src/core/ms_matrix_util.c:88 (host arithmetic) */
void build_plane_wave(msgpu_ref_medium* med, msgpu_dcomplex k, double theta, msgpu_dcomplex* vec);
/* replaces tracelog_lu, src/core/ms_matrix_util.c:185; `matrix` is left intact */
msgpu_dcomplex tracelog_lu(int n, msgpu_dcomplex* matrix);
/* replaces dk_log_det_ms, src/core/ms_matrix_util.c:242 */
msgpu_dcomplex dk_log_det_ms(msgpu_ref_medium* med, msgpu_dcomplex k);
/* replaces total_cross_section, src/core/ms_matrix_util.c:344 */
double total_cross_section(msgpu_ref_medium* med, double k);
/* replaces run_tracelog_omp, src/core/ms_core.c:96: every (seed, k) of the
 * task in one batched GPU job; the seeds are filled with the reference's
 * generator (seed s = 1..nseed), data[] is the same running average. */
void run_tracelog_omp(msgpu_ref_medium* med, msgpu_ref_cdata* cdata, int nthread);
/* replaces run_random_function_omp, src/core/ms_core.c:476: every (seed, bin)
 * sample in one batched GPU job, bins sorted; the medium is left filled with
 * the last seed, as the reference leaves it */
void run_random_function_omp(msgpu_ref_medium* med, msgpu_ref_rfun* rfun, int nthread);
/* replaces run_chistogram_omp, src/core/ms_core.c:173: the eigenvalues of M(k)
 * (or N(k), mtype normalized) of seeds 1..nseed in one batched GPU kernel, then
 * the reference's own fill_chist (chistogram_util.c:253) on them, in seed order;
 * fill_chist is taken from the program the library is linked into (a weak
 * reference: a program without it gets an error message and no histogram).  The
 * medium is left untouched, as the reference's private copies leave it. */
void run_chistogram_omp(msgpu_ref_medium* med, msgpu_ref_chist* chist, int nthread);
/* replaces run_imag_mu_histogram_omp, src/core/ms_core.c:225-282: the eigenvalues
 * and Tr[G^+ G]/N of seeds 1..nseed in one batched GPU kernel; the range from seed
 * 1's eigenvalues as setup_domain_ihist (imag_mu_histogram_util.c:80) takes it,
 * without its CPU zgeev, leaving med filled with seed 1 as that function does; the
 * eigenvalues appended in seed order with the reference's append_list_ihist and
 * normalised with its normalize_ihist (weak references, resolved from the
 * program); avgx = Re I(k, 0) by the GPU's Green function.  varx_expc is
 * Tr[G^+ G]/(4N) of M(k) itself (the reference evaluates it on the matrix zgeev
 * has overwritten). */
void run_imag_mu_histogram_omp(msgpu_ref_medium* med, msgpu_ref_ihist* ihist, int nthread);

#ifdef __cplusplus
}
#endif
#endif
