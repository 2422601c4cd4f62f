/*
 * msgpu_dropin.h -- symbol-compatible replacements for the reference's own
 * hot-path functions and for every task driver of src/core/ms_core.c.
 * libmsgpu.so exports these names with the reference's signatures, so the
 * reference's callers (src/core/ms_core.c, root_finder.c users, the tests)
 * relink against the GPU without source changes.
 *
 * The structs below are layout-identical to the reference types they stand
 * for, field for field and under the reference's field names
 * (tests/test_dropin_layouts.py asserts every size and offset against the
 * reference's own headers).  The task drop-ins hand their results to the
 * reference's own histogram, eigenstate-list and cut-statistics functions
 * through weak references, resolved from the program they are linked into;
 * without those functions they print an error and return.
 */
#ifndef MSGPU_DROPIN_H
#define MSGPU_DROPIN_H
#include <complex.h>
#include <stdint.h>

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

/* reference Domain, src/core/domain_type.h:19-24 */
typedef struct msgpu_ref_domain {
    double xmin;
    double xmax;
    double ymin;
    double ymax;
} msgpu_ref_domain;

/* reference IncidentWave, src/core/incident_wave_type.h:23-31 */
typedef struct msgpu_ref_iwave {
    int source; /* IncidentWaveSource: 0 plane, 1 spherical */
    msgpu_dcomplex k;
    char desc_ascii[80];
    char desc_latex[80];
} msgpu_ref_iwave;

/* reference WaveFunction, src/core/wave_function_type.h:22-41 */
typedef struct msgpu_ref_wfun {
    int nseed;
    uint64_t iseed;
    msgpu_ref_iwave* iwave;
    int nx;
    int ny;
    msgpu_ref_domain* dom;
    double dx;
    double dy;
    double* function;
    double* density;
    void* colrule1;
    void* colrule2;
    double realtime;
} msgpu_ref_wfun;

/* reference WaveFunctionCut, src/core/wave_function_cut_type.h:20-38 */
typedef struct msgpu_ref_wfcut {
    int nseed;
    uint64_t iseed;
    msgpu_ref_iwave* iwave;
    int nbin;
    double xmin;
    double xmax;
    double dx;
    int ntot;
    double* repsi;
    double* impsi;
    double* density;
    double realtime;
} msgpu_ref_wfcut;

/* reference DiffCrossSection, src/core/diff_cross_section_type.h:15-31 */
typedef struct msgpu_ref_dcs {
    int nseed;
    uint64_t iseed;
    double k;
    double thmin;
    double thmax;
    int nbin;
    int nq;
    int ntot;
    double* data;
    double* mean;
    int nc;
    double* curve;
    char title[80];
    double realtime;
} msgpu_ref_dcs;

/* reference Eigenstate, src/core/eigenstate_type.h:23-35 */
typedef struct msgpu_ref_eigenstate {
    msgpu_dcomplex kroot;
    msgpu_dcomplex mu;
    msgpu_dcomplex* eigv;
    int isfitted;
    double* center;
    double locfac;
    double ampcst;
} msgpu_ref_eigenstate;

/* reference EigenstateList, src/core/eigenstate_list_type.h:25-44 */
typedef struct msgpu_ref_eigls {
    msgpu_ref_medium* med;
    uint64_t seed;
    int method; /* EigenstateMethod: 0 determinant, 1 mineigval, 2 invtraceinv */
    int ntarget;
    msgpu_ref_domain* dom;
    int maxit;
    double toler;
    int verb;
    int nstate;
    int nfitted;
    msgpu_ref_eigenstate** eigtab;
    double realtime;
} msgpu_ref_eigls;

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
/* replaces run_wave_function_omp, src/core/ms_core.c:596-649, for the plane
 * incident wave (a spherical source prints an error and leaves the arrays as
 * they are): the realisations of seeds iseed..iseed+nseed-1 solved and summed
 * over the nx*ny grid in one batched GPU job (msgpu_wave_function, mixed LU
 * refined to an FP64 residual); function/density receive the averages added
 * to their entry values divided by nseed, i.e. (entry + sum)/nseed as the
 * reference's sum and divide_wfun; med is left holding the last seed. */
void run_wave_function_omp(msgpu_ref_medium* med, msgpu_ref_wfun* wfun, int nthread);
/* replaces run_wave_function_cut_omp, src/core/ms_core.c:654-703, for the plane
 * incident wave: psi of every seed iseed..iseed+nseed-1 on the cut in one
 * batched GPU job (msgpu_wave_cut, mixed LU refined to an FP64 residual), the
 * samples laid out bin-major as the reference's and handed to its own
 * store_data_wfcut (weak reference, resolved from the program) for the means
 * and quartiles.  med is left as it was, as the reference's private copies
 * leave it. */
void run_wave_function_cut_omp(msgpu_ref_medium* med, msgpu_ref_wfcut* wfcut, int nthread);
/* replaces run_differential_cross_section_omp, src/core/ms_core.c:526-594: the
 * samples of seeds iseed..iseed+nseed-1 in one batched GPU job
 * (msgpu_diff_cross_section, mixed LU refined to an FP64 residual), then the
 * reference's statistics in its order: the first nc seeds' curves, each bin's
 * samples sorted, its nq quantiles at q/(nq-1) and its mean (real_vector_util.c
 * quantile and mean_vector).  med is left as it was. */
void run_differential_cross_section_omp(msgpu_ref_medium* med, msgpu_ref_dcs* dcs, int nthread);
/* replace find_eigenstates_serial_1/2/3, src/core/ms_core.c:320-401: the
 * resonance search on the realisation in eigls->med from the *nroot starting
 * points kroot, by the determinant (Aberth on dlogf, nexpsup = 4), mineigval or
 * invtraceinv (Muller) method, every step's function values in one batched
 * FP64 GPU job (msgpu_solve_aberth_batch, msgpu_find_roots_muller_batch);
 * kroot and *nroot receive the roots as the reference leaves them; realtime set. */
void find_eigenstates_serial_1(msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot);
void find_eigenstates_serial_2(msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot);
void find_eigenstates_serial_3(msgpu_ref_eigls* eigls, int* nroot, msgpu_dcomplex* kroot);
/* replaces compute_eigenstates, src/core/ms_core.c:296-313: the eigenvectors
 * of every root in one batched FP64 GPU job (msgpu_inverse_iteration_batch:
 * constant unit start, 50 steps, tolerance 1e-10, the only values the
 * reference passes; others print an error and return), stored through the
 * reference's own alloc_eigenstate_list and checked with its
 * check_eigenstate_list (weak references, resolved from the program). */
void compute_eigenstates(msgpu_ref_eigls* eigls, int nroot, msgpu_dcomplex* kroot, int maxit, double toler, int verb);

#ifdef __cplusplus
}
#endif
#endif
