/*
 * msoracle.h -- CPU oracle for the Foldy-Lax ln det / dlogf / resonance /
 * wavefunction path of MSModel (david-gaspard/msmodel v1.0.0).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product (msmodel_gb300) never links, loads or calls it.
 *
 * Every entry point restates one reference function; the .c file cites the
 * reference file:line for each.  Complex numbers cross this ABI as two
 * doubles (re, im) so that Python ctypes can drive it.
 *
 * Dense LU: either the oracle's own restatement of LAPACK zgetf2 (partial
 * pivoting, IZAMAX |re|+|im| rule) or, after orc_set_lapack(), the LAPACK the
 * reference links against (the scipy-bundled OpenBLAS: scipy_zgetrf_ ...).
 */
#ifndef MSORACLE_H
#define MSORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scattering model, enum order of src/core/scattering_model_type.h:241. */
enum { ORC_HARDSPHERE = 0, ORC_SOFTSPHERE = 1, ORC_RESONANT = 2, ORC_MAXIMUM = 3 };
/* Medium shape, enum order of src/core/medium_type.h:37. */
enum { ORC_CUBE = 0, ORC_BALL = 1, ORC_LATTICE = 2, ORC_GAUSSIAN = 3 };

typedef struct {
    int type;      /* ORC_* model */
    int np;        /* number of parameters used */
    double p[2];   /* model parameters */
} orc_model;

/* LAPACK plumbing */
int  orc_set_lapack(const char* openblas_path); /* 0 on success */
int  orc_have_lapack(void);
const char* orc_lapack_config(void);

/* RNG + medium (bit-exact) */
void     orc_rng_init(uint64_t* st4, uint64_t seed);
uint64_t orc_rng_next(uint64_t* st4);
double   orc_rng_double(uint64_t* st4);
void     orc_fill_medium(int d, int n, int shape, double ratio, uint64_t seed, double* pos);
double   orc_uball_volume(int d);
double   orc_uball_surface(int d);

/* special functions, complex as double[2] */
void orc_bessel_k(int twonu, const double* z, double* out);
void orc_free_green(int d, const double* k, double r, double* out);
void orc_dk_free_green(int d, const double* k, double r, double* out);
void orc_free_green_imag(int d, const double* k, double r, double* out);
void orc_hyp0f1(double a, const double* z, double* out);
void orc_invf(const orc_model* m, int d, const double* k, double* out);

/* matrices: mat is n*n complex (2*n*n doubles), column-major */
void orc_build_ms_matrix(int d, int n, const double* pos, const orc_model* m, const double* k, double* mat);
void orc_build_dk_ms_matrix(int d, int n, const double* pos, const orc_model* m, const double* k, double* mat);
int  orc_lu(int n, double* mat, int* ipiv, int use_lapack);             /* returns LAPACK-style info */
int  orc_tracelog_lu(int n, double* mat, int use_lapack, double* out);  /* out = ln det / n */
int  orc_dk_log_det(int d, int n, const double* pos, const orc_model* m, const double* k, int use_lapack, double* out);
double orc_total_cross_section(int d, int n, const double* pos, const orc_model* m, double k, int use_lapack);
int  orc_solve(int n, double* mat, double* rhs, int use_lapack);         /* M x = rhs, 1 RHS, in place */

/* batched drivers (OpenMP over points, one private matrix per thread) */
void orc_tracelog_batch(int d, int n, const double* pos, const orc_model* m, int nk, const double* ks,
                        double* out, int* info, int nthreads, int use_lapack);
void orc_dlogf_batch(int d, int n, const double* pos, const orc_model* m, int nk, const double* ks,
                     double* out, int nthreads, int use_lapack);

/* k-grids and Halton points */
void orc_kplane_args(int nx, int ny, double xmin, double xmax, double ymin, double ymax, double* ks);
void orc_kcut_args(int ns, const double* zmin, const double* zmax, double* ks);
void orc_halton_points(const double* dom, int n, double* z);

/* Maehly-Aberth-Ehrlich on dlogf = tr(M^-1 dM/dk); z in/out (2*nz doubles);
 * returns the number of converged roots (sorted by Re). */
int orc_solve_aberth(int d, int n, const double* pos, const orc_model* m, const double* dom,
                     int nz, double* z, int nexpsup, int maxit, double toler, int use_lapack,
                     int* nevals);

/* plane-wave (+x) wavefunction: a = M^-1 phi, psi on an nx*ny grid of (x,y,0) */
void orc_psi_grid(int d, int n, const double* pos, const double* k, int nx, int ny, const double* dom,
                  const double* amp, double* psi, int nthreads);
int orc_wavefunction(int d, int n, const double* pos, const orc_model* m, const double* k,
                     int nx, int ny, const double* dom, double* amp, double* psi, int nthreads,
                     int use_lapack);

#ifdef __cplusplus
}
#endif
#endif
