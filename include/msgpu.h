/*
 * msgpu.h -- C ABI of the GB300 Foldy-Lax engine (libmsgpu.so).
 *
 * Plain C types only: no torch, no CUDA types in the signatures (streams are
 * passed as void*).  Complex numbers are two doubles {re, im}, the layout of
 * C99 `double _Complex` and LAPACK COMPLEX*16.  Matrices are column-major.
 *
 * Two layers:
 *   1. Batched entry points (msgpu_*): the performance path.  Each replaces
 *      a driver loop of the reference, cited below.
 *   2. Symbol-compatible drop-ins for the reference's own functions
 *      (build_ms_matrix, tracelog_lu, dk_log_det_ms, ...) in msgpu_dropin.h.
 *
 * Errors: functions return 0 on success, a negative MSGPU_E* code on a usage
 * or CUDA error (text in msgpu_last_error()).  Numerical conditions are
 * reported per result in a status word (MSGPU_S*), never by aborting.
 */
#ifndef MSGPU_H
#define MSGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scattering models, enum order of reference src/core/scattering_model_type.h:241 */
enum { MSGPU_HARDSPHERE = 0, MSGPU_SOFTSPHERE = 1, MSGPU_RESONANT = 2, MSGPU_MAXIMUM = 3 };
/* Medium shapes, enum order of reference src/core/medium_type.h:37 */
enum { MSGPU_CUBE = 0, MSGPU_BALL = 1, MSGPU_LATTICE = 2, MSGPU_GAUSSIAN = 3 };
/* Arithmetic of the LU */
enum { MSGPU_FP64 = 0, MSGPU_MIXED = 1 };
/* Root methods of the eigenstate search, enum order of reference src/core/eigenstate_list_type.h:20 */
enum { MSGPU_EIG_DETERMINANT = 0, MSGPU_EIG_MINEIGVAL = 1, MSGPU_EIG_INVTRACEINV = 2 };
/* Random functions, enum order of reference src/core/random_function_type.h:18 */
enum { MSGPU_RF_CRSEC = 0, MSGPU_RF_DOS = 1 };

/* per-result status bits */
#define MSGPU_S_OK 0
#define MSGPU_S_SINGULAR 1  /* an exactly-zero pivot (LAPACK info > 0), ln det = -inf */
#define MSGPU_S_NONFINITE 2 /* NaN or Inf reached the result */
#define MSGPU_S_RANGE 4     /* mixed precision: an entry beyond the FP32-safe range (|M_ij| >= 1e18), no result */
#define MSGPU_S_TIMEOUT 8   /* a bounded device wait gave up; the result is void */
#define MSGPU_S_NOCONV 16   /* inverse iteration: not converged within its 50 steps (value = last estimate) */
#define MSGPU_S_SPAN 32     /* mixed precision: the matrix entries spanned more than 2^8 but the run sliced four
                               ways, so the 1e-8 accuracy target is not guaranteed (never set when the job's
                               entry span was predicted correctly on the host) */

/* error codes */
#define MSGPU_E_ARG (-1)
#define MSGPU_E_CUDA (-2)
#define MSGPU_E_NODEV (-3)
#define MSGPU_E_SIZE (-4)

/* Inverse single-atom amplitude model (reference ScatteringModel,
 * src/core/scattering_model_type.h:246-258, parameters only). */
typedef struct msgpu_model {
    int type;     /* MSGPU_MAXIMUM, ... */
    int np;       /* parameters used */
    double p[2];  /* hardsphere/softsphere: alpha; resonant: Re p, Im p */
} msgpu_model;

/* One scatterer set (reference Medium, src/core/medium_type.h:42-54):
 * d coordinates per atom, n atoms, pos[i*d + c] atom-major, host memory. */
typedef struct msgpu_medium {
    int d;
    int n;
    const double* pos;
    msgpu_model model;
} msgpu_medium;

/* ---- runtime ------------------------------------------------------------ */
int msgpu_init(int device);               /* select and warm up the device */
const char* msgpu_last_error(void);
int msgpu_sm_count(void);
/* number of kernels this library has launched since load (all entry points) */
uint64_t msgpu_launch_count(void);
/* measured FP64 FMA throughput of the device in TFLOP/s (roofline denominator of the FP64 path) */
int msgpu_probe_fp64(double* tflops);
/* The same for the FP64 tensor path (warp-level mma.sync m8n8k4 f64), the
 * other candidate roofline of the FP64 engine */
int msgpu_probe_fp64_mma(double* tflops);

/* Tensor-core self-check: one 128 x 64 x 32 bf16 product D = A B^T (A 128x32,
 * B 64x32, row-major f32 holding small integers) through the engine's tcgen05
 * operand descriptors; mode bit 0 exchanges the descriptor's two core-matrix
 * strides, bit 1 negates B.  Used by the tests to pin the operand layout. */
int msgpu_probe_umma(int mode, const float* A, const float* B, float* D);

/* ---- host-side inputs (bit-exact with the reference) -------------------- */
/* fill_medium (src/core/medium_util.c:164): seeded scatterers, pos[n*d] */
int msgpu_fill_medium(int d, int n, int shape, double ratio, uint64_t seed, double* pos);
/* n successive random_double (src/core/nru_random.c:39) after init_random(seed) (:63) */
void msgpu_random_doubles(uint64_t seed, int n, double* out);
/* get_arg_cmap (src/core/complex_map_util.c:27) for l = 0..nx*ny-1 */
void msgpu_kplane_args(int nx, int ny, double xmin, double xmax, double ymin, double ymax, double* ks);
/* get_arg_ccut (src/core/complex_cut_util.c:32) for l = 0..3(ns+2)-1 */
void msgpu_kcut_args(int ns, const double* zmin, const double* zmax, double* ks);
/* init_logcut's logarithmic mesh (src/core/log_cut_util.c:93-96), k_i = rek +
 * i imkmin exp(ln(imkmax/imkmin) i/(ns-1)), i = 0..ns-1: the log cut that
 * run_tracelog_omp evaluates for a [logkcut] task (ms_core.c:734-740) */
void msgpu_logcut_args(int ns, double rek, double imkmin, double imkmax, double* ks);
/* set_halton_points (src/core/domain_util.c:180); dom = {xmin,xmax,ymin,ymax} */
void msgpu_halton_points(const double* dom, int n, double* z);

/* ---- device special functions (check against the reference goldens) ---- */
/* which: 0 = G_d(k,r) (free_green, src/core/green_bessel.c:280),
 *        1 = dG/dk (dk_free_green, :311), 2 = I_d(k,r) (free_green_imag, :298),
 *        3 = K_{d/2}(k) (bessel_k with twonu = d, :224; r ignored),
 *        4 = F(k)^-1 of *model (invf, src/core/medium_util.c:296; r ignored),
 *        5 = the d = 3 element M_ij = -G(k,r) and 6 = dM_ij/dk with FP64
 *            distance and reductions, double-float series (d ignored),
 *        7, 8 = the same two entirely in double-float on the FP32 pipe, as the
 *            mixed engine assembles d = 3 matrices (r rounded to 48 bits),
 *        9, 10 = the d = 2 element M_ij = K_0(-ikr)/(2 pi) and dM_ij/dk in
 *            double-float on the FP32 pipe, as the mixed engine assembles
 *            d = 2 matrices (d ignored) */
int msgpu_eval_special(int which, int d, const msgpu_model* model, int n, const double* ks, const double* rs,
                       double* out);

/* ---- matrices ----------------------------------------------------------- */
/* build_ms_matrix / build_dk_ms_matrix (src/core/ms_matrix_util.c:32, :68):
 * writes the n*n column-major matrix to host memory `mat`. */
int msgpu_build_matrix(const msgpu_medium* med, const double* k, int deriv, double* mat);
/* tracelog_lu (src/core/ms_matrix_util.c:185) of a host matrix: out = ln det / n
 * with the reference's branch (sum of Arg U_ii, + i pi for odd interchanges).
 * info (may be NULL) = LAPACK zgetrf info: 0, or the 1-based index of the
 * first exactly-zero pivot. */
int msgpu_tracelog_matrix(int n, const double* mat, double* out, int* info);

/* ---- batched hot path --------------------------------------------------- */
/* ln det M(k)/n for nitem items (medium item_med[i], wave number ks[2i..]).
 * Replaces the k-point loop of run_tracelog_omp (src/core/ms_core.c:115-136)
 * and build_ms_matrix + tracelog_lu per point.  Host pointers, synchronous.
 * out[2*nitem], status[nitem] (may be NULL). */
int msgpu_tracelog_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                         double* out, int* status, int precision);
/* dlogf = tr(M^-1 dM/dk) (dk_log_det_ms, src/core/ms_matrix_util.c:242) for each item. */
int msgpu_dk_log_det_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                           double* out, int* status, int precision);

/* Scattering amplitudes a = M^-1 phi for a plane wave along +x, phi_i =
 * exp(i k x_i) (reference ms_core.c:616-620 zgesv, incident_wave_util.c:76),
 * and the optical-theorem cross section -Im(conj(phi).a)/k in out[2i]
 * (total_cross_section, src/core/ms_matrix_util.c:344; out[2i+1] is its
 * imaginary part for complex k).  amps (may be NULL) receives a for every
 * item, n_i complex values each, concatenated in item order. */
int msgpu_amplitude_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                          double* out, double* amps, int* status, int precision);

/* ln det M(k)/n for one medium at nk wave numbers without allocating any
 * device memory.  For callers that cannot call cudaMalloc (a CUDA graph being
 * captured, a device whose memory another allocator owns).  No counterpart in
 * the reference.  All pointers are DEVICE pointers: d_pos[n*d] positions,
 * d_ks[2*nk] wave numbers, d_out[2*nk] results, d_status[nk] status words;
 * the work is queued on `stream` (cudaStream_t or NULL) and the call returns
 * without synchronizing.  Scratch is a fixed 128 MiB __device__ array inside
 * the library (held by every GPU that loads it): n <= 2048, nk <= 65536, else
 * MSGPU_E_SIZE.  The array holds floor(~128 MiB / (16 n^2)) matrix slots, one
 * per engine CTA, capped at 2 per SM: 304 CTAs for n <= 165, 127 at n = 256,
 * 31 at n = 512, 7 at n = 1024 and 1 at n = 2048, against the 304 the
 * allocating entry points run, so large n runs at a fraction of their
 * throughput (1/43 at n = 1024).  Calls share that array, so calls that
 * overlap on the GPU race: keep them on one stream.  The first call on a
 * device looks up the array's address; make it before any stream capture.
 * Counted in msgpu_launch_count (two launches per call); errors set the text
 * of msgpu_last_error. */
int msgpu_tracelog_batch_noalloc(int d, int n, const double* d_pos, msgpu_model model, int nk, const double* d_ks,
                                 double* d_out, int* d_status, void* stream);

/* Resonance search, find_eigenstates_serial_1 (src/core/ms_core.c:320-328) /
 * solve_aberth (src/core/root_finder.c:522-577) for every medium: the
 * Maehly-Aberth-Ehrlich iteration on dlogf = tr(M^-1 dM/dk) from the nz
 * starting points z0 (re, im pairs; the same for every medium), with the
 * exponential background polynomial of degree nexpsup-1 fitted on 6*nexpsup
 * Halton samples of dom = {xmin, xmax, ymin, ymax}.  Each sweep evaluates
 * dlogf for all roots still in progress in one batched GPU job, then replays
 * the reference's Gauss-Seidel update in FP64.  roots[2*(m*nz + i)] receives
 * the converged roots of medium m sorted by Re, nroots[m] their number;
 * *nevals (may be NULL) the dlogf evaluations made. */
int msgpu_solve_aberth_batch(int nmed, const msgpu_medium* media, const double* dom, int nz, const double* z0,
                             int nexpsup, int maxit, double toler, int precision, double* roots, int* nroots,
                             int* nevals);

/* Wavefunction of run_wave_function_omp (src/core/ms_core.c:596-649), plane
 * wave along +x: for each medium (realisation, all of equal n and d) the
 * amplitudes a = M^-1 phi on the GPU, then psi(r) = exp(i k x) + sum_i a_i
 * G(k,|r - x_i|) on the nx*ny pixel grid of dom = {xmin,xmax,ymin,ymax} in the
 * (x, y, 0...) plane, row-major from (xmin, ymax) (wave_function_util.c:76).
 * function/density[nx*ny] receive Re psi and |psi|^2 averaged over the media;
 * psi (may be NULL) the complex psi of media[0]; amps (may be NULL) a for
 * every medium (n complex each). */
int msgpu_wave_function(int nmed, const msgpu_medium* media, const double* k, int nx, int ny, const double* dom,
                        double* function, double* density, double* psi, double* amps, int precision);
/* The same at nk wave numbers ks[2*nk] (one solve per medium and k, all in
 * one batched job): function/density[nk*nx*ny] and psi[nk*nx*ny] (complex,
 * media[0]) are k-major, amps[nmed][nk][n].  MSGPU_MIXED solves with the
 * mixed engine plus FP64-residual refinement and, for d = 3, evaluates the
 * Green functions of the grid in double-float arithmetic on the FP32 pipe
 * (|Im k| * r < 80 over the grid; otherwise FP64).  Both return a negative
 * MSGPU_E_* code on error, else the OR of the MSGPU_S_* status words of every
 * solve: 0 when all are clean, MSGPU_S_SINGULAR or MSGPU_S_NONFINITE when a
 * singular or non-finite solve was averaged into function and density (the
 * reference's zgesv_ loop, ms_core.c:620, goes on silently in that case). */
int msgpu_wave_function_batch(int nmed, const msgpu_medium* media, int nk, const double* ks, int nx, int ny,
                              const double* dom, double* function, double* density, double* psi, double* amps,
                              int precision);
/* Wavefunction cut of run_wave_function_cut_omp (src/core/ms_core.c:654-703),
 * plane wave along +x: every medium's amplitudes a = M^-1 phi in one batched
 * job, then psi of each medium at the nbin points (xmin + i dx, 0, ...),
 * dx = (xmax - xmin)/(nbin - 1) (get_pos_wfcut, init_wfcut):
 * psi[2*(m*nbin + i)] complex; amps (may be NULL) as above.  Returns the OR of
 * the solves' MSGPU_S_* words, or a negative MSGPU_E_* code. */
int msgpu_wave_cut(int nmed, const msgpu_medium* media, const double* k, int nbin, double xmin, double xmax,
                   double* psi, double* amps, int precision);
/* Differential cross section of run_differential_cross_section_omp
 * (src/core/ms_core.c:526-594) at real k, plane wave along +x: every medium's
 * amplitudes a in one batched job, then for the nbin angles
 * th_i = thmin exp(i log(thmax/thmin)/(nbin-1)) degrees (get_arg_dcs,
 * diff_cross_section_util.c:86; thmin, thmax > 0) the far-field sample
 * (k/2pi)^(d-3)/(16 pi^2) |sum_j conj(b_j) a_j|^2, b the plane wave of
 * direction th_i (build_plane_wave), into samples[m + i*nmed] (nmed <= 65535).
 * Returns the OR of the solves' MSGPU_S_* words, or a negative MSGPU_E_* code. */
int msgpu_diff_cross_section(int nmed, const msgpu_medium* media, double k, int nbin, double thmin, double thmax,
                             double* samples, int precision);

/* Random function of run_random_function_omp (src/core/ms_core.c:476-519):
 * for every seed g < nseed (medium filled with seed g+1 by fill_medium) and
 * every bin i < nbin, k_i = xmin exp(i log(xmax/xmin)/(nbin-1))
 * (random_function_util.c:103), the total cross section
 * (MSGPU_RF_CRSEC, ms_matrix_util.c:344) or the density of states
 * -Im dlogf(k_i)/(2 pi k_i) (MSGPU_RF_DOS) into data[g + i*nseed]; each bin's
 * nseed samples then sorted ascending (sort_random_function,
 * random_function_util.c:110).  status (may be NULL) per sample, same
 * layout before sorting. */
int msgpu_random_function(int type, int d, int n, int shape, double ratio, const msgpu_model* model, int nseed,
                          int nbin, double xmin, double xmax, double* data, int* status, int precision);

/* traceinv (src/core/ms_matrix_util.c:319): tr M(k)^-1 per item, by the FP64
 * engine's n-right-hand-side solve (a MSGPU_MIXED request runs on it too). */
int msgpu_traceinv_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                         double* out, int* status, int precision);
/* inverse_iteration (ms_matrix_util.c:279) on M(k) from the constant unit
 * vector, 50 steps, tolerance 1e-10 (the reference's compute_eigenstates,
 * ms_core.c:296-312): lambda[2*i] the eigenvalue of smallest modulus, vecs
 * (may be NULL) the normalised eigenvectors (n complex per item, item order),
 * status bit MSGPU_S_NOCONV if the iteration did not converge. */
int msgpu_inverse_iteration_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                                  const double* ks, double* lambda, double* vecs, int* status, int precision);

/* The root methods "mineigval" and "invtraceinv" (find_eigenstates_serial_2/3,
 * src/core/ms_core.c:335-401): Muller's method (root_finder.c:342) from each of
 * the nz starting points z0 (the same for every medium) on the smallest
 * eigenvalue of M(k) or on 1/tr M(k)^-1; all function values of one step, over
 * every root and medium, in one batched GPU job.  Non-converged roots dropped,
 * duplicates (relative 1e-14) removed, order kept: roots[2*(m*nz + i)],
 * nroots[m]; *nevals (may be NULL) the function evaluations.  mineigval chains
 * one eigenvector through every evaluation of a realisation, as the reference
 * does (ms_core.c:339-340): each inverse iteration starts from the vector the
 * previous one returned, roots in the reference's order (including the check of
 * f at each root, ms_core.c:356), from the constant unit vector at the start;
 * the batch is over the realisations. */
int msgpu_find_roots_muller_batch(int method, int nmed, const msgpu_medium* media, const double* dom, int nz,
                                  const double* z0, int maxit, double toler, int precision, double* roots,
                                  int* nroots, int* nevals);

/* The eigenvalues mu of M(k) per item (eigvals, src/core/ms_matrix_util.c:147,
 * zgeev_ without eigenvectors; the input of the mu-plane histograms,
 * ms_core.c:173-282), one kernel over the batch: each CTA assembles M(k),
 * reduces it to Hessenberg form by Householder reflectors and takes its
 * eigenvalues by single-shift complex QR (LAPACK's zgehd2 and zlahqr
 * schemes, FP64, no balancing).  n <= 4097.  mu receives n complex values per
 * item, items in order, in deflation order within an item; status (may be
 * NULL) MSGPU_S_NOCONV where the QR iteration did not converge within
 * 30 max(10, n) iterations (those values read 0). */
int msgpu_eigvals_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                        double* mu, int* status);

/* The same for the matrix type of the mu-plane task (mtype in run_chistogram_omp,
 * ms_core.c:173-232): MSGPU_MTYPE_MSMATRIX, M(k), as msgpu_eigvals_batch; or
 * MSGPU_MTYPE_NORMALIZED, N(k) = i - G(k)/I(k,0) with I(k,0) = -Im G(k, 0)
 * (build_normalized_matrix, ms_matrix_util.c:50), independent of the
 * scattering model.  trg2 (may be NULL) receives per item Tr[G^+ G]/N of the
 * matrix, 2 sum_{i<j} |A_ij|^2 / n (tracegtwo, ms_matrix_util.c:167), which the
 * Im mu histogram task uses for its expected variance. */
#define MSGPU_MTYPE_MSMATRIX 0
#define MSGPU_MTYPE_NORMALIZED 1
int msgpu_eigvals_batch_mtype(int mtype, int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                              const double* ks, double* mu, int* status, double* trg2);

/* Launch choices (autotuning).  Per (kind, requested precision, size bucket
 * of the job's largest n: (2^(b-1), 2^b]) the engine that runs and the
 * resident CTAs per SM of the persistent grid.  engine: MSGPU_FP64,
 * MSGPU_MIXED (only for a mixed request) or -1 = the requested one; ctas 0 =
 * as many as fit.  The FP64 engine may serve a mixed request: it meets the
 * mixed accuracy bound with room to spare. */
int msgpu_tune_set(int kind, int precision, int n, int engine, int ctas_per_sm);
int msgpu_tune_get(int kind, int precision, int n, int* engine, int* ctas_per_sm);
/* Time every candidate (engine x 1 or 2 CTAs per SM) on a probe batch of
 * nitem k for n scatterers of d dimensions (the reference ball, seed 1) and
 * keep the fastest for that size bucket.  seconds[4] receives the times
 * (fp64 x1, fp64 x2, mixed x1, mixed x2; -1 where not run). */
int msgpu_autotune(int kind, int precision, int d, int n, int nitem, double* seconds);

/* Resident jobs: inputs uploaded once, the hot path run on device-resident
 * data (asynchronously on `stream`, a cudaStream_t or NULL), results fetched
 * separately.  kind: 0 = ln det / n, 1 = dlogf, 2 = amplitudes (as above),
 * 3 = traceinv, 4 = inverse iteration (FP64 engine). */
typedef struct msgpu_job msgpu_job;
msgpu_job* msgpu_job_create(int kind, int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                            const double* ks, int precision);
int msgpu_job_run(msgpu_job* job, void* stream);
/* Replace the job's items (nitem <= the count it was created with) keeping
 * its media resident: the next run evaluates these points. */
int msgpu_job_set_points(msgpu_job* job, int nitem, const int* item_med, const double* ks);
/* on != 0: msgpu_job_run replays a CUDA graph of the run (queue reset plus
 * the persistent engine launch), captured on first use and recaptured only if
 * the library's shared workspace moved; set_points needs no recapture (the
 * engine reads the live item count from device memory). */
int msgpu_job_use_graph(msgpu_job* job, int on);
int msgpu_job_results(msgpu_job* job, double* out, int* status);
int msgpu_job_amplitudes(msgpu_job* job, double* amps);
/* Eigenvector jobs (kind 4): the starting vector of every item's inverse
 * iteration, in the layout msgpu_job_amplitudes returns (n_i complex values
 * per item, concatenated in item order); from then on the job starts each
 * inverse iteration from these vectors instead of the constant unit vector,
 * as the reference's mineigval does with the vector of its previous call
 * (src/core/ms_core.c:339-340).  Each run overwrites them with its eigenvectors. */
int msgpu_job_set_vectors(msgpu_job* job, const double* vecs);
/* kernels launched by one msgpu_job_run */
int msgpu_job_launches(const msgpu_job* job);
/* algorithmic real flops of one msgpu_job_run (8/3 n^3 per ln det; 8/3 n^3 + 8 n^3 per dlogf) */
double msgpu_job_flops(const msgpu_job* job);
void msgpu_job_destroy(msgpu_job* job);
/* Per-phase SM cycles, summed over CTAs, of the last mixed-precision run made
 * with the environment variable MSGPU_STATS set: out[0..6] = assembly, panel,
 * TRSM, slicing, tensor tiles, solves, items.  Returns the count written. */
int msgpu_engine_stats(double* out, int n);
/* Failure-path test hook, no counterpart in the reference: the poll limit of
 * the first operand wait (an mbarrier wait on a bulk copy) of every mixed
 * trailing update in later runs; polls < 0 restores the normal limit.  With 0
 * that wait runs out at once: the engine issues no MMA, lets the copy in
 * flight land, marks the item and every item not yet taken MSGPU_S_TIMEOUT
 * (value NaN), frees its tensor memory and returns; the device stays usable. */
int msgpu_debug_first_wait_limit(int polls);

#ifdef __cplusplus
}
#endif
#endif
