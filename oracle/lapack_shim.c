/*
 * lapack_shim.c -- forwards the Fortran LAPACK symbols the reference declares
 * (src/core/ms_matrix_util.c:137-142, src/core/root_finder.c:27-28,
 * src/core/ms_core.c:47) to the OpenBLAS that scipy bundles, whose exports
 * carry a "scipy_" prefix.  Only linked into oracle/_ref (test
 * infrastructure).
 */
typedef double _Complex zc;
void scipy_zgetrf_(int*, int*, zc*, int*, int*, int*);
void scipy_zgetrs_(char*, int*, int*, zc*, int*, int*, zc*, int*, int*);
void scipy_zgesv_(int*, int*, zc*, int*, int*, zc*, int*, int*);
void scipy_zgeev_(char*, char*, int*, zc*, int*, zc*, zc*, int*, zc*, int*, zc*, int*, double*, int*);
void scipy_zgetri_(int*, zc*, int*, int*, zc*, int*, int*);
void scipy_zgeqrf_(int*, int*, zc*, int*, zc*, zc*, int*, int*);
void scipy_zgels_(char*, int*, int*, int*, zc*, int*, zc*, int*, zc*, int*, int*);
void scipy_dgels_(char*, int*, int*, int*, double*, int*, double*, int*, double*, int*, int*);
void scipy_dgesv_(int*, int*, double*, int*, int*, double*, int*, int*);
void scipy_openblas_set_num_threads(int);

void zgetrf_(int* m, int* n, zc* a, int* lda, int* ipiv, int* info) { scipy_zgetrf_(m, n, a, lda, ipiv, info); }
void zgetrs_(char* t, int* n, int* nr, zc* a, int* lda, int* ip, zc* b, int* ldb, int* info) {
    scipy_zgetrs_(t, n, nr, a, lda, ip, b, ldb, info);
}
void zgesv_(int* n, int* nr, zc* a, int* lda, int* ip, zc* b, int* ldb, int* info) {
    scipy_zgesv_(n, nr, a, lda, ip, b, ldb, info);
}
void zgeev_(char* jl, char* jr, int* n, zc* a, int* lda, zc* w, zc* vl, int* ldvl, zc* vr, int* ldvr, zc* work,
            int* lwork, double* rwork, int* info) {
    scipy_zgeev_(jl, jr, n, a, lda, w, vl, ldvl, vr, ldvr, work, lwork, rwork, info);
}
void zgetri_(int* n, zc* a, int* lda, int* ip, zc* work, int* lwork, int* info) {
    scipy_zgetri_(n, a, lda, ip, work, lwork, info);
}
void zgeqrf_(int* m, int* n, zc* a, int* lda, zc* tau, zc* work, int* lwork, int* info) {
    scipy_zgeqrf_(m, n, a, lda, tau, work, lwork, info);
}
void zgels_(char* t, int* m, int* n, int* nr, zc* a, int* lda, zc* b, int* ldb, zc* w, int* lw, int* info) {
    scipy_zgels_(t, m, n, nr, a, lda, b, ldb, w, lw, info);
}
void dgels_(char* t, int* m, int* n, int* nr, double* a, int* lda, double* b, int* ldb, double* w, int* lw,
            int* info) {
    scipy_dgels_(t, m, n, nr, a, lda, b, ldb, w, lw, info);
}
void dgesv_(int* n, int* nr, double* a, int* lda, int* ip, double* b, int* ldb, int* info) {
    scipy_dgesv_(n, nr, a, lda, ip, b, ldb, info);
}
__attribute__((constructor)) static void one_thread(void) { scipy_openblas_set_num_threads(1); }
