/* lapack_shim.c -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference program calls the Fortran-ABI LAPACK/BLAS routines dsyevd_,
 * dgeev_ and dgemm_ (source/BcDor-DysonMatrix.cpp:35-36, source/BcDor-gII_b.cpp:36,
 * source/BcDor-CCD_b.cpp:37).  This image has no system LAPACK; SciPy ships an
 * OpenBLAS build whose exports carry a "scipy_" prefix and 32-bit integers.
 * These three forwards let the reference objects link against it. */
void scipy_dsyevd_(char *, char *, int *, double *, int *, double *, double *, int *, int *, int *, int *);
void scipy_dgeev_(char *, char *, int *, double *, int *, double *, double *, double *, int *, double *,
                  int *, double *, int *, int *);
void scipy_dgemm_(char *, char *, int *, int *, int *, double *, double *, int *, double *, int *, double *,
                  double *, int *);

void dsyevd_(char *a, char *b, int *n, double *m, int *lda, double *w, double *work, int *lwork, int *iwork,
             int *liwork, int *info) {
    scipy_dsyevd_(a, b, n, m, lda, w, work, lwork, iwork, liwork, info);
}
void dgeev_(char *a, char *b, int *n, double *m, int *lda, double *wr, double *wi, double *vl, int *ldvl,
            double *vr, int *ldvr, double *work, int *lwork, int *info) {
    scipy_dgeev_(a, b, n, m, lda, wr, wi, vl, ldvl, vr, ldvr, work, lwork, info);
}
void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *al, double *a, int *lda, double *b, int *ldb,
            double *be, double *c, int *ldc) {
    scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc);
}
