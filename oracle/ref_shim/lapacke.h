/*
 * LAPACKE declarations (LP64) for compiling the unmodified reference
 * sources into the CPU oracle binary (oracle/_ref), routed to scipy's
 * bundled OpenBLAS ("scipy_" prefixed exports).  Test infrastructure only.
 */
#ifndef LDG_REF_SHIM_LAPACKE_H
#define LDG_REF_SHIM_LAPACKE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

lapack_int scipy_LAPACKE_dgesv(int layout, lapack_int n, lapack_int nrhs, double* a,
                               lapack_int lda, lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int scipy_LAPACKE_dsyev(int layout, char jobz, char uplo, lapack_int n, double* a,
                               lapack_int lda, double* w);
lapack_int scipy_LAPACKE_dsytrf(int layout, char uplo, lapack_int n, double* a, lapack_int lda,
                                lapack_int* ipiv);
lapack_int scipy_LAPACKE_dsytrs(int layout, char uplo, lapack_int n, lapack_int nrhs,
                                const double* a, lapack_int lda, const lapack_int* ipiv,
                                double* b, lapack_int ldb);

#ifdef __cplusplus
}
#endif

#define LAPACKE_dgesv scipy_LAPACKE_dgesv
#define LAPACKE_dsyev scipy_LAPACKE_dsyev
#define LAPACKE_dsytrf scipy_LAPACKE_dsytrf
#define LAPACKE_dsytrs scipy_LAPACKE_dsytrs

#endif
