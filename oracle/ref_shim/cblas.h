/*
 * CBLAS declarations for compiling the unmodified reference sources into
 * the CPU oracle binary (oracle/_ref).  The calls are routed to the
 * OpenBLAS build that ships inside scipy (its exports carry a "scipy_"
 * prefix); oracle/build_ref.sh links it.  Test infrastructure only.
 */
#ifndef LDG_REF_SHIM_CBLAS_H
#define LDG_REF_SHIM_CBLAS_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

void scipy_cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                       int m, int n, int k, double alpha, const double* a, int lda,
                       const double* b, int ldb, double beta, double* c, int ldc);
void scipy_cblas_dscal(int n, double alpha, double* x, int incx);
void scipy_openblas_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dscal scipy_cblas_dscal

#endif
