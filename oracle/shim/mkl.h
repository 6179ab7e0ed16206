/*
 * Declaration-only stand-in for <mkl.h>, used ONLY to compile the reference
 * Kylin-V sources in place as a CPU oracle (test infrastructure, never shipped
 * and never linked into the GPU library).
 *
 * Intel MKL is not installed here.  The reference calls ten CBLAS/LAPACKE
 * routines (util/allocation.h:149-230, holstein/block.h:90-113,
 * holstein/product.h:221-423, holstein/svd.h:241-342).  scipy's bundled LP64
 * OpenBLAS exports the same routines under a "scipy_" prefix, with the same
 * calling convention as CBLAS/LAPACKE; this header declares them and maps the
 * MKL names onto them.  Integer width: the reference defines MKL_INT as int
 * (util/global.h:24), which matches the LP64 interface.
 *
 * Enum values are the standard CBLAS ones (row major 101, no-trans 111,
 * trans 112, conj-trans 113) and LAPACK_ROW_MAJOR is 101.
 */
#ifndef KV_ORACLE_MKL_SHIM_H
#define KV_ORACLE_MKL_SHIM_H

#include <complex>

#ifndef MKL_INT
#define MKL_INT int
#endif

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
#define LAPACK_ROW_MAJOR 101

extern "C" {
/* level 3 */
void scipy_cblas_zgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb,
                       int m, int n, int k, const void *alpha, const void *a, int lda,
                       const void *b, int ldb, const void *beta, void *c, int ldc);
/* level 1 */
void scipy_cblas_zaxpy(int n, const void *alpha, const void *x, int incx, void *y, int incy);
void scipy_cblas_zscal(int n, const void *alpha, void *x, int incx);
void scipy_cblas_zdscal(int n, double alpha, void *x, int incx);
void scipy_cblas_zcopy(int n, const void *x, int incx, void *y, int incy);
void scipy_cblas_zdotc_sub(int n, const void *x, int incx, const void *y, int incy, void *dotc);
double scipy_cblas_dznrm2(int n, const void *x, int incx);
double scipy_cblas_dnrm2(int n, const double *x, int incx);
/* LAPACKE */
int scipy_LAPACKE_zgesvd(int layout, char jobu, char jobvt, int m, int n, void *a, int lda,
                         double *s, void *u, int ldu, void *vt, int ldvt, double *superb);
int scipy_LAPACKE_zheevd(int layout, char jobz, char uplo, int n, void *a, int lda, double *w);
}

#define cblas_zgemm      scipy_cblas_zgemm
#define cblas_zaxpy      scipy_cblas_zaxpy
#define cblas_zscal      scipy_cblas_zscal
#define cblas_zdscal     scipy_cblas_zdscal
#define cblas_zcopy      scipy_cblas_zcopy
#define cblas_zdotc_sub  scipy_cblas_zdotc_sub
#define cblas_dznrm2     scipy_cblas_dznrm2
#define cblas_dnrm2      scipy_cblas_dnrm2
#define LAPACKE_zgesvd   scipy_LAPACKE_zgesvd
#define LAPACKE_zheevd   scipy_LAPACKE_zheevd

#endif
