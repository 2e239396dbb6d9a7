/* Test infrastructure (oracle build only): a minimal CBLAS header so that the
 * reference library's sources compile against the OpenBLAS that ships inside
 * the scipy wheel.  That library exports its CBLAS entry points with a
 * `scipy_` prefix, so each name the reference uses is mapped onto the
 * exported one.  Enum values are the standard CBLAS ones. */
#pragma once

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };

#define cblas_zgemm scipy_cblas_zgemm
#define cblas_zgemv scipy_cblas_zgemv
#define cblas_zdotc_sub scipy_cblas_zdotc_sub
#define cblas_dznrm2 scipy_cblas_dznrm2
#define cblas_zscal scipy_cblas_zscal
#define cblas_zdscal scipy_cblas_zdscal
#define cblas_ztrsm scipy_cblas_ztrsm
#define cblas_ztrsv scipy_cblas_ztrsv
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dscal scipy_cblas_dscal

typedef int blasint;

void cblas_zgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                 blasint m, blasint n, blasint k, void const *alpha,
                 void const *a, blasint lda, void const *b, blasint ldb,
                 void const *beta, void *c, blasint ldc);
void cblas_zgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, blasint m, blasint n,
                 void const *alpha, void const *a, blasint lda, void const *x,
                 blasint incx, void const *beta, void *y, blasint incy);
void cblas_zdotc_sub(blasint n, void const *x, blasint incx, void const *y,
                     blasint incy, void *ret);
double cblas_dznrm2(blasint n, void const *x, blasint incx);
void cblas_zscal(blasint n, void const *alpha, void *x, blasint incx);
void cblas_zdscal(blasint n, double alpha, void *x, blasint incx);
void cblas_ztrsm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO,
                 enum CBLAS_TRANSPOSE, enum CBLAS_DIAG, blasint m, blasint n,
                 void const *alpha, void const *a, blasint lda, void *b,
                 blasint ldb);
void cblas_ztrsv(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE,
                 enum CBLAS_DIAG, blasint n, void const *a, blasint lda,
                 void *x, blasint incx);
void cblas_daxpy(blasint n, double alpha, double const *x, blasint incx,
                 double *y, blasint incy);
void cblas_dgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, blasint m, blasint n,
                 double alpha, double const *a, blasint lda, double const *x,
                 blasint incx, double beta, double *y, blasint incy);
void cblas_dscal(blasint n, double alpha, double *x, blasint incx);
