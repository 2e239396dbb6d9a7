/* Test infrastructure (oracle build only): a minimal LAPACKE header mapping
 * the reference's LAPACKE calls onto the `scipy_`-prefixed exports of the
 * OpenBLAS bundled with scipy. */
#pragma once

#include <complex.h>

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#define LAPACK_WORK_MEMORY_ERROR -1010

typedef int lapack_int;
typedef double _Complex lapack_complex_double;

#define LAPACKE_zgesvd scipy_LAPACKE_zgesvd
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_zgesv scipy_LAPACKE_zgesv
#define LAPACKE_zgetrf scipy_LAPACKE_zgetrf
#define LAPACKE_zgetrs scipy_LAPACKE_zgetrs
#define LAPACKE_zlaswp scipy_LAPACKE_zlaswp

lapack_int LAPACKE_zgesvd(int layout, char jobu, char jobvt, lapack_int m,
                          lapack_int n, lapack_complex_double *a,
                          lapack_int lda, double *s, lapack_complex_double *u,
                          lapack_int ldu, lapack_complex_double *vt,
                          lapack_int ldvt, double *superb);
lapack_int LAPACKE_dgesvd(int layout, char jobu, char jobvt, lapack_int m,
                          lapack_int n, double *a, lapack_int lda, double *s,
                          double *u, lapack_int ldu, double *vt,
                          lapack_int ldvt, double *superb);
lapack_int LAPACKE_zgesv(int layout, lapack_int n, lapack_int nrhs,
                         lapack_complex_double *a, lapack_int lda,
                         lapack_int *ipiv, lapack_complex_double *b,
                         lapack_int ldb);
lapack_int LAPACKE_zgetrf(int layout, lapack_int m, lapack_int n,
                          lapack_complex_double *a, lapack_int lda,
                          lapack_int *ipiv);
lapack_int LAPACKE_zgetrs(int layout, char trans, lapack_int n,
                          lapack_int nrhs, lapack_complex_double const *a,
                          lapack_int lda, lapack_int const *ipiv,
                          lapack_complex_double *b, lapack_int ldb);
lapack_int LAPACKE_zlaswp(int layout, lapack_int n, lapack_complex_double *a,
                          lapack_int lda, lapack_int k1, lapack_int k2,
                          lapack_int const *ipiv, lapack_int incx);
