/* Test infrastructure (oracle build only): ARPACK is not available here.  The
 * reference's eigensolver (used only by its Laplace-Beltrami code, not by the
 * Helmholtz butterfly path) is declared so that the library compiles; the
 * stubs in ref_stubs.c abort if it is ever called. */
#pragma once

#include <complex.h>

typedef int a_int;

void dnaupd_c(a_int *ido, char const *bmat, a_int n, char const *which,
              a_int nev, double tol, double *resid, a_int ncv, double *v,
              a_int ldv, a_int *iparam, a_int *ipntr, double *workd,
              double *workl, a_int lworkl, a_int *info);
void dneupd_c(int rvec, char const *howmny, a_int const *select, double *dr,
              double *di, double *z, a_int ldz, double sigmar, double sigmai,
              double *workev, char const *bmat, a_int n, char const *which,
              a_int nev, double tol, double *resid, a_int ncv, double *v,
              a_int ldv, a_int *iparam, a_int *ipntr, double *workd,
              double *workl, a_int lworkl, a_int *info);
