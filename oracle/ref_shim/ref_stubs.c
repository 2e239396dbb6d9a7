/* Test infrastructure (oracle build only): stand-ins for the few external
 * routines the reference library references but that are absent here
 * (ARPACK's reverse-communication eigensolver and the SuiteSparse-backed
 * sparse LU).  None of them lies on the Helmholtz butterfly path; each one
 * aborts loudly if reached. */
#include <stdio.h>
#include <stdlib.h>

#define ORACLE_STUB(name)                                              \
  void name(void) {                                                    \
    fprintf(stderr, "oracle build: %s is not available\n", #name);     \
    abort();                                                           \
  }

ORACLE_STUB(dnaupd_c)
ORACLE_STUB(dneupd_c)
ORACLE_STUB(bfLuCsrRealNew)
ORACLE_STUB(bfLuCsrRealInit)
ORACLE_STUB(bfLuCsrRealSolveVec)
ORACLE_STUB(bfLuCsrRealDeinitAndDealloc)
