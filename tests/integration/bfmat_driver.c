/* Drives the BfMatFunc adapter (bfmat_gpu.c) through the reference's own
 * bfMatMul (mat.c:183-185) and bfSolveGMRES (linalg.c:47-317), with the
 * adapter's host apply replaced by a host stand-in (a dense product on the
 * CPU), so that it runs without a GPU; the reference's BfMatDenseComplex
 * product of the same matrix is the expected result.  Prints one line per
 * check and exits non-zero on the first failure. */
#include <complex.h>
#include <math.h>
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <sys/wait.h>
#include <unistd.h>

#include <bf/error.h>
#include <bf/linalg.h>
#include <bf/mat_dense_complex.h>
#include <bf/rand.h>

#include "bfmat_gpu.h"

static int64_t gN;
static BfComplex *gA;          /* row-major gN x gN */
static bfgStatus gFail = BFG_OK;
static int64_t gCalls = 0;

/* stand-in for bfgFacApplyHost: Y = A X on the host, same arguments */
static bfgStatus standinApply(bfgFac fac, bfgPrecision precision, double const *X, int64_t ldx,
                              int64_t R, double *Y, int64_t ldy, uint32_t flags) {
  (void)fac;
  ++gCalls;
  if (gFail != BFG_OK) return gFail;
  if (precision != BFG_PRECISION_FP64 || flags != 0 || ldx < R || ldy < R) return BFG_ERROR_INVALID_ARGUMENTS;
  BfComplex const *x = (BfComplex const *)X;
  BfComplex *y = (BfComplex *)Y;
  for (int64_t i = 0; i < gN; ++i)
    for (int64_t r = 0; r < R; ++r) {
      BfComplex s = 0;
      for (int64_t j = 0; j < gN; ++j) s += gA[i * gN + j] * x[j * ldx + r];
      y[i * ldy + r] = s;
    }
  return BFG_OK;
}

static double relDiff(BfMat const *a, BfMat const *b) {
  BfMatDenseComplex const *x = bfMatConstToMatDenseComplexConst(a);
  BfMatDenseComplex const *y = bfMatConstToMatDenseComplexConst(b);
  double num = 0, den = 0;
  for (BfSize i = 0; i < bfMatGetNumRows(a); ++i)
    for (BfSize j = 0; j < bfMatGetNumCols(a); ++j) {
      BfComplex u = x->data[i * x->rowStride + j * x->colStride];
      BfComplex v = y->data[i * y->rowStride + j * y->colStride];
      num += cabs(u - v) * cabs(u - v);
      den += cabs(v) * cabs(v);
    }
  return sqrt(num / den);
}

#define CHECK(cond, what)                       \
  do {                                          \
    if (!(cond)) {                              \
      printf("FAIL %s\n", what);                \
      return 1;                                 \
    }                                           \
    printf("ok %s\n", what);                    \
  } while (0)

int main(void) {
  /* libbfg itself links and answers (a host-only call) */
  bfgFacOptions o;
  bfgFacOptionsDefault(&o);
  CHECK(o.leafSize == 1 && o.pinvCut == 0, "libbfg bfgFacOptionsDefault");

  gN = 40;
  bfSeed(5);
  BfMatDenseComplex *Ad = bfMatDenseComplexNewRandn((BfSize)gN, (BfSize)gN);
  gA = malloc(sizeof(BfComplex) * (size_t)(gN * gN));
  for (int64_t i = 0; i < gN; ++i)
    for (int64_t j = 0; j < gN; ++j) {
      /* well conditioned: I + 0.1 randn / sqrt(n) */
      BfComplex v = 0.1 * Ad->data[i * Ad->rowStride + j] / sqrt((double)gN) + (i == j ? 1.0 : 0.0);
      Ad->data[i * Ad->rowStride + j] = v;
      gA[i * gN + j] = v;
    }

  GpuHelm2 g = {0};
  g.apply = standinApply;
  g.precision = BFG_PRECISION_FP64;
  BfMat *A = gpuHelm2Wrap(&g, NULL, gN, gN);
  CHECK(A != NULL && bfMatGetNumRows(A) == (BfSize)gN && bfMatGetNumCols(A) == (BfSize)gN,
        "BfMatFunc wrap, shape through the reference's dispatchers");

  /* bfMatMul through the adapter against the reference's dense product */
  BfMatDenseComplex *X = bfMatDenseComplexNewRandn((BfSize)gN, 3);
  BfMat *Y1 = bfMatMul(A, bfMatDenseComplexToMat(X));
  BfMat *Y2 = bfMatMul(bfMatDenseComplexToMat(Ad), bfMatDenseComplexToMat(X));
  CHECK(Y1 && Y2 && bfMatInstanceOf(Y1, BF_TYPE_MAT_DENSE_COMPLEX), "bfMatMul result type");
  double e = relDiff(Y1, Y2);
  printf("bfMatMul rel diff %.3e\n", e);
  CHECK(e < 1e-14, "bfMatMul through the adapter equals the dense product");

  /* a column-range view (rowStride > numCols) goes through as a strided operand */
  BfMat *Xv = bfMatDenseComplexGetColRange(X, 1, 3);
  BfMatDenseComplex const *xv = bfMatConstToMatDenseComplexConst(Xv);
  CHECK(xv->rowStride == 3 && bfMatGetNumCols(Xv) == 2, "column-range view is strided");
  BfMat *Y3 = bfMatMul(A, Xv);
  BfMat *Y4 = bfMatMul(bfMatDenseComplexToMat(Ad), Xv);
  e = relDiff(Y3, Y4);
  printf("strided view rel diff %.3e\n", e);
  CHECK(e < 1e-14, "bfMatMul on a strided view");

  /* the reference's GMRES with the adapter as its operator */
  BfMatDenseComplex *Bm = bfMatDenseComplexNewRandn((BfSize)gN, 1);
  BfSize numIter = 0;
  int64_t calls0 = gCalls;
  BfMat *Xs = bfSolveGMRES(A, bfMatDenseComplexToMat(Bm), NULL, 1e-12, (BfSize)gN, &numIter, NULL);
  CHECK(Xs != NULL && gCalls > calls0, "bfSolveGMRES ran on the adapter");
  BfMat *AX = bfMatMul(bfMatDenseComplexToMat(Ad), Xs);
  e = relDiff(AX, bfMatDenseComplexToMat(Bm));
  printf("bfSolveGMRES: %zu iterations, adapter calls %lld, residual %.3e\n", (size_t)numIter,
         (long long)(gCalls - calls0), e);
  CHECK(e < 1e-10, "bfSolveGMRES solution through the adapter");

  /* A libbfg failure becomes the reference's error code.  The reference
   * treats any error as fatal (bfSetError asserts, error.c:20-24; most
   * callers BF_DIE), so the check runs in a child process: the failing call
   * must end it by that route, not return a result. */
  fflush(stdout);
  pid_t pid = fork();
  if (pid == 0) {
    gFail = BFG_ERROR_MEMORY;
    BfMat *Yf = gpuHelm2Mul(bfMatDenseComplexToMat(X), &g);
    (void)Yf;
    _exit(0);                   /* reached only if the failure was swallowed */
  }
  int status = 0;
  waitpid(pid, &status, 0);
  CHECK(WIFSIGNALED(status) && WTERMSIG(status) == SIGABRT,
        "a failing apply ends in the reference's error handling");
  pid = fork();
  if (pid == 0) {
    BfHelm2 helm = {.k = 10.0, .layerPot = BF_LAYER_POTENTIAL_SINGLE, .alpha = 0, .beta = 0};
    BfPoints2 pts = {0};
    GpuHelm2 g2 = {0};
    BfMat *F = gpuHelm2Make(&g2, NULL, &helm, &pts, NULL, &pts, NULL);
    (void)F;
    _exit(0);
  }
  waitpid(pid, &status, 0);
  CHECK(WIFSIGNALED(status) && WTERMSIG(status) == SIGABRT,
        "a refused factorization ends in the reference's error handling");
  printf("all ok\n");
  return 0;
}
