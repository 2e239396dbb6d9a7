/* The BfMatFunc adapter of bfmat_gpu.h (compiled against the reference's
 * headers and linked with its library and libbfg). */
#include "bfmat_gpu.h"

#include <complex.h>
#include <stdlib.h>
#include <string.h>

#include <bf/error.h>
#include <bf/mat_dense_complex.h>
#include <bf/mat_func.h>

void gpuHelm2SetError(bfgStatus st) {
  if (st == BFG_OK) return;
  bfSetError(st >= 1 && st <= 8 ? (enum BfError)st : BF_ERROR_RUNTIME_ERROR);
}

BfMat *gpuHelm2Mul(BfMat const *X, void *aux) {
  GpuHelm2 *g = aux;
  if (!bfMatInstanceOf(X, BF_TYPE_MAT_DENSE_COMPLEX)) {
    bfSetError(BF_ERROR_TYPE_ERROR);
    return NULL;
  }
  BfMatDenseComplex const *x = bfMatConstToMatDenseComplexConst(X);
  int64_t const R = (int64_t)bfMatGetNumCols(X);
  if ((int64_t)bfMatGetNumRows(X) != g->numCols) {
    bfSetError(BF_ERROR_INCOMPATIBLE_SHAPES);
    return NULL;
  }
  /* the operand as row-major rows of R entries with leading dimension
   * rowStride; a view with a column stride other than 1 is copied first */
  BfComplex const *xd = x->data;
  int64_t ldx = (int64_t)x->rowStride;
  BfComplex *tmp = NULL;
  if (x->colStride != 1) {
    tmp = malloc(sizeof(BfComplex) * (size_t)(g->numCols * R));
    if (!tmp) {
      bfSetError(BF_ERROR_MEMORY_ERROR);
      return NULL;
    }
    for (int64_t i = 0; i < g->numCols; ++i)
      for (int64_t j = 0; j < R; ++j)
        tmp[i * R + j] = x->data[i * x->rowStride + j * x->colStride];
    xd = tmp;
    ldx = R;
  }
  BfMatDenseComplex *y = bfMatDenseComplexNew();
  bfMatDenseComplexInit(y, (BfSize)g->numRows, (BfSize)R);
  if (bfGetError()) {
    free(tmp);
    return NULL;
  }
  bfgStatus const st = g->apply(g->fac, g->precision, (double const *)xd, ldx, R,
                                (double *)y->data, (int64_t)y->rowStride, 0);
  free(tmp);
  if (st != BFG_OK) {
    gpuHelm2SetError(st);
    bfMatDenseComplexDeinitAndDealloc(&y);
    return NULL;
  }
  return bfMatDenseComplexToMat(y);
}

BfMat *gpuHelm2Wrap(GpuHelm2 *g, bfgFac fac, int64_t numRows, int64_t numCols) {
  g->fac = fac;
  g->numRows = numRows;
  g->numCols = numCols;
  if (!g->apply) g->apply = bfgFacApplyHost;
  BfMatFunc *f = bfMatFuncNew();
  bfMatFuncInit(f, (BfSize)numRows, (BfSize)numCols, gpuHelm2Mul, g);
  if (bfGetError()) return NULL;
  return bfMatFuncToMat(f);
}

BfMat *gpuHelm2Make(GpuHelm2 *g, bfgContext ctx, BfHelm2 const *helm, BfPoints2 const *src,
                    BfVectors2 const *srcNormals, BfPoints2 const *tgt,
                    BfVectors2 const *tgtNormals) {
  bfgHelm2 h;
  memset(&h, 0, sizeof h);
  h.k = helm->k;
  h.layerPot = (int32_t)helm->layerPot;
  h.alphaRe = creal(helm->alpha);
  h.alphaIm = cimag(helm->alpha);
  h.betaRe = creal(helm->beta);
  h.betaIm = cimag(helm->beta);
  bfgFac fac = NULL;
  bfgStatus const st = bfgFacHelm2MakeMultilevel(
      ctx, &h, (double const *)src->data, srcNormals ? (double const *)srcNormals->data : NULL,
      (int64_t)src->size, (double const *)tgt->data,
      tgtNormals ? (double const *)tgtNormals->data : NULL, (int64_t)tgt->size, NULL, &fac);
  if (st != BFG_OK) {
    gpuHelm2SetError(st);
    return NULL;
  }
  return gpuHelm2Wrap(g, fac, (int64_t)tgt->size, (int64_t)src->size);
}
