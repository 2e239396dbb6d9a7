/* A libbfg factorization as a reference BfMat, through the reference's
 * callback operator BfMatFunc (mat_func.h:5-28) -- the way its drivers wrap
 * the FMM operator (multiple_scattering_context.c:538-542) -- so that
 * bfMatMul (mat.c:183-185) and bfSolveGMRES (linalg.c:47-317) run on the GPU
 * factorization with no change to the reference's own sources. */
#pragma once

#include <bf/mat.h>
#include <bf/helm2.h>
#include <bf/points.h>
#include <bf/vectors.h>

#include "bfg.h"

/* the host-operand apply the callback issues: bfgFacApplyHost by default */
typedef bfgStatus (*BfgHostApplyFn)(bfgFac fac, bfgPrecision precision, double const *X,
                                    int64_t ldx, int64_t numRhs, double *Y, int64_t ldy,
                                    uint32_t flags);

typedef struct {
  bfgFac fac;
  int64_t numRows, numCols;
  bfgPrecision precision;
  BfgHostApplyFn apply;
} GpuHelm2;

/* BfMatFunc callback: X is a BfMatDenseComplex n x R with rows in tree
 * order, as bfMatMul takes it; returns a new BfMatDenseComplex (owned by the
 * caller), or NULL with the reference's error code set. */
BfMat *gpuHelm2Mul(BfMat const *X, void *aux);

/* Wraps an existing factorization (shape numRows x numCols). */
BfMat *gpuHelm2Wrap(GpuHelm2 *g, bfgFac fac, int64_t numRows, int64_t numCols);

/* bfQuadtreeInit x 2 + bfFacHelm2MakeMultilevel (fac_helm2.c:943) on the
 * GPU, wrapped; NULL with the reference's error code set on failure. */
BfMat *gpuHelm2Make(GpuHelm2 *g, bfgContext ctx, BfHelm2 const *helm, BfPoints2 const *src,
                    BfVectors2 const *srcNormals, BfPoints2 const *tgt,
                    BfVectors2 const *tgtNormals);

/* a bfgStatus as the reference's BfError (the codes 1-8 are the same) */
void gpuHelm2SetError(bfgStatus st);
