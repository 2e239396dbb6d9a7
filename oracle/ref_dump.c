/* Test infrastructure: golden-data driver linked against the reference
 * library built by oracle/build_ref.sh.  It drives the reference's own code
 * path for the Helmholtz multilevel butterfly and writes what the parity
 * tests need:
 *
 *   ref_dump rng <seed> <n> <out.f64>
 *       n draws of bfRealUniform1 after bfSeed(seed), then 2n doubles of
 *       bfComplexRandn(n) after bfSeed(seed) again (rand.c:19-76).
 *
 *   ref_dump fac <outdir> <k> <src.f64> <tgt.f64> <R> <xseed> <ndense> <blocks>
 *       src/tgt: raw float64 (N,2) point files.  Builds both quadtrees
 *       (quadtree.c:80-98), runs bfFacHelm2MakeMultilevel with the
 *       single-layer kernel (fac_helm2.c:943-1002), draws X (n_src x R,
 *       tree order) with bfSeed(xseed) + bfComplexRandn, applies with
 *       bfMatMul (mat.c:183-185), and evaluates `ndense` dense kernel rows
 *       (helm2.c:282-319) for the dense comparison.  Writes
 *         src_perm.u64 tgt_perm.u64     tree position -> original index
 *         plan.txt                      block structure of the factorization
 *         blocks.c128                   every stored block (if blocks != 0)
 *         x.c128 y_bf.c128              X and A*X, tree order, row-major
 *         dense_rows.u64 y_dense.c128   sampled rows (tree order) of K*X
 *         stats.txt                     wall times and bfMatNumBytes
 *
 * The plan.txt grammar (written identically by the Python oracle and by the
 * library's plan export):
 *   BD nr nc / RO ... / CO ...   block-dense; then nr*nc children row-major
 *   PR nf                        product; then factors 0..nf-1 as stored
 *   DG nb / RO ... / CO ...      block-diagonal; then nb lines "B m n"
 *   CB nr nc nb / RO ... / CO .. block-COO; then nb lines "B ri ci m n"
 *   DC m n                       dense complex block
 */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <bf/fac_helm2.h>
#include <bf/helm2.h>
#include <bf/layer_pot.h>
#include <bf/mat.h>
#include <bf/mat_block.h>
#include <bf/mat_block_coo.h>
#include <bf/mat_block_dense.h>
#include <bf/mat_block_diag.h>
#include <bf/mat_dense_complex.h>
#include <bf/mat_product.h>
#include <bf/points.h>
#include <bf/quadtree.h>
#include <bf/rand.h>
#include <bf/tree.h>
#include <bf/types.h>

static double wallSeconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static double *readPoints(char const *path, size_t *n) {
  FILE *fp = fopen(path, "rb");
  if (!fp) { perror(path); exit(2); }
  fseek(fp, 0, SEEK_END);
  long bytes = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  *n = (size_t)bytes / (2 * sizeof(double));
  double *xy = malloc(bytes);
  if (fread(xy, 1, bytes, fp) != (size_t)bytes) { perror(path); exit(2); }
  fclose(fp);
  return xy;
}

static void writeRaw(char const *dir, char const *name, void const *data, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE *fp = fopen(path, "wb");
  if (!fp) { perror(path); exit(2); }
  fwrite(data, 1, bytes, fp);
  fclose(fp);
}

static void printOffsets(FILE *fp, char const *tag, BfSize const *off, BfSize n) {
  fprintf(fp, "%s", tag);
  for (BfSize i = 0; i <= n; ++i) fprintf(fp, " %zu", off[i]);
  fprintf(fp, "\n");
}

static void dumpDense(FILE *blk, BfMat const *mat) {
  if (!blk) return;
  BfMatDenseComplex const *d = bfMatConstToMatDenseComplexConst(mat);
  BfSize m = bfMatGetNumRows(mat), n = bfMatGetNumCols(mat);
  for (BfSize i = 0; i < m; ++i)
    for (BfSize j = 0; j < n; ++j) {
      BfComplex z = d->data[i * d->rowStride + j * d->colStride];
      fwrite(&z, sizeof z, 1, blk);
    }
}

static void dumpPlan(FILE *fp, FILE *blk, BfMat const *mat) {
  BfType type = bfMatGetType(mat);
  if (type == BF_TYPE_MAT_BLOCK_DENSE) {
    BfMatBlock const *mb = (BfMatBlock const *)mat;
    BfSize nr = bfMatBlockGetNumRowBlocks(mb), nc = bfMatBlockGetNumColBlocks(mb);
    fprintf(fp, "BD %zu %zu\n", nr, nc);
    printOffsets(fp, "RO", mb->rowOffset, nr);
    printOffsets(fp, "CO", mb->colOffset, nc);
    for (BfSize i = 0; i < nr; ++i)
      for (BfSize j = 0; j < nc; ++j)
        dumpPlan(fp, blk, mb->block[i * nc + j]);
  } else if (type == BF_TYPE_MAT_PRODUCT) {
    BfMatProduct const *prod = (BfMatProduct const *)mat;
    BfSize nf = bfMatProductNumFactors(prod);
    fprintf(fp, "PR %zu\n", nf);
    for (BfSize i = 0; i < nf; ++i)
      dumpPlan(fp, blk, bfMatProductGetFactorConst(prod, i));
  } else if (type == BF_TYPE_MAT_BLOCK_DIAG) {
    BfMatBlock const *mb = (BfMatBlock const *)mat;
    BfSize nb = bfMatBlockDiagNumBlocks((BfMatBlockDiag const *)mat);
    fprintf(fp, "DG %zu\n", nb);
    printOffsets(fp, "RO", mb->rowOffset, nb);
    printOffsets(fp, "CO", mb->colOffset, nb);
    for (BfSize i = 0; i < nb; ++i) {
      fprintf(fp, "B %zu %zu\n", bfMatGetNumRows(mb->block[i]), bfMatGetNumCols(mb->block[i]));
      dumpDense(blk, mb->block[i]);
    }
  } else if (type == BF_TYPE_MAT_BLOCK_COO) {
    BfMatBlock const *mb = (BfMatBlock const *)mat;
    BfMatBlockCoo const *coo = (BfMatBlockCoo const *)mat;
    BfSize nr = bfMatBlockGetNumRowBlocks(mb), nc = bfMatBlockGetNumColBlocks(mb);
    BfSize nb = bfMatBlockCooNumBlocks(coo);
    fprintf(fp, "CB %zu %zu %zu\n", nr, nc, nb);
    printOffsets(fp, "RO", mb->rowOffset, nr);
    printOffsets(fp, "CO", mb->colOffset, nc);
    for (BfSize k = 0; k < nb; ++k) {
      fprintf(fp, "B %zu %zu %zu %zu\n", coo->rowInd[k], coo->colInd[k],
              bfMatGetNumRows(mb->block[k]), bfMatGetNumCols(mb->block[k]));
      dumpDense(blk, mb->block[k]);
    }
  } else if (type == BF_TYPE_MAT_DENSE_COMPLEX) {
    fprintf(fp, "DC %zu %zu\n", bfMatGetNumRows(mat), bfMatGetNumCols(mat));
    dumpDense(blk, mat);
  } else {
    fprintf(stderr, "ref_dump: unexpected matrix type %d\n", (int)type);
    exit(3);
  }
}

static int cmdRng(int argc, char **argv) {
  if (argc != 5) { fprintf(stderr, "usage: ref_dump rng <seed> <n> <out>\n"); return 1; }
  BfSize seed = strtoull(argv[2], NULL, 10), n = strtoull(argv[3], NULL, 10);
  double *out = malloc(3 * n * sizeof(double));
  bfSeed(seed);
  for (BfSize i = 0; i < n; ++i) out[i] = bfRealUniform1();
  bfSeed(seed);
  bfComplexRandn(n, (BfComplex *)(out + n));
  FILE *fp = fopen(argv[4], "wb");
  fwrite(out, sizeof(double), 3 * n, fp);
  fclose(fp);
  free(out);
  return 0;
}

static int cmdFac(int argc, char **argv) {
  if (argc != 10) {
    fprintf(stderr, "usage: ref_dump fac <outdir> <k> <src> <tgt> <R> <xseed> <ndense> <blocks>\n");
    return 1;
  }
  char const *outdir = argv[2];
  double k = atof(argv[3]);
  size_t nsrc, ntgt;
  double *srcXy = readPoints(argv[4], &nsrc);
  double *tgtXy = readPoints(argv[5], &ntgt);
  BfSize R = strtoull(argv[6], NULL, 10);
  BfSize xseed = strtoull(argv[7], NULL, 10);
  BfSize ndense = strtoull(argv[8], NULL, 10);
  int dumpBlocks = atoi(argv[9]);

  BfPoints2 srcPts = {.data = (BfPoint2 *)srcXy, .size = nsrc, .capacity = nsrc, .isView = true};
  BfPoints2 tgtPts = {.data = (BfPoint2 *)tgtXy, .size = ntgt, .capacity = ntgt, .isView = true};

  BfHelm2 helm = {.k = k, .layerPot = BF_LAYER_POTENTIAL_SINGLE, .alpha = 0, .beta = 0};

  double t0 = wallSeconds();
  BfQuadtree srcTree, tgtTree;
  bfQuadtreeInit(&srcTree, &srcPts, NULL);
  bfQuadtreeInit(&tgtTree, &tgtPts, NULL);
  double tTree = wallSeconds() - t0;

  BfPerm const *srcPerm = bfTreeGetPermConst(bfQuadtreeToTree(&srcTree));
  BfPerm const *tgtPerm = bfTreeGetPermConst(bfQuadtreeToTree(&tgtTree));
  writeRaw(outdir, "src_perm.u64", srcPerm->index, nsrc * sizeof(BfSize));
  writeRaw(outdir, "tgt_perm.u64", tgtPerm->index, ntgt * sizeof(BfSize));

  t0 = wallSeconds();
  BfMat *A = bfFacHelm2MakeMultilevel(&helm, &srcTree, &tgtTree);
  double tFac = wallSeconds() - t0;

  char path[4096];
  snprintf(path, sizeof path, "%s/plan.txt", outdir);
  FILE *fp = fopen(path, "w");
  FILE *blk = NULL;
  if (dumpBlocks) {
    snprintf(path, sizeof path, "%s/blocks.c128", outdir);
    blk = fopen(path, "wb");
  }
  dumpPlan(fp, blk, A);
  fclose(fp);
  if (blk) fclose(blk);

  bfSeed(xseed);
  BfMat *X = bfMatDenseComplexToMat(bfMatDenseComplexNewRandn(nsrc, R));
  writeRaw(outdir, "x.c128", bfMatToMatDenseComplex(X)->data, nsrc * R * sizeof(BfComplex));

  /* one warm-up apply, then the median of five timed ones */
  BfMat *Y = bfMatMul(A, X);
  double tApply[5];
  for (int rep = 0; rep < 5; ++rep) {
    bfMatDelete(&Y);
    t0 = wallSeconds();
    Y = bfMatMul(A, X);
    tApply[rep] = wallSeconds() - t0;
  }
  for (int a = 0; a < 5; ++a)
    for (int b = a + 1; b < 5; ++b)
      if (tApply[b] < tApply[a]) { double t = tApply[a]; tApply[a] = tApply[b]; tApply[b] = t; }
  BfMatDenseComplex *Yd = bfMatToMatDenseComplex(Y);
  BfComplex *ybuf = malloc(ntgt * R * sizeof(BfComplex));
  for (BfSize i = 0; i < ntgt; ++i)
    for (BfSize r = 0; r < R; ++r)
      ybuf[i * R + r] = Yd->data[i * Yd->rowStride + r * Yd->colStride];
  writeRaw(outdir, "y_bf.c128", ybuf, ntgt * R * sizeof(BfComplex));

  /* Dense rows: evenly spaced tree-order target rows, all source columns
   * (tree order), evaluated with the reference's own kernel matrix. */
  if (ndense > ntgt) ndense = ntgt;
  BfSize *rows = malloc((ndense ? ndense : 1) * sizeof(BfSize));
  BfComplex *yd = calloc((ndense ? ndense : 1) * R, sizeof(BfComplex));
  if (ndense) {
    BfPoints2 *tgtSel = bfPoints2NewWithCapacity(ndense);
    for (BfSize s = 0; s < ndense; ++s) {
      rows[s] = (s * ntgt) / ndense;
      BfSize orig = tgtPerm->index[rows[s]];
      bfPoints2Append(tgtSel, tgtXy + 2 * orig);
    }
    BfSize chunk = 4096;
    BfComplex const *xd = bfMatToMatDenseComplex(X)->data;
    for (BfSize j0 = 0; j0 < nsrc; j0 += chunk) {
      BfSize j1 = j0 + chunk < nsrc ? j0 + chunk : nsrc;
      BfPoints2 *srcSel = bfPoints2NewWithCapacity(j1 - j0);
      for (BfSize j = j0; j < j1; ++j)
        bfPoints2Append(srcSel, srcXy + 2 * srcPerm->index[j]);
      BfMat *K = bfHelm2GetKernelMatrix(&helm, srcSel, tgtSel, NULL, NULL);
      BfMatDenseComplex const *Kd = bfMatConstToMatDenseComplexConst(K);
      for (BfSize s = 0; s < ndense; ++s)
        for (BfSize j = j0; j < j1; ++j) {
          BfComplex kij = Kd->data[s * Kd->rowStride + (j - j0) * Kd->colStride];
          for (BfSize r = 0; r < R; ++r)
            yd[s * R + r] += kij * xd[j * R + r];
        }
      bfMatDelete(&K);
      bfPoints2DeinitAndDealloc(&srcSel);
    }
    bfPoints2DeinitAndDealloc(&tgtSel);
  }
  writeRaw(outdir, "dense_rows.u64", rows, ndense * sizeof(BfSize));
  writeRaw(outdir, "y_dense.c128", yd, ndense * R * sizeof(BfComplex));

  snprintf(path, sizeof path, "%s/stats.txt", outdir);
  fp = fopen(path, "w");
  fprintf(fp, "tree_s %.6f\nfac_s %.6f\napply_median_s %.6f\nnum_bytes %zu\n",
          tTree, tFac, tApply[2], bfMatNumBytes(A));
  fclose(fp);

  free(rows); free(yd); free(ybuf);
  bfMatDelete(&Y);
  bfMatDelete(&X);
  bfMatDelete(&A);
  return 0;
}

int main(int argc, char **argv) {
  if (argc >= 2 && !strcmp(argv[1], "rng")) return cmdRng(argc, argv);
  if (argc >= 2 && !strcmp(argv[1], "fac")) return cmdFac(argc, argv);
  fprintf(stderr, "usage: ref_dump rng|fac ...\n");
  return 1;
}
