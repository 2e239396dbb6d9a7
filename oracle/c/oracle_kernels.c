/* Test infrastructure: CPU oracle helpers for the butterfly Helmholtz path.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the correctness reference or the timed CPU
 * baseline; the product never calls it.
 *
 * 1. Kernel matrices restating helm2.c:93-280 with the reference's own
 *    Bessel functions: bf_H0(x) = j0(x) + i y0(x), bf_H1(x) = j1(x) + i y1(x)
 *    from glibc libm (bessel.c:284-308; the GSL branch above it is dead
 *    because def.h:7-8 always defines _DEFAULT_SOURCE).  Distances use
 *    hypot(src - tgt) as bfPoints2PairwiseDists does (points.c:484-505).
 *    Matrices are row-major m x n, rows = targets, columns = sources.
 *
 * 2. A port of the reference's apply (mat_block_dense.c:512-572,
 *    mat_product.c:211-245, mat_block_diag.c:372-407,
 *    mat_block_coo.c:382-425, mat_dense_complex.c:1705-1766) over a flat
 *    list of block products, used as the timed CPU baseline.  Plain C
 *    loops; the parallel variant splits the work over disjoint output row
 *    ranges with OpenMP.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

/* layer potentials, numbered as in layer_pot.h:52-65 */
enum { LP_SINGLE = 1, LP_PV_DOUBLE = 2, LP_PV_NORMAL_DERIV_SINGLE = 3, LP_COMBINED_FIELD = 5 };

void oracle_h0(double const *x, int64_t n, double *out /* 2n: re, im */) {
  for (int64_t i = 0; i < n; ++i) {
    out[2 * i] = j0(x[i]);
    out[2 * i + 1] = y0(x[i]);
  }
}

void oracle_h1(double const *x, int64_t n, double *out) {
  for (int64_t i = 0; i < n; ++i) {
    out[2 * i] = j1(x[i]);
    out[2 * i + 1] = y1(x[i]);
  }
}

/* p points (and unit normals) on a circle, theta_i = (2 pi / p) i, with
 * glibc cos/sin as bfCircle2SamplePoints / SampleUnitNormals do
 * (circle.c:12-58). */
void oracle_circle_points(double cx, double cy, double r, int64_t p,
                          double *pts /* 2p */, double *nrm /* 2p */) {
  double const scale = 6.283185307179586 / (double)p;
  for (int64_t i = 0; i < p; ++i) {
    double theta = scale * i;
    double c = cos(theta), s = sin(theta);
    pts[2 * i] = r * c + cx;
    pts[2 * i + 1] = r * s + cy;
    nrm[2 * i] = c;
    nrm[2 * i + 1] = s;
  }
}

/* Point kernel bfHelm2GetKernelValue(helm, xsrc, xtgt, nsrc, NULL)
 * (helm2.c:61-91) for q < count pairs (source q, target q); NaN at r == 0
 * for the single layer, 0 for the double layer, as get_S_value /
 * get_D_value (helm2.c:38-59). */
int oracle_kernel_pairs(int layerPot, double k, double alphaRe, double alphaIm,
                        double betaRe, double betaIm, double const *sx,
                        double const *sy, double const *snx, double const *sny,
                        double const *tx, double const *ty, int64_t count,
                        cplx *out) {
  cplx const alpha = alphaRe + I * alphaIm, beta = betaRe + I * betaIm;
  for (int64_t q = 0; q < count; ++q) {
    double r = hypot(tx[q] - sx[q], ty[q] - sy[q]);
    cplx S = r == 0 ? NAN : I * (j0(k * r) + I * y0(k * r)) / 4;
    cplx D = 0;
    if (r >= 1e-15) {
      double dot = snx[q] * (tx[q] - sx[q]) + sny[q] * (ty[q] - sy[q]);
      cplx scale = (I / 4) * k * (j1(k * r) + I * y1(k * r)) / r;
      D = scale * dot;
    }
    if (layerPot == LP_SINGLE) out[q] = S;
    else if (layerPot == LP_PV_DOUBLE) out[q] = D;
    else if (layerPot == LP_COMBINED_FIELD) out[q] = alpha * S + beta * D;
    else return -1;
  }
  return 0;
}

/* K[i, j] for target i (tx, ty, tnx, tny) and source j (sx, sy, snx, sny).
 * Normal arrays may be NULL when the layer potential does not use them. */
int oracle_kernel_matrix(int layerPot, double k, double alphaRe, double alphaIm,
                         double betaRe, double betaIm,
                         double const *tx, double const *ty,
                         double const *tnx, double const *tny, int64_t m,
                         double const *sx, double const *sy,
                         double const *snx, double const *sny, int64_t n,
                         cplx *out) {
  cplx const alpha = alphaRe + I * alphaIm, beta = betaRe + I * betaIm;
  if (layerPot != LP_SINGLE && layerPot != LP_PV_DOUBLE &&
      layerPot != LP_PV_NORMAL_DERIV_SINGLE && layerPot != LP_COMBINED_FIELD)
    return -1;
  /* rows are independent: the host cores split them (same values whatever
   * the thread count) */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    for (int64_t j = 0; j < n; ++j) {
      double r = hypot(sx[j] - tx[i], sy[j] - ty[i]);
      cplx z = 0;
      if (layerPot == LP_SINGLE) {
        z = r == 0 ? 0 : I * (j0(k * r) + I * y0(k * r)) / 4;
      } else if (layerPot == LP_PV_DOUBLE) {
        if (r != 0) {
          double dot = snx[j] * (tx[i] - sx[j]) + sny[j] * (ty[i] - sy[j]);
          cplx scale = (I / 4) * k * (j1(k * r) + I * y1(k * r)) / r;
          z = scale * dot;
        }
      } else if (layerPot == LP_PV_NORMAL_DERIV_SINGLE) {
        if (r != 0) {
          double dot = tnx[i] * (tx[i] - sx[j]) + tny[i] * (ty[i] - sy[j]);
          cplx scale = (I / 4) * k * (j1(k * r) + I * y1(k * r)) / r;
          z = scale * dot;
        }
      } else if (layerPot == LP_COMBINED_FIELD) {
        if (r != 0) {
          cplx S = (I / 4) * (j0(k * r) + I * y0(k * r));
          double dot = snx[j] * (tx[i] - sx[j]) + sny[j] * (ty[i] - sy[j]);
          cplx scale = (I / 4) * k * (j1(k * r) + I * y1(k * r)) / r;
          cplx D = scale * dot;
          z = alpha * S + beta * D;
        }
      }
      out[i * n + j] = z;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------
 * Apply port.
 *
 * The factorization is a list of terms.  Each term adds A_t * X[src rows]
 * into Y[tgt rows]; A_t is either a dense block (row-major m x n) or a
 * butterfly product given as factors in application order (the reference
 * stores them in the opposite order and applies from the highest index,
 * mat_product.c:211-245).  Every factor is a list of blocks whose products
 * accumulate into the factor's zero-initialised output (block-diagonal and
 * block-COO factors alike, mat_block_diag.c:372-407, mat_block_coo.c:382-425).
 * Terms that share a group write the same rows and run in list order;
 * different groups write disjoint rows and run concurrently.
 * X and Y are row-major with R columns.
 * ------------------------------------------------------------------------ */
typedef struct {
  int32_t kind; /* 0 = dense block, 1 = butterfly product */
  int32_t group;
  int64_t tgtRow, srcRow;
  int32_t m, n;
  int32_t firstFactor, numFactors;
  int64_t dataOff; /* dense blocks only */
} OracleTerm;

typedef struct {
  int32_t rows, cols;
  int64_t firstBlock;
  int32_t numBlocks, pad;
} OracleFactor;

typedef struct {
  int64_t rowOff, colOff;
  int32_t m, n;
  int64_t dataOff;
} OracleFBlock;

static int gColMajor = 0;

/* Y[m x R] += A[m x n] X[n x R]; A row-major, or column-major when the
 * blocks come straight from the GPU arena. */
static void blockGemmAcc(cplx const *A, int32_t m, int32_t n, cplx const *X,
                         cplx *Y, int64_t R) {
  if (gColMajor) {
    for (int32_t j = 0; j < n; ++j) {
      cplx const *x = X + (int64_t)j * R;
      cplx const *a = A + (int64_t)j * m;
      for (int32_t i = 0; i < m; ++i) {
        cplx *y = Y + (int64_t)i * R;
        cplx const ai = a[i];
        for (int64_t r = 0; r < R; ++r)
          y[r] += ai * x[r];
      }
    }
    return;
  }
  for (int32_t i = 0; i < m; ++i) {
    cplx *y = Y + (int64_t)i * R;
    for (int32_t j = 0; j < n; ++j) {
      cplx a = A[(int64_t)i * n + j];
      cplx const *x = X + (int64_t)j * R;
      for (int64_t r = 0; r < R; ++r)
        y[r] += a * x[r];
    }
  }
}

int oracle_apply_port(int64_t nterm, OracleTerm const *terms,
                      OracleFactor const *factors, OracleFBlock const *fblocks,
                      cplx const *data, cplx const *X, cplx *Y, int64_t nrowsY,
                      int64_t R, int32_t nthreads, int32_t colMajor) {
  gColMajor = colMajor;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  memset(Y, 0, (size_t)nrowsY * R * sizeof(cplx));
  int64_t ngroups = 0;
  for (int64_t t = 0; t < nterm; ++t)
    if (t == 0 || terms[t].group != terms[t - 1].group) ++ngroups;
  int64_t *gstart = malloc((ngroups + 1) * sizeof(int64_t));
  int64_t g = 0;
  for (int64_t t = 0; t < nterm; ++t)
    if (t == 0 || terms[t].group != terms[t - 1].group) gstart[g++] = t;
  gstart[ngroups] = nterm;
  int status = 0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t gi = 0; gi < ngroups; ++gi) {
    for (int64_t t = gstart[gi]; t < gstart[gi + 1]; ++t) {
      OracleTerm const *term = &terms[t];
      cplx const *x = X + term->srcRow * R;
      cplx *y = Y + term->tgtRow * R;
      if (term->kind == 0) {
        blockGemmAcc(data + term->dataOff, term->m, term->n, x, y, R);
        continue;
      }
      cplx *v = NULL;
      cplx const *in = x;
      for (int32_t f = 0; f < term->numFactors; ++f) {
        OracleFactor const *fac = &factors[term->firstFactor + f];
        cplx *w = calloc((size_t)fac->rows * R, sizeof(cplx));
        if (!w) { status = -1; break; }
        for (int32_t b = 0; b < fac->numBlocks; ++b) {
          OracleFBlock const *bl = &fblocks[fac->firstBlock + b];
          blockGemmAcc(data + bl->dataOff, bl->m, bl->n, in + bl->colOff * R,
                       w + bl->rowOff * R, R);
        }
        free(v);
        v = w;
        in = v;
      }
      if (v) {
        for (int64_t i = 0; i < (int64_t)term->m * R; ++i) y[i] += v[i];
        free(v);
      }
    }
  }
  free(gstart);
  return status;
}
