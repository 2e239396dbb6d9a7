// CUDA kernels of the butterfly Helmholtz path (sm_103a).
//
//  * fillBlocksKernel      evaluation (LAST) and dense blocks: fused
//                          points -> distance -> H0/H1 -> complex entry,
//                          written column-major straight into the arena
//                          (helm2.c:93-319, fac_helm2.c:403-509, 741-775).
//  * reexpansionKernel     FIRST/MIDDLE blocks: both proxy kernel matrices
//                          (helm2.c:321-365) plus the pseudo-inverse
//                          least-squares solve (mat_dense_complex.c:1768-1849)
//                          in one CTA.  The SVD is a one-sided (Hestenes)
//                          Jacobi on the stacked matrix M = [Z_equiv^H ;
//                          Z_orig^H]: rotating columns until the top part is
//                          orthogonal gives top = V S and bottom = Z_orig^H U,
//                          so Z_shift = sum_a top_a conj(bottom_a)^T / s_a^2
//                          over kept singular values, with no U or V stored.
//  * applyGemvKernel /     one stage of the staged apply (single / many RHS),
//    applyTileKernel       each item a row chunk of one block row summing its
//                          blocks in order; no atomics, so results are
//                          reproducible bit for bit.
//  * applyReduceKernel     sums the per-product outputs into Y in a fixed
//                          order (the reference's block-dense accumulation,
//                          mat_block_dense.c:512-572), optionally scattering
//                          to original point order.
#include <cuda_runtime.h>

#include <cstdint>

#include "bfg_kernels.cuh"
#include "hankel.cuh"

namespace bfg {

namespace {

constexpr double kTwoPiD = 6.283185307179586;   // const.h BF_TWO_PI
constexpr double kEps = 2.220446049250313e-16;
constexpr int kMaxSweeps = 60;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Kernel value K(x_tgt, x_src) for the layer potential in kp (helm2.c:38-91;
// matrix fills return 0 at r == 0, helm2.c:114, 159-160, 207, 255).
__device__ __forceinline__ double2 kernelValue(KernelParams const &kp, double tx,
                                               double ty, double tnx, double tny,
                                               double sx, double sy, double snx,
                                               double sny) {
  double const r = hypot(sx - tx, sy - ty);
  if (r == 0.0) return make_double2(0.0, 0.0);
  double const kr = kp.k * r;
  if (kp.layerPot == kLpSingle) {
    Bessel01 b = bessel01<false>(kr);
    return make_double2(-0.25 * b.y0, 0.25 * b.j0);          // (i/4) H0
  }
  Bessel01 b = bessel01<true>(kr);
  // (i/4) k H1(kr) / r = (k/(4r)) (-Y1 + i J1)
  double const f = 0.25 * kp.k / r;
  double2 const scale = make_double2(-f * b.y1, f * b.j1);
  if (kp.layerPot == kLpPvDouble) {
    double const dot = snx * (tx - sx) + sny * (ty - sy);
    return make_double2(scale.x * dot, scale.y * dot);
  }
  if (kp.layerPot == kLpPvNormalDerivSingle) {
    double const dot = tnx * (tx - sx) + tny * (ty - sy);
    return make_double2(scale.x * dot, scale.y * dot);
  }
  // combined field alpha S + beta D
  double const dot = snx * (tx - sx) + sny * (ty - sy);
  double2 const S = make_double2(-0.25 * b.y0, 0.25 * b.j0);
  double2 const D = make_double2(scale.x * dot, scale.y * dot);
  double2 const a = cmul(make_double2(kp.alphaRe, kp.alphaIm), S);
  double2 const c = cmul(make_double2(kp.betaRe, kp.betaIm), D);
  return make_double2(a.x + c.x, a.y + c.y);
}

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// LAST and DENSE blocks
// ---------------------------------------------------------------------------
__global__ void fillBlocksKernel(FillDesc const *__restrict__ descs, PointsDev src,
                                 PointsDev tgt, KernelParams kp, double2 *arena,
                                 int32_t *status) {
  extern __shared__ double proxy[];   // 4 * n for LAST blocks
  FillDesc const d = descs[blockIdx.x];
  int const m = d.m, n = d.n;
  double2 *out = arena + d.arenaOff;
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;
  bool const useTgtN = kp.layerPot == kLpPvNormalDerivSingle;
  if (d.kind == kLast) {
    double const scale = kTwoPiD / (double)n;
    for (int b = threadIdx.x; b < n; b += blockDim.x) {
      double s, c;
      sincos(scale * b, &s, &c);
      proxy[b] = d.ceq[2] * c + d.ceq[0];
      proxy[n + b] = d.ceq[2] * s + d.ceq[1];
      proxy[2 * n + b] = c;
      proxy[3 * n + b] = s;
    }
    __syncthreads();
    int64_t const total = (int64_t)m * n;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      int const i = (int)(e % m), j = (int)(e / m);
      int64_t const ti = d.t0 + i;
      out[e] = kernelValue(kp, tgt.x[ti], tgt.y[ti], useTgtN ? tgt.nx[ti] : 0.0,
                           useTgtN ? tgt.ny[ti] : 0.0, proxy[j], proxy[n + j],
                           useSrcN ? proxy[2 * n + j] : 0.0,
                           useSrcN ? proxy[3 * n + j] : 0.0);
    }
  } else if (d.kind == kDense) {
    int64_t const total = (int64_t)m * n;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      int const i = (int)(e % m), j = (int)(e / m);
      int64_t const ti = d.t0 + i, sj = d.s0 + j;
      out[e] = kernelValue(kp, tgt.x[ti], tgt.y[ti], useTgtN ? tgt.nx[ti] : 0.0,
                           useTgtN ? tgt.ny[ti] : 0.0, src.x[sj], src.y[sj],
                           useSrcN ? src.nx[sj] : 0.0, useSrcN ? src.ny[sj] : 0.0);
    }
  } else if (threadIdx.x == 0) {
    atomicOr(status, kStatusBadDescriptor);
  }
}

// ---------------------------------------------------------------------------
// FIRST and MIDDLE blocks: proxy fills + Jacobi pseudo-inverse re-expansion
// ---------------------------------------------------------------------------
template <bool kSmem>
__global__ void reexpansionKernel(FillDesc const *__restrict__ descs, PointsDev src,
                                  KernelParams kp, int32_t cutMode, double cutTol,
                                  double2 *arena, double2 *scratch,
                                  int64_t const *scratchOff, int32_t *status) {
  extern __shared__ double2 smem2[];
  FillDesc const d = descs[blockIdx.x];
  int const p = d.m, n = d.n, LD = p + n;
  double2 *M = kSmem ? smem2 : scratch + scratchOff[blockIdx.x];
  double *geo = reinterpret_cast<double *>(kSmem ? smem2 + (int64_t)LD * p : smem2);
  double *chkX = geo, *chkY = geo + p;
  double *eqX = geo + 2 * p, *eqY = geo + 3 * p, *eqNx = geo + 4 * p, *eqNy = geo + 5 * p;
  double *orX = geo + 6 * p, *orY = orX + n, *orNx = orX + 2 * n, *orNy = orX + 3 * n;
  double *wgt = orX + 4 * n;
  __shared__ int sRotated;

  int const tid = threadIdx.x, nthr = blockDim.x;
  int const lane = tid & 31, warp = tid >> 5, nWarps = nthr >> 5;
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;

  // proxy geometry: check points on cchk and equivalent sources on ceq share
  // theta_a = (2 pi / p) a (circle.c:12-58)
  {
    double const scale = kTwoPiD / (double)p;
    for (int a = tid; a < p; a += nthr) {
      double s, c;
      sincos(scale * a, &s, &c);
      chkX[a] = d.cchk[2] * c + d.cchk[0];
      chkY[a] = d.cchk[2] * s + d.cchk[1];
      eqX[a] = d.ceq[2] * c + d.ceq[0];
      eqY[a] = d.ceq[2] * s + d.ceq[1];
      eqNx[a] = c;
      eqNy[a] = s;
    }
    if (d.kind == kFirst) {
      for (int b = tid; b < n; b += nthr) {
        int64_t const sj = d.s0 + b;
        orX[b] = src.x[sj];
        orY[b] = src.y[sj];
        orNx[b] = (useSrcN && src.nx) ? src.nx[sj] : 0.0;
        orNy[b] = (useSrcN && src.ny) ? src.ny[sj] : 0.0;
      }
    } else {
      double const scale2 = kTwoPiD / (double)n;
      for (int b = tid; b < n; b += nthr) {
        double s, c;
        sincos(scale2 * b, &s, &c);
        orX[b] = d.corig[2] * c + d.corig[0];
        orY[b] = d.corig[2] * s + d.corig[1];
        orNx[b] = c;
        orNy[b] = s;
      }
    }
  }
  __syncthreads();

  // M[a*LD + r] = conj(K(chk_a, src_r)), src_r = eq_r (r < p) or orig_{r-p}
  {
    int64_t const total = (int64_t)LD * p;
    for (int64_t e = tid; e < total; e += nthr) {
      int const a = (int)(e / LD), r = (int)(e % LD);
      double sx, sy, snx, sny;
      if (r < p) {
        sx = eqX[r]; sy = eqY[r]; snx = eqNx[r]; sny = eqNy[r];
      } else {
        sx = orX[r - p]; sy = orY[r - p]; snx = orNx[r - p]; sny = orNy[r - p];
      }
      double2 v = kernelValue(kp, chkX[a], chkY[a], 0.0, 0.0, sx, sy, snx, sny);
      M[e] = make_double2(v.x, -v.y);
    }
  }
  __syncthreads();

  // one-sided Jacobi, round-robin pair schedule
  int const P = p + (p & 1);
  int const nPairs = P / 2;
  double const tolRot = kEps * sqrt((double)p);
  bool converged = false;
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    if (tid == 0) sRotated = 0;
    __syncthreads();
    for (int round = 0; round < P - 1; ++round) {
      for (int pr = warp; pr < nPairs; pr += nWarps) {
        int i, j;
        if (pr == 0) {
          i = round;
          j = P - 1;
        } else {
          i = (round + pr) % (P - 1);
          j = (round - pr + (P - 1)) % (P - 1);
        }
        if (i >= p || j >= p) continue;
        double2 *ci = M + (int64_t)i * LD, *cj = M + (int64_t)j * LD;
        double al = 0, be = 0, gr = 0, gi = 0;
        for (int r = lane; r < p; r += 32) {
          double2 x = ci[r], y = cj[r];
          al += x.x * x.x + x.y * x.y;
          be += y.x * y.x + y.y * y.y;
          gr += x.x * y.x + x.y * y.y;     // conj(x) y
          gi += x.x * y.y - x.y * y.x;
        }
        al = warpSum(al);
        be = warpSum(be);
        gr = warpSum(gr);
        gi = warpSum(gi);
        double const ag = sqrt(gr * gr + gi * gi);
        if (ag > tolRot * sqrt(al * be) && ag > 0.0) {
          double const zeta = (be - al) / (2.0 * ag);
          double const t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          double const c = 1.0 / sqrt(1.0 + t * t), s = c * t;
          double const er = gr / ag, ei = -gi / ag;   // exp(-i phi) = conj(gamma)/|gamma|
          for (int r = lane; r < LD; r += 32) {
            double2 x = ci[r], y = cj[r];
            double const ytr = y.x * er - y.y * ei, yti = y.x * ei + y.y * er;
            ci[r] = make_double2(c * x.x - s * ytr, c * x.y - s * yti);
            cj[r] = make_double2(s * x.x + c * ytr, s * x.y + c * yti);
          }
          if (lane == 0) sRotated = 1;
        }
      }
      __syncthreads();
    }
    int const rotated = sRotated;
    __syncthreads();
    if (!rotated) {
      converged = true;
      break;
    }
  }
  if (!converged && tid == 0) atomicOr(status, kStatusJacobiNotConverged);

  // singular values and the pseudo-inverse cut (mat_dense_complex.c:1797-1808)
  for (int a = warp; a < p; a += nWarps) {
    double2 const *ca = M + (int64_t)a * LD;
    double s2 = 0;
    for (int r = lane; r < p; r += 32) s2 += ca[r].x * ca[r].x + ca[r].y * ca[r].y;
    s2 = warpSum(s2);
    if (lane == 0) wgt[a] = s2;
  }
  __syncthreads();
  if (tid == 0) {
    double smax = 0;
    for (int a = 0; a < p; ++a) smax = fmax(smax, sqrt(wgt[a]));
    double const cut = cutMode == 0 ? (double)p * kEps * smax + kEps : cutTol * smax;
    for (int a = 0; a < p; ++a) {
      double const sa = sqrt(wgt[a]);
      wgt[a] = (sa < cut || sa == 0.0) ? 0.0 : 1.0 / wgt[a];
    }
  }
  __syncthreads();

  // Z_shift[i, j] = sum_a top[i,a] conj(bottom[j,a]) / s_a^2, column-major
  double2 *out = arena + d.arenaOff;
  int64_t const total = (int64_t)p * n;
  for (int64_t e = tid; e < total; e += nthr) {
    int const i = (int)(e % p), j = (int)(e / p);
    double sr = 0, si = 0;
    for (int a = 0; a < p; ++a) {
      double const w = wgt[a];
      if (w == 0.0) continue;
      double2 const t = M[(int64_t)a * LD + i], b = M[(int64_t)a * LD + p + j];
      sr += w * (t.x * b.x + t.y * b.y);   // t * conj(b)
      si += w * (t.y * b.x - t.x * b.y);
    }
    out[e] = make_double2(sr, si);
  }
}

// ---------------------------------------------------------------------------
// dense rows, kernel matrices, Bessel probes
// ---------------------------------------------------------------------------
__global__ void denseRowsKernel(PointsDev src, int64_t nSrc, PointsDev tgt,
                                int64_t const *rows, KernelParams kp,
                                double2 const *x, int64_t ldx, int64_t R,
                                double2 *out, int64_t ldo) {
  // one CTA per sampled row; threads stride over sources, R <= 8 per pass
  int64_t const s = blockIdx.x;
  int64_t const ti = rows[s];
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;
  bool const useTgtN = kp.layerPot == kLpPvNormalDerivSingle;
  __shared__ double red[2][32];
  for (int64_t r0 = 0; r0 < R; r0 += 8) {
    int const rc = (int)((R - r0) < 8 ? (R - r0) : 8);
    double accr[8] = {0, 0, 0, 0, 0, 0, 0, 0}, acci[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t j = threadIdx.x; j < nSrc; j += blockDim.x) {
      double2 kv = kernelValue(kp, tgt.x[ti], tgt.y[ti], useTgtN ? tgt.nx[ti] : 0.0,
                               useTgtN ? tgt.ny[ti] : 0.0, src.x[j], src.y[j],
                               useSrcN ? src.nx[j] : 0.0, useSrcN ? src.ny[j] : 0.0);
      for (int c = 0; c < rc; ++c) {
        double2 xv = x[j * ldx + r0 + c];
        accr[c] += kv.x * xv.x - kv.y * xv.y;
        acci[c] += kv.x * xv.y + kv.y * xv.x;
      }
    }
    for (int c = 0; c < rc; ++c) {
      double vr = warpSum(accr[c]), vi = warpSum(acci[c]);
      if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = vr;
        red[1][threadIdx.x >> 5] = vi;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double sr = 0, si = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
          sr += red[0][w];
          si += red[1][w];
        }
        out[s * ldo + r0 + c] = make_double2(sr, si);
      }
      __syncthreads();
    }
  }
}

__global__ void kernelMatrixKernel(PointsDev src, int64_t n, PointsDev tgt, int64_t m,
                                   KernelParams kp, double2 *out) {
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;
  bool const useTgtN = kp.layerPot == kLpPvNormalDerivSingle;
  int64_t const total = m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / n, j = e % n;
    out[e] = kernelValue(kp, tgt.x[i], tgt.y[i], useTgtN ? tgt.nx[i] : 0.0,
                         useTgtN ? tgt.ny[i] : 0.0, src.x[j], src.y[j],
                         useSrcN ? src.nx[j] : 0.0, useSrcN ? src.ny[j] : 0.0);
  }
}

__global__ void bessel01Kernel(double const *x, int64_t n, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    Bessel01 b = bessel01<true>(x[i]);
    out[4 * i] = b.j0;
    out[4 * i + 1] = b.y0;
    out[4 * i + 2] = b.j1;
    out[4 * i + 3] = b.y1;
  }
}

__global__ void arenaToF32Kernel(double2 const *a, float2 *b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 v = a[i];
    b[i] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void c128ToC64Kernel(double2 const *a, int64_t lda, int64_t rows, int64_t cols,
                                float2 *b, int64_t ldb) {
  int64_t const total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / cols, j = e % cols;
    double2 v = a[i * lda + j];
    b[i * ldb + j] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void c64ToC128Kernel(float2 const *a, int64_t lda, int64_t rows, int64_t cols,
                                double2 *b, int64_t ldb) {
  int64_t const total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / cols, j = e % cols;
    float2 v = a[i * lda + j];
    b[i * ldb + j] = make_double2((double)v.x, (double)v.y);
  }
}

// ---------------------------------------------------------------------------
// apply
// ---------------------------------------------------------------------------
template <typename T2> struct Real;
template <> struct Real<double2> { using T = double; };
template <> struct Real<float2> { using T = float; };

template <typename T2>
__device__ __forceinline__ T2 mk2(typename Real<T2>::T a, typename Real<T2>::T b) {
  T2 v;
  v.x = a;
  v.y = b;
  return v;
}

// R == 1: one warp per item, lane = output row
template <typename T2>
__global__ void applyGemvKernel(ApplyItem const *__restrict__ items, int64_t nItems,
                                ApplyContrib const *__restrict__ contribs,
                                T2 const *__restrict__ arena, T2 const *__restrict__ X,
                                int64_t ldx, T2 *__restrict__ W) {
  using T = typename Real<T2>::T;
  int64_t const item = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (item >= nItems) return;
  int const lane = threadIdx.x & 31;
  ApplyItem const it = items[item];
  bool const active = lane < it.rows;
  T accr = 0, acci = 0;
  for (int c = 0; c < it.nContrib; ++c) {
    ApplyContrib const cb = contribs[it.contrib0 + c];
    T2 const *a = arena + cb.aOff + lane;
    T2 const *x = cb.inIsX ? X + cb.inRow * ldx : W + cb.inRow;
    int64_t const xs = cb.inIsX ? ldx : 1;
    int const n = cb.n;
    int64_t const lda = cb.lda;
    int j = 0;
    for (; j + 4 <= n; j += 4) {
      T2 a0, a1, a2, a3;
      if (active) {
        a0 = a[(j + 0) * lda];
        a1 = a[(j + 1) * lda];
        a2 = a[(j + 2) * lda];
        a3 = a[(j + 3) * lda];
      } else {
        a0 = a1 = a2 = a3 = mk2<T2>(0, 0);
      }
      T2 const x0 = x[(j + 0) * xs], x1 = x[(j + 1) * xs];
      T2 const x2 = x[(j + 2) * xs], x3 = x[(j + 3) * xs];
      accr += a0.x * x0.x - a0.y * x0.y;
      acci += a0.x * x0.y + a0.y * x0.x;
      accr += a1.x * x1.x - a1.y * x1.y;
      acci += a1.x * x1.y + a1.y * x1.x;
      accr += a2.x * x2.x - a2.y * x2.y;
      acci += a2.x * x2.y + a2.y * x2.x;
      accr += a3.x * x3.x - a3.y * x3.y;
      acci += a3.x * x3.y + a3.y * x3.x;
    }
    for (; j < n; ++j) {
      T2 const a0 = active ? a[j * lda] : mk2<T2>(0, 0);
      T2 const x0 = x[j * xs];
      accr += a0.x * x0.x - a0.y * x0.y;
      acci += a0.x * x0.y + a0.y * x0.x;
    }
  }
  if (active) W[it.outRow + lane] = mk2<T2>(accr, acci);
}

// R > 1: one CTA per (item, RHS tile of RT columns); 32 rows x RT outputs,
// K staged through shared memory in chunks of KC columns.
template <typename T2, int RT>
__global__ void __launch_bounds__(256) applyTileKernel(
    ApplyItem const *__restrict__ items, ApplyContrib const *__restrict__ contribs,
    T2 const *__restrict__ arena, T2 const *__restrict__ X, int64_t ldx,
    T2 *__restrict__ W, int64_t R) {
  using T = typename Real<T2>::T;
  constexpr int KC = 32;
  constexpr int NT = 256;
  constexpr int PER = 32 * RT / NT;      // outputs per thread
  static_assert(PER >= 1, "tile too small");
  __shared__ T2 As[KC][32];
  __shared__ T2 Bs[KC][RT];
  ApplyItem const it = items[blockIdx.x];
  int64_t const r0 = (int64_t)blockIdx.y * RT;
  int const tid = threadIdx.x;
  // thread -> (row, first rhs); rhs columns strided by NT/32
  int const row = tid & 31;
  int const c0 = tid >> 5;               // 0..7
  T accr[PER], acci[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) accr[q] = acci[q] = 0;
  for (int cbi = 0; cbi < it.nContrib; ++cbi) {
    ApplyContrib const cb = contribs[it.contrib0 + cbi];
    T2 const *xin = cb.inIsX ? X + cb.inRow * ldx : W + cb.inRow * R;
    int64_t const xld = cb.inIsX ? ldx : R;
    for (int k0 = 0; k0 < cb.n; k0 += KC) {
      int const kc = (cb.n - k0) < KC ? (cb.n - k0) : KC;
      for (int e = tid; e < KC * 32; e += NT) {
        int const kk = e >> 5, rr = e & 31;
        As[kk][rr] = (kk < kc && rr < it.rows) ? arena[cb.aOff + (int64_t)(k0 + kk) * cb.lda + rr]
                                              : mk2<T2>(0, 0);
      }
      for (int e = tid; e < KC * RT; e += NT) {
        int const kk = e / RT, cc = e % RT;
        Bs[kk][cc] = (kk < kc && r0 + cc < R) ? xin[(int64_t)(k0 + kk) * xld + r0 + cc]
                                             : mk2<T2>(0, 0);
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < kc; ++kk) {
        T2 const a = As[kk][row];
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          T2 const b = Bs[kk][c0 + q * (NT / 32)];
          accr[q] += a.x * b.x - a.y * b.y;
          acci[q] += a.x * b.y + a.y * b.x;
        }
      }
      __syncthreads();
    }
  }
  if (row < it.rows) {
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      int64_t const col = r0 + c0 + q * (NT / 32);
      if (col < R) W[(it.outRow + row) * R + col] = mk2<T2>(accr[q], acci[q]);
    }
  }
}

template <typename T2>
__global__ void applyReduceKernel(int32_t const *__restrict__ rowSeg,
                                  int64_t const *__restrict__ segStart,
                                  int64_t const *__restrict__ segContrib0,
                                  int64_t const *__restrict__ segBase,
                                  T2 const *__restrict__ W, int64_t R,
                                  T2 *__restrict__ Y, int64_t ldy, int64_t nRows,
                                  int64_t const *__restrict__ outPerm) {
  using T = typename Real<T2>::T;
  int64_t const total = nRows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / R, r = e % R;
    int const s = rowSeg[i];
    int64_t const di = i - segStart[s];
    T sr = 0, si = 0;
    for (int64_t c = segContrib0[s]; c < segContrib0[s + 1]; ++c) {
      T2 const v = W[(segBase[c] + di) * R + r];
      sr += v.x;
      si += v.y;
    }
    int64_t const oi = outPerm ? outPerm[i] : i;
    Y[oi * ldy + r] = mk2<T2>(sr, si);
  }
}

template <typename T2>
__global__ void gatherRowsKernel(T2 const *X, int64_t ldx, int64_t const *perm,
                                 int64_t nRows, int64_t R, T2 *out) {
  int64_t const total = nRows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / R, r = e % R;
    out[e] = X[perm[i] * ldx + r];
  }
}

int gridFor(int64_t total, int threads) {
  int64_t g = (total + threads - 1) / threads;
  if (g > 152 * 64) g = 152 * 64;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

int64_t reexpansionSmemBytes(int32_t m, int32_t n) {
  return (int64_t)16 * (m + n) * m + (int64_t)8 * (7 * (int64_t)m + 4 * (int64_t)n);
}

int64_t reexpansionScratchEntries(int32_t m, int32_t n) {
  int64_t e = (int64_t)(m + n) * m;
  return (e + 15) & ~int64_t(15);
}

cudaError_t launchFillBlocks(FillDesc const *descs, int32_t nDesc, PointsDev src,
                             PointsDev tgt, KernelParams kp, double2 *arena,
                             int32_t maxProxyN, int32_t *status, cudaStream_t stream) {
  if (nDesc == 0) return cudaSuccess;
  size_t const smem = 4 * (size_t)(maxProxyN > 0 ? maxProxyN : 1) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(fillBlocksKernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  fillBlocksKernel<<<nDesc, 256, smem, stream>>>(descs, src, tgt, kp, arena, status);
  return cudaGetLastError();
}

cudaError_t launchReexpansion(FillDesc const *descs, int32_t nDesc, PointsDev src,
                              KernelParams kp, int32_t cutMode, double cutTol,
                              double2 *arena, double2 *scratch,
                              int64_t const *scratchOff, int32_t *status, bool smem,
                              int32_t maxSmemBytes, int32_t threads, cudaStream_t stream) {
  if (nDesc == 0) return cudaSuccess;
  cudaError_t e;
  if (smem) {
    e = cudaFuncSetAttribute(reexpansionKernel<true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmemBytes);
    if (e != cudaSuccess) return e;
    reexpansionKernel<true><<<nDesc, threads, maxSmemBytes, stream>>>(
        descs, src, kp, cutMode, cutTol, arena, scratch, scratchOff, status);
  } else {
    e = cudaFuncSetAttribute(reexpansionKernel<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmemBytes);
    if (e != cudaSuccess) return e;
    reexpansionKernel<false><<<nDesc, threads, maxSmemBytes, stream>>>(
        descs, src, kp, cutMode, cutTol, arena, scratch, scratchOff, status);
  }
  return cudaGetLastError();
}

cudaError_t launchDenseRows(PointsDev src, int64_t nSrc, PointsDev tgt,
                            int64_t const *rows, int64_t nRows, KernelParams kp,
                            double2 const *x, int64_t ldx, int64_t R, double2 *out,
                            int64_t ldo, cudaStream_t stream) {
  if (nRows == 0) return cudaSuccess;
  denseRowsKernel<<<(unsigned)nRows, 256, 0, stream>>>(src, nSrc, tgt, rows, kp, x, ldx, R,
                                                       out, ldo);
  return cudaGetLastError();
}

cudaError_t launchKernelMatrix(PointsDev src, int64_t n, PointsDev tgt, int64_t m,
                               KernelParams kp, double2 *out, cudaStream_t stream) {
  if (m * n == 0) return cudaSuccess;
  kernelMatrixKernel<<<gridFor(m * n, 256), 256, 0, stream>>>(src, n, tgt, m, kp, out);
  return cudaGetLastError();
}

cudaError_t launchBessel01(double const *x, int64_t n, double *out, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  bessel01Kernel<<<gridFor(n, 256), 256, 0, stream>>>(x, n, out);
  return cudaGetLastError();
}

cudaError_t launchArenaToF32(double2 const *a64, float2 *a32, int64_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  arenaToF32Kernel<<<gridFor(n, 256), 256, 0, stream>>>(a64, a32, n);
  return cudaGetLastError();
}

cudaError_t launchC128ToC64(double2 const *a, int64_t lda, int64_t rows, int64_t cols,
                            float2 *b, int64_t ldb, cudaStream_t stream) {
  if (rows * cols == 0) return cudaSuccess;
  c128ToC64Kernel<<<gridFor(rows * cols, 256), 256, 0, stream>>>(a, lda, rows, cols, b, ldb);
  return cudaGetLastError();
}

cudaError_t launchC64ToC128(float2 const *a, int64_t lda, int64_t rows, int64_t cols,
                            double2 *b, int64_t ldb, cudaStream_t stream) {
  if (rows * cols == 0) return cudaSuccess;
  c64ToC128Kernel<<<gridFor(rows * cols, 256), 256, 0, stream>>>(a, lda, rows, cols, b, ldb);
  return cudaGetLastError();
}

template <typename T2>
cudaError_t launchApplyStage(ApplyItem const *items, int64_t nItems,
                             ApplyContrib const *contribs, T2 const *arena,
                             T2 const *X, int64_t ldx, T2 *W, int64_t R,
                             cudaStream_t stream) {
  if (nItems == 0) return cudaSuccess;
  if (R == 1) {
    int const warps = 8;
    unsigned const grid = (unsigned)((nItems + warps - 1) / warps);
    applyGemvKernel<T2><<<grid, 32 * warps, 0, stream>>>(items, nItems, contribs, arena, X,
                                                         ldx, W);
  } else if (R <= 8) {
    dim3 grid((unsigned)nItems, 1);
    applyTileKernel<T2, 8><<<grid, 256, 0, stream>>>(items, contribs, arena, X, ldx, W, R);
  } else if (R <= 16) {
    dim3 grid((unsigned)nItems, 1);
    applyTileKernel<T2, 16><<<grid, 256, 0, stream>>>(items, contribs, arena, X, ldx, W, R);
  } else {
    dim3 grid((unsigned)nItems, (unsigned)((R + 31) / 32));
    applyTileKernel<T2, 32><<<grid, 256, 0, stream>>>(items, contribs, arena, X, ldx, W, R);
  }
  return cudaGetLastError();
}

template <typename T2>
cudaError_t launchApplyReduce(int32_t const *rowSeg, int64_t const *segStart,
                              int64_t const *segContrib0, int64_t const *segBase,
                              T2 const *W, int64_t R, T2 *Y, int64_t ldy,
                              int64_t nRows, int64_t const *outPerm,
                              cudaStream_t stream) {
  applyReduceKernel<T2><<<gridFor(nRows * R, 256), 256, 0, stream>>>(
      rowSeg, segStart, segContrib0, segBase, W, R, Y, ldy, nRows, outPerm);
  return cudaGetLastError();
}

template <typename T2>
cudaError_t launchGatherRows(T2 const *X, int64_t ldx, int64_t const *perm,
                             int64_t nRows, int64_t R, T2 *out, cudaStream_t stream) {
  gatherRowsKernel<T2><<<gridFor(nRows * R, 256), 256, 0, stream>>>(X, ldx, perm, nRows, R,
                                                                    out);
  return cudaGetLastError();
}

template cudaError_t launchApplyStage<double2>(ApplyItem const *, int64_t, ApplyContrib const *,
                                               double2 const *, double2 const *, int64_t,
                                               double2 *, int64_t, cudaStream_t);
template cudaError_t launchApplyStage<float2>(ApplyItem const *, int64_t, ApplyContrib const *,
                                              float2 const *, float2 const *, int64_t, float2 *,
                                              int64_t, cudaStream_t);
template cudaError_t launchApplyReduce<double2>(int32_t const *, int64_t const *, int64_t const *,
                                                int64_t const *, double2 const *, int64_t,
                                                double2 *, int64_t, int64_t, int64_t const *,
                                                cudaStream_t);
template cudaError_t launchApplyReduce<float2>(int32_t const *, int64_t const *, int64_t const *,
                                               int64_t const *, float2 const *, int64_t, float2 *,
                                               int64_t, int64_t, int64_t const *, cudaStream_t);
template cudaError_t launchGatherRows<double2>(double2 const *, int64_t, int64_t const *, int64_t,
                                               int64_t, double2 *, cudaStream_t);
template cudaError_t launchGatherRows<float2>(float2 const *, int64_t, int64_t const *, int64_t,
                                              int64_t, float2 *, cudaStream_t);

}  // namespace bfg
