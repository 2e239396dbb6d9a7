// Two-level preconditioner of a boundary-integral system (a GB300 addition;
// the reference preconditions with block-Jacobi only,
// multiple_scattering_context.c:545-634).
//
// Block-Jacobi inverts every scatterer's self-interaction; what it leaves is
// the coupling between scatterers, which the low Fourier modes of every curve
// carry.  The coarse space Phi holds, for curve b with points j = 0 .. n_b-1
// equispaced in its parameter, the modes e^{i mu 2 pi j / n_b} / sqrt(n_b),
// mu = -q_b .. q_b, q_b = min(ceil(k L_b / 2 pi) + extra, (n_b - 1) / 2) with
// L_b the curve's length (the sum of its quadrature weights): the modes that
// radiate.  Built once:
//   Y   = A Phi             one apply of the system to all D coarse basis
//                           vectors: the butterfly part as one D-RHS
//                           split-BF16 tensor-core apply, the diagonal shift
//                           and the Kapur-Rokhlin correction beside it;
//   A_c = Phi^H Y           a batched complex GEMM over the curves;
//   A_c^-1                  block Gauss-Jordan elimination with the curves'
//                           mode blocks as pivots in order (partial pivoting
//                           inside a block's own inverse), FP32.
// Applied in every FGMRES iteration (multiplicative, right preconditioner):
//   z1 = Phi A_c^-1 Phi^H r,   z = z1 + M_bj (r - A z1).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/bfg.h"
#include "bfg_kernels.cuh"
#include "bfg_system.hpp"

namespace {

using bfg::Dev;

constexpr int kMaxModes = 128;   // modes per curve (the block inverse's shared memory)

bfgStatus coarseFail(bfgSystem s, bfgStatus st, std::string const &msg) {
  s->err = msg;
  return st;
}

#define CO_CK(expr)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (expr);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return coarseFail(sys, BFG_ERROR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// ---- the basis: curve b's table n_b x M_b (row j, mode column m), row-major
__global__ void coarseTableKernel(int64_t const *offsets, int64_t const *cStart,
                                  int64_t const *tabOff, float2 *tab) {
  int const b = blockIdx.x;
  int64_t const n = offsets[b + 1] - offsets[b];
  int const M = (int)(cStart[b + 1] - cStart[b]);
  int const q = (M - 1) / 2;
  double const sc = 1.0 / sqrt((double)n);
  for (int64_t e = threadIdx.x; e < n * M; e += blockDim.x) {
    int64_t const j = e / M;
    int64_t const mu = (e % M) - q;
    // the angle 2 pi (mu j mod n) / n, reduced exactly in integers
    int64_t idx = (mu * j) % n;
    if (idx < 0) idx += n;
    double s, c;
    sincospi(2.0 * (double)idx / (double)n, &s, &c);
    tab[tabOff[b] + e] = make_float2((float)(c * sc), (float)(s * sc));
  }
}

// Xw = diag(w) Phi (n x D, row-major): row i of curve b holds w_i Phi_b[j, .]
// in the curve's coarse columns, zeros elsewhere
__global__ void coarseFillKernel(int64_t n, int64_t D, int64_t const *curveOf,
                                 int64_t const *offsets, int64_t const *cStart,
                                 int64_t const *tabOff, float2 const *tab, double const *w,
                                 float2 *Xw) {
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    int64_t const b = curveOf[i], j = i - offsets[b], c0 = cStart[b];
    int64_t const M = cStart[b + 1] - c0;
    float const wi = (float)w[i];
    float2 const *t = tab + tabOff[b] + j * M;
    float2 *row = Xw + i * D;
    for (int64_t c = threadIdx.x; c < D; c += blockDim.x) {
      int64_t const m = c - c0;
      float2 v = make_float2(0.f, 0.f);
      if (m >= 0 && m < M) v = make_float2(wi * t[m].x, wi * t[m].y);
      row[c] = v;
    }
  }
}

// Y = shift Phi + K Xw + C Xw, with K Xw in KY on entry and Y on exit; the
// Kapur-Rokhlin entries of row i reach columns of i's own curve only
__global__ void coarsePostKernel(int64_t n, int64_t D, double shift, int64_t const *curveOf,
                                 int64_t const *offsets, int64_t const *cStart,
                                 int64_t const *tabOff, float2 const *tab, float2 const *Xw,
                                 double2 const *krVal, int64_t const *krCol, int nc,
                                 float2 *KY) {
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    int64_t const b = curveOf[i], j = i - offsets[b], c0 = cStart[b];
    int64_t const M = cStart[b + 1] - c0;
    float2 const *t = tab + tabOff[b] + j * M;
    for (int64_t m = threadIdx.x; m < M; m += blockDim.x) {
      int64_t const c = c0 + m;
      float2 y = KY[i * D + c];
      y.x += (float)shift * t[m].x;
      y.y += (float)shift * t[m].y;
      for (int q = 0; q < nc; ++q) {
        double2 const v = krVal[i * nc + q];
        float2 const x = Xw[krCol[i * nc + q] * D + c];
        y = make_float2(y.x + (float)v.x * x.x - (float)v.y * x.y,
                        y.y + (float)v.x * x.y + (float)v.y * x.x);
      }
      KY[i * D + c] = y;
    }
  }
}

// ---- batched complex GEMM, row-major: C = alpha op(A) B + beta C with
// op(A)[i, k] = A[i * lda + k] (opA 0) or conj(A[k * lda + i]) (opA 1);
// 64 x 64 tiles of C per CTA, 16 columns of K at a time through shared
// memory, 4 x 4 outputs per thread, FP32 (the coarse space is a
// preconditioner: FP32 is enough).  Batch z of the grid = descriptor z;
// tiles past a descriptor's M or N return.
struct CGemm {
  float2 const *A;
  float2 const *B;
  float2 *C;
  int64_t lda, ldb, ldc;
  int32_t M, N, K, opA;
  float alpha, beta;
};
constexpr int kCT = 64, kCK = 16;

__global__ void __launch_bounds__(256) cgemmKernel(CGemm const *__restrict__ descs) {
  CGemm const g = descs[blockIdx.z];
  int const i0 = blockIdx.y * kCT, j0 = blockIdx.x * kCT;
  if (i0 >= g.M || j0 >= g.N) return;
  __shared__ float2 As[kCK][kCT + 1];
  __shared__ float2 Bs[kCK][kCT + 1];
  int const tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float2 acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < g.K; k0 += kCK) {
    if (g.opA == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int const kk = tid & 15, i = (tid >> 4) + 16 * q;
        int const gi = i0 + i, gk = k0 + kk;
        As[kk][i] = (gi < g.M && gk < g.K) ? g.A[gi * g.lda + gk] : make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int const i = tid & 63, kk = (tid >> 6) + 4 * q;
        int const gi = i0 + i, gk = k0 + kk;
        float2 v = make_float2(0.f, 0.f);
        if (gi < g.M && gk < g.K) {
          v = g.A[gk * g.lda + gi];
          v.y = -v.y;
        }
        As[kk][i] = v;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const j = tid & 63, kk = (tid >> 6) + 4 * q;
      int const gj = j0 + j, gk = k0 + kk;
      Bs[kk][j] = (gj < g.N && gk < g.K) ? g.B[gk * g.ldb + gj] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kCK; ++kk) {
      float2 a[4], bv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) bv[c] = Bs[kk][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          acc[r][c].x = fmaf(a[r].x, bv[c].x, fmaf(-a[r].y, bv[c].y, acc[r][c].x));
          acc[r][c].y = fmaf(a[r].x, bv[c].y, fmaf(a[r].y, bv[c].x, acc[r][c].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int const gi = i0 + ty + 16 * r;
    if (gi >= g.M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int const gj = j0 + tx + 16 * c;
      if (gj >= g.N) continue;
      float2 *p = g.C + gi * g.ldc + gj;
      float2 v = make_float2(g.alpha * acc[r][c].x, g.alpha * acc[r][c].y);
      if (g.beta != 0.f) v = make_float2(v.x + g.beta * p->x, v.y + g.beta * p->y);
      *p = v;
    }
  }
}

// ---- the inverse of one m x m block (m <= kMaxModes) in shared memory:
// in-place Gauss-Jordan with partial pivoting, the row exchanges undone on
// the columns at the end.  A zero pivot sets *flag.
__global__ void __launch_bounds__(1024) blockInverseKernel(float2 const *A, int64_t lda, int m,
                                                           float2 *P, int32_t *flag) {
  extern __shared__ float2 sa[];   // m x m
  __shared__ int perm[kMaxModes];
  __shared__ float pv[32];
  __shared__ int pi[32];
  __shared__ int piv;
  int const tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < m * m; e += nt) sa[e] = A[(e / m) * lda + e % m];
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    // pivot: the largest |a_ik|, i >= k (first of equals)
    float best = -1.f;
    int bi = k;
    for (int i = k + tid; i < m; i += nt) {
      float2 const v = sa[i * m + k];
      float const a = v.x * v.x + v.y * v.y;
      if (a > best) {
        best = a;
        bi = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      float const ob = __shfl_down_sync(0xffffffffu, best, o);
      int const oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if ((tid & 31) == 0) {
      pv[tid >> 5] = best;
      pi[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      float b0 = pv[0];
      int i0 = pi[0];
      for (int w = 1; w < (nt + 31) / 32; ++w)
        if (pv[w] > b0 || (pv[w] == b0 && pi[w] < i0)) {
          b0 = pv[w];
          i0 = pi[w];
        }
      piv = i0;
      perm[k] = i0;
      if (!(b0 > 0.f)) atomicOr(flag, 1);
    }
    __syncthreads();
    int const p = piv;
    if (p != k)
      for (int j = tid; j < m; j += nt) {
        float2 const t = sa[k * m + j];
        sa[k * m + j] = sa[p * m + j];
        sa[p * m + j] = t;
      }
    __syncthreads();
    float2 const d = sa[k * m + k];
    float const dd = d.x * d.x + d.y * d.y;
    float2 const inv = dd > 0.f ? make_float2(d.x / dd, -d.y / dd) : make_float2(0.f, 0.f);
    __syncthreads();
    // row k: a_kk <- 1, then the row divided by the pivot
    for (int j = tid; j < m; j += nt) sa[k * m + j] = j == k ? inv : cmulf(sa[k * m + j], inv);
    __syncthreads();
    // the other rows: a_ij -= a_ik a_kj, with a_ik <- 0 first (so column k
    // ends as -a_ik / pivot)
    for (int e = tid; e < m * m; e += nt) {
      int const i = e / m, j = e % m;
      if (i == k) continue;
      float2 const f = sa[i * m + k];
      float2 const akj = sa[k * m + j];
      float2 const old = j == k ? make_float2(0.f, 0.f) : sa[i * m + j];
      float2 const pr = cmulf(f, akj);
      // every thread reads a_ik before any writes it: column k is written
      // in a second pass below
      if (j != k) sa[i * m + j] = make_float2(old.x - pr.x, old.y - pr.y);
    }
    __syncthreads();
    for (int i = tid; i < m; i += nt)
      if (i != k) {
        float2 const f = sa[i * m + k];
        float2 const pr = cmulf(f, inv);
        sa[i * m + k] = make_float2(-pr.x, -pr.y);
      }
    __syncthreads();
  }
  // undo the row exchanges on the columns, last first
  for (int k = m - 1; k >= 0; --k) {
    int const p = perm[k];
    if (p != k)
      for (int i = tid; i < m; i += nt) {
        float2 const t = sa[i * m + k];
        sa[i * m + k] = sa[i * m + p];
        sa[i * m + p] = t;
      }
    __syncthreads();
  }
  for (int e = tid; e < m * m; e += nt) P[e] = sa[e];
}

// U = A[:, c0 .. c0+m) (D x m, row-major), rows c0 .. c0+m zeroed
__global__ void takeColumnsKernel(float2 const *A, int64_t D, int64_t c0, int m, float2 *U) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < D * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / m;
    int const j = (int)(e % m);
    U[e] = (i >= c0 && i < c0 + m) ? make_float2(0.f, 0.f) : A[i * D + c0 + j];
  }
}

// rows c0 .. c0+m of A: T, with the block columns c0 .. c0+m from P
__global__ void putRowsKernel(float2 *A, int64_t D, int64_t c0, int m, float2 const *T,
                              float2 const *P) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)m * D;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const r = e / D, c = e % D;
    A[(c0 + r) * D + c] = (c >= c0 && c < c0 + m) ? P[r * m + (c - c0)] : T[e];
  }
}

// ---- per-iteration kernels
// cin[c0 + m] = sum_j conj(Phi_b[j, m]) r[off_b + j]  (one CTA per curve)
__global__ void coarseRestrictKernel(int64_t const *offsets, int64_t const *cStart,
                                     int64_t const *tabOff, float2 const *tab, double2 const *r,
                                     float2 *cin) {
  int const b = blockIdx.x;
  int64_t const o = offsets[b], n = offsets[b + 1] - o, c0 = cStart[b];
  int const M = (int)(cStart[b + 1] - c0);
  float2 const *t = tab + tabOff[b];
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      float2 const p = t[j * M + m];
      double2 const v = r[o + j];
      sr += (double)p.x * v.x + (double)p.y * v.y;
      si += (double)p.x * v.y - (double)p.y * v.x;
    }
    cin[c0 + m] = make_float2((float)sr, (float)si);
  }
}

// cout = Ainv cin (D x D row-major): one warp per row
__global__ void coarseGemvKernel(int64_t D, float2 const *Ainv, float2 const *cin, float2 *cout) {
  int64_t const row = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  int const lane = threadIdx.x & 31;
  if (row >= D) return;
  float2 const *a = Ainv + row * D;
  float sr = 0.f, si = 0.f;
  for (int64_t c = lane; c < D; c += 32) {
    float2 const v = a[c], x = cin[c];
    sr = fmaf(v.x, x.x, fmaf(-v.y, x.y, sr));
    si = fmaf(v.x, x.y, fmaf(v.y, x.x, si));
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (lane == 0) cout[row] = make_float2(sr, si);
}

// z[off_b + j] = sum_m Phi_b[j, m] cout[c0 + m]  (one CTA per curve)
__global__ void coarseProlongKernel(int64_t const *offsets, int64_t const *cStart,
                                    int64_t const *tabOff, float2 const *tab, float2 const *cout,
                                    double2 *z) {
  int const b = blockIdx.x;
  int64_t const o = offsets[b], n = offsets[b + 1] - o, c0 = cStart[b];
  int const M = (int)(cStart[b + 1] - c0);
  float2 const *t = tab + tabOff[b];
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int m = 0; m < M; ++m) {
      float2 const p = t[j * M + m], y = cout[c0 + m];
      sr += (double)p.x * y.x - (double)p.y * y.y;
      si += (double)p.x * y.y + (double)p.y * y.x;
    }
    z[o + j] = make_double2(sr, si);
  }
}

__global__ void addToKernel(int64_t n, double2 const *x, double2 *y) {   // y += x
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = make_double2(y[i].x + x[i].x, y[i].y + x[i].y);
}

unsigned gridOf(int64_t n, int t) {
  int64_t const g = (n + t - 1) / t;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

cudaError_t runGemm(CGemm const *host, int nb, int maxM, int maxN, Dev &dDesc, cudaStream_t s) {
  cudaError_t e = dDesc.alloc(sizeof(CGemm) * nb);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(dDesc.p, host, sizeof(CGemm) * nb, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((maxN + kCT - 1) / kCT), (unsigned)((maxM + kCT - 1) / kCT), (unsigned)nb);
  cgemmKernel<<<grid, 256, 0, s>>>(dDesc.as<CGemm>());
  return cudaGetLastError();
}

// z = Phi A_c^-1 Phi^H r
void coarseCorrection(bfgSystem sys, double2 const *r, double2 *z, cudaStream_t s) {
  int const nb = (int)sys->numCurves;
  int64_t const D = sys->coarseDim;
  coarseRestrictKernel<<<nb, 128, 0, s>>>(sys->dOffsets.as<int64_t>(), sys->dCStart.as<int64_t>(),
                                          sys->dTabOff.as<int64_t>(), sys->dTab.as<float2>(), r,
                                          sys->dCoarseIn.as<float2>());
  coarseGemvKernel<<<(unsigned)((D + 7) / 8), 256, 0, s>>>(D, sys->dAcInv.as<float2>(),
                                                          sys->dCoarseIn.as<float2>(),
                                                          sys->dCoarseOut.as<float2>());
  coarseProlongKernel<<<nb, 256, 0, s>>>(sys->dOffsets.as<int64_t>(), sys->dCStart.as<int64_t>(),
                                         sys->dTabOff.as<int64_t>(), sys->dTab.as<float2>(),
                                         sys->dCoarseOut.as<float2>(), z);
}

}  // namespace

namespace bfg {
bfgStatus applyTwoLevel(bfgSystem sys, double2 const *r, double2 *z) {
  cudaStream_t s = sys->stream();
  int64_t const n = sys->n;
  double2 *z1 = sys->dZ1.as<double2>(), *t = sys->dT1.as<double2>();
  coarseCorrection(sys, r, z1, s);
  CO_CK(cudaGetLastError());
  // t = r - A z1, z = M_bj t + z1
  bfgStatus st = systemApplyPrec(sys, sys->applyPrec, z1, t);
  if (st != BFG_OK) return st;
  launchSubFrom(n, r, t, s);
  applyBlockJacobi32(sys, t, z, s);
  addToKernel<<<gridOf(n, 256), 256, 0, s>>>(n, z1, z);
  CO_CK(cudaGetLastError());
  return BFG_OK;
}
}  // namespace bfg

extern "C" {

bfgStatus bfgSystemBuildCoarse(bfgSystem sys, int32_t extraModes, int64_t *dimOut) {
  if (!sys || extraModes < 0) return BFG_ERROR_INVALID_ARGUMENTS;
  sys->haveCoarse = false;   // a rebuild that fails leaves no half-built space in use
  cudaStream_t s = sys->stream();
  int64_t const n = sys->n, nb = sys->numCurves;
  double const pi2 = 6.283185307179586;
  // modes per curve from its length (the sum of its weights)
  sys->cStart.assign(1, 0);
  sys->tabOff.assign(1, 0);
  int maxM = 0;
  for (int64_t b = 0; b < nb; ++b) {
    int64_t const nbp = sys->offsets[b + 1] - sys->offsets[b];
    double L = 0.0;
    for (int64_t i = sys->offsets[b]; i < sys->offsets[b + 1]; ++i) L += sys->weights[(size_t)i];
    int64_t q = (int64_t)std::ceil(sys->kp.k * L / pi2) + extraModes;
    q = std::max<int64_t>(0, std::min<int64_t>(q, (nbp - 1) / 2));
    if (2 * q + 1 > kMaxModes)
      return coarseFail(sys, BFG_ERROR_OUT_OF_RANGE,
                        "coarse space: a curve needs more than 128 modes");
    int const M = (int)(2 * q + 1);
    maxM = std::max(maxM, M);
    sys->cStart.push_back(sys->cStart.back() + M);
    sys->tabOff.push_back(sys->tabOff.back() + nbp * M);
  }
  int64_t const D = sys->cStart.back();
  sys->coarseDim = D;
  if (D > 0x7fffffff / kCT) return coarseFail(sys, BFG_ERROR_OUT_OF_RANGE, "coarse space too large");
  CO_CK(sys->dCStart.alloc((nb + 1) * 8));
  CO_CK(sys->dTabOff.alloc((nb + 1) * 8));
  CO_CK(sys->dTab.alloc((size_t)sys->tabOff.back() * 8));
  CO_CK(cudaMemcpyAsync(sys->dCStart.p, sys->cStart.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s));
  CO_CK(cudaMemcpyAsync(sys->dTabOff.p, sys->tabOff.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s));
  coarseTableKernel<<<(unsigned)nb, 256, 0, s>>>(sys->dOffsets.as<int64_t>(),
                                                 sys->dCStart.as<int64_t>(),
                                                 sys->dTabOff.as<int64_t>(), sys->dTab.as<float2>());
  CO_CK(cudaGetLastError());

  // Y = A Phi: Xw = diag(w) Phi, K Xw in one D-RHS tensor-core apply
  Dev xw, ky;
  CO_CK(xw.alloc((size_t)n * D * 8));
  CO_CK(ky.alloc((size_t)n * D * 8));
  coarseFillKernel<<<gridOf(n, 1), 256, 0, s>>>(n, D, sys->dCurveOf.as<int64_t>(),
                                                sys->dOffsets.as<int64_t>(),
                                                sys->dCStart.as<int64_t>(),
                                                sys->dTabOff.as<int64_t>(), sys->dTab.as<float2>(),
                                                sys->dW.as<double>(), xw.as<float2>());
  CO_CK(cudaGetLastError());
  bfgStatus st = bfgFacApply(sys->fac, BFG_PRECISION_BF16X3, xw.p, D, D, ky.p, D,
                             BFG_APPLY_ORIGINAL_ORDER);
  if (st != BFG_OK) return coarseFail(sys, st, "coarse space: the butterfly apply failed");
  coarsePostKernel<<<gridOf(n, 1), 128, 0, s>>>(
      n, D, sys->shift, sys->dCurveOf.as<int64_t>(), sys->dOffsets.as<int64_t>(),
      sys->dCStart.as<int64_t>(), sys->dTabOff.as<int64_t>(), sys->dTab.as<float2>(),
      xw.as<float2>(), sys->dKrVal.as<double2>(), sys->dKrCol.as<int64_t>(), 2 * sys->order,
      ky.as<float2>());
  CO_CK(cudaGetLastError());

  // A_c = Phi^H Y, curve by curve
  CO_CK(sys->dAc.alloc((size_t)D * D * 8));
  std::vector<CGemm> g((size_t)nb);
  for (int64_t b = 0; b < nb; ++b) {
    int const M = (int)(sys->cStart[b + 1] - sys->cStart[b]);
    int64_t const nbp = sys->offsets[b + 1] - sys->offsets[b];
    g[b] = CGemm{sys->dTab.as<float2>() + sys->tabOff[b], ky.as<float2>() + sys->offsets[b] * D,
                 sys->dAc.as<float2>() + sys->cStart[b] * D, M, D, D, M, (int32_t)D,
                 (int32_t)nbp, 1, 1.f, 0.f};
  }
  Dev dDesc;
  CO_CK(runGemm(g.data(), (int)nb, maxM, (int)D, dDesc, s));
  CO_CK(cudaStreamSynchronize(s));
  xw.release();
  ky.release();

  // A_c^-1 by block Gauss-Jordan over the curves' mode blocks
  CO_CK(sys->dAcInv.alloc((size_t)D * D * 8));
  CO_CK(cudaMemcpyAsync(sys->dAcInv.p, sys->dAc.p, (size_t)D * D * 8, cudaMemcpyDeviceToDevice, s));
  Dev dP, dTr, dU, dFlag, dG;
  CO_CK(dP.alloc((size_t)maxM * maxM * 8));
  CO_CK(dTr.alloc((size_t)maxM * D * 8));
  CO_CK(dU.alloc((size_t)D * maxM * 8));
  CO_CK(dFlag.alloc(4));
  CO_CK(dG.alloc(sizeof(CGemm) * 3));
  CO_CK(cudaMemsetAsync(dFlag.p, 0, 4, s));
  size_t const invSmem = (size_t)maxM * maxM * 8;
  CO_CK(cudaFuncSetAttribute(blockInverseKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)std::max<size_t>(invSmem, 1)));
  float2 *Ai = sys->dAcInv.as<float2>();
  for (int64_t b = 0; b < nb; ++b) {
    int64_t const c0 = sys->cStart[b];
    int const m = (int)(sys->cStart[b + 1] - c0);
    blockInverseKernel<<<1, 1024, (size_t)m * m * 8, s>>>(Ai + c0 * D + c0, D, m, dP.as<float2>(),
                                                           dFlag.as<int32_t>());
    CO_CK(cudaGetLastError());
    // T = P A[K, :]
    CGemm t{dP.as<float2>(), Ai + c0 * D, dTr.as<float2>(), m, D, D, m, (int32_t)D, m, 0, 1.f, 0.f};
    CO_CK(runGemm(&t, 1, m, (int)D, dG, s));
    takeColumnsKernel<<<gridOf(D * m, 256), 256, 0, s>>>(Ai, D, c0, m, dU.as<float2>());
    CO_CK(cudaGetLastError());
    // A -= U T, then A[:, K] = -U P, then rows K = T with block P
    CGemm u{dU.as<float2>(), dTr.as<float2>(), Ai, m, D, D, (int32_t)D, (int32_t)D, m, 0, -1.f, 1.f};
    CO_CK(runGemm(&u, 1, (int)D, (int)D, dG, s));
    CGemm v{dU.as<float2>(), dP.as<float2>(), Ai + c0, m, m, D, (int32_t)D, m, m, 0, -1.f, 0.f};
    CO_CK(runGemm(&v, 1, (int)D, m, dG, s));
    putRowsKernel<<<gridOf((int64_t)m * D, 256), 256, 0, s>>>(Ai, D, c0, m, dTr.as<float2>(),
                                                             dP.as<float2>());
    CO_CK(cudaGetLastError());
  }
  int32_t flag = 0;
  CO_CK(cudaMemcpyAsync(&flag, dFlag.p, 4, cudaMemcpyDeviceToHost, s));
  CO_CK(cudaStreamSynchronize(s));
  if (flag) return coarseFail(sys, BFG_ERROR_NUMERICAL, "coarse space: a singular pivot block");
  CO_CK(sys->dCoarseIn.alloc((size_t)D * 8));
  CO_CK(sys->dCoarseOut.alloc((size_t)D * 8));
  CO_CK(sys->dZ1.alloc((size_t)n * 16));
  CO_CK(sys->dT1.alloc((size_t)n * 16));
  sys->haveCoarse = true;
  if (dimOut) *dimOut = D;
  return BFG_OK;
}

bfgStatus bfgSystemCoarseMatrices(bfgSystem sys, void *Ac, void *AcInv) {
  if (!sys) return BFG_ERROR_INVALID_ARGUMENTS;
  if (!sys->haveCoarse) return coarseFail(sys, BFG_ERROR_INVALID_ARGUMENTS, "coarse space not built");
  cudaStream_t s = sys->stream();
  size_t const bytes = (size_t)sys->coarseDim * sys->coarseDim * 8;
  if (Ac) CO_CK(cudaMemcpyAsync(Ac, sys->dAc.p, bytes, cudaMemcpyDeviceToDevice, s));
  if (AcInv) CO_CK(cudaMemcpyAsync(AcInv, sys->dAcInv.p, bytes, cudaMemcpyDeviceToDevice, s));
  CO_CK(cudaStreamSynchronize(s));
  return BFG_OK;
}

bfgStatus bfgSystemApplyCoarse(bfgSystem sys, void const *R, void *Z) {
  if (!sys || !R || !Z) return BFG_ERROR_INVALID_ARGUMENTS;
  if (!sys->haveCoarse) return coarseFail(sys, BFG_ERROR_INVALID_ARGUMENTS, "coarse space not built");
  cudaStream_t s = sys->stream();
  coarseCorrection(sys, static_cast<double2 const *>(R), static_cast<double2 *>(Z), s);
  CO_CK(cudaGetLastError());
  return BFG_OK;
}

}  // extern "C"
