// Randomized re-expansion of FIRST/MIDDLE blocks (sm_103a, FP64).
//
// The reference computes every re-expansion block as
//   Z_shift = pinv(Z_equiv) Z_orig          (helm2.c:321-365,
//                                            mat_dense_complex.c:1768-1849)
// with Z_equiv p x p and p the a-priori rank estimate of helm2.c:14-36,
// p = k r1 r2 / (R - r1 - r2) - log10(eps).  That estimate divides by the
// gap between the two proxy circles, so for nearly touching circles p is many
// times the numerical rank of Z_equiv, which follows k r1 r2 / R: at 262,144
// points and k = 2048 a block with p = 9,982 has 482 singular values above
// 1e-13 sigma0, and one with p = 3,710 has 173 above 1e-12 sigma0.  The
// reference's SVD spends O(p^3) on directions that the pseudo-inverse cut
// then drops.  This path spends its work on the numerical rank instead
// (a randomized range finder; Halko, Martinsson and Tropp, SIAM Review 53,
// 2011, algorithms 4.1 and 5.1), in FP64 throughout:
//
//   Y  = Z_equiv Omega        Omega p x l with iid complex Gaussian entries
//   Q  = qr(Y)                Householder (explicit Q, p x l)
//   G  = Z_equiv^H Q          so Z_equiv ~ Q G^H
//   G  = Q2 R2                Householder
//   [R2^H ; I] W  ->  [T ; W] one-sided Jacobi: T = R2^H W has orthogonal
//                             columns, sigma_a = |t_a|, W unitary
//   Z_equiv ~ (Q T diag(1/sigma)) diag(sigma) (Q2 W)^H, hence
//   Z_shift = Q2 (W (diag(w) (T^H (Q^H Z_orig))))
//             with w_a = 1/sigma_a^2 for sigma_a >= cut, else 0 -- the
//             reference's cut rule applied to the same singular values.
//
// The sketch is accepted when its smallest sigma_a lies below
// capture * sigma_max: Y then reached Z_equiv's rounding floor (about 1e-14
// sigma0 for these kernels), so Q holds every direction above the cut to
// within that floor.  Otherwise the block is sketched again with l doubled.
// No atomics: results are reproducible bit for bit.
#include <cuda_runtime.h>

#include <cooperative_groups.h>

#include <algorithm>
#include <array>
#include <map>
#include <cmath>
#include <cstdint>
#include <vector>

#include "bfg_device.cuh"
#include "bfg_kernels.cuh"

namespace bfg {

namespace {

constexpr double kEpsS = 2.220446049250313e-16;
constexpr int kSketchMaxSweeps = 60;
constexpr int kSketchCluster = 8;      // CTAs per block in cluster mode
constexpr int kGT = 64, kGK = 16;      // GEMM tile and K chunk
constexpr int kFillTile = 16384;       // entries per fill CTA

// one block of the randomized path, as the kernels read it (offsets in
// complex entries from the scratch base)
struct SketchDev {
  int32_t kind, p, n, l;
  int64_t arenaOff, s0;
  double corig[3], ceq[3], cchk[3];
  double k;
  uint64_t seed;
  int64_t oZ, oB0, oB1, oB2, oM, oZo, oC, oD, oTau, oSW, oFlags;
};

struct FillTileDesc {
  int32_t blk, what;        // what: 0 Z_equiv, 1 Omega, 2 Z_orig
  int32_t cnt, pad;
  int64_t e0;
};

struct GemmDesc {
  double2 const *A, *B;
  double2 *C;
  double const *rowScale;   // optional: row i of C scaled by rowScale[i]
  int64_t lda, ldb, ldc;
  int32_t M, N, K, opA;     // opA 0: A is M x K; 1: C = A^H B with A stored K x M
  double const *colScale;   // optional: column j of C scaled by colScale[j]
};

struct HqrDesc {
  double2 *A;     // rows x cols, ld rows: overwritten by the reflectors and R
  double2 *Q;     // rows x cols, ld rows: receives the explicit Q
  double2 *tau;   // cols
  double2 *Rt;    // optional: R^H (cols x cols, lower triangular) and the
                  // identity below it, ld = 2 cols
  int32_t rows, cols;
};

struct JacobiDesc {
  double2 *M;     // ld x cols; dot products over the first rowsDot rows,
                  // rotations over all ld rows
  double *s2;     // cols: squared column norms over the first rowsDot rows
  int32_t *flags; // kSketchCluster ints (cluster mode)
  int32_t cols, rowsDot, ld, pad;
};

struct WeightDesc {
  double const *s2;
  double *w;
  int32_t cols, p;          // p: order of Z_equiv (the reference cut's max(m, n))
};

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// a complex Gaussian with iid N(0,1) parts from a counter (Box-Muller)
__device__ __forceinline__ double2 gaussianAt(uint64_t seed, int64_t e) {
  uint64_t const h1 = splitmix64(seed ^ ((uint64_t)e * 0xD1B54A32D192ED03ull));
  uint64_t const h2 = splitmix64(h1);
  double const u1 = ((double)(h1 >> 11) + 0.5) * 0x1.0p-53;
  double const u2 = (double)(h2 >> 11) * 0x1.0p-53;
  double const r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  return make_double2(r * c, r * s);
}

template <int kMode>
struct SMem {
  static __device__ __forceinline__ double2 ld(double2 const *p) {
    if (kMode == 2) return __ldcg(p);   // other CTAs of the cluster write it
    return *p;
  }
  static __device__ __forceinline__ void st(double2 *p, double2 v) {
    if (kMode == 2) __stcg(p, v);
    else *p = v;
  }
  static __device__ __forceinline__ void sync() {
    if (kMode == 2) cooperative_groups::this_cluster().sync();
    else __syncthreads();
  }
};

// the CTA-wide sum, the same bits in every thread (and in every CTA that
// sums the same values)
__device__ __forceinline__ double blockSumAll(double v, double *red) {
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warpSum(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; ++w) t += red[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ double2 conjD(double2 a) { return make_double2(a.x, -a.y); }

// ---------------------------------------------------------------------------
// Z_equiv, Omega and Z_orig of every block, column-major (entry e: row
// e % p, column e / p).  Proxy points are those of the full path: theta_a =
// (2 pi / p) a on the check and equivalent circles, (2 pi / n) b on the
// source-child circle of a MIDDLE block.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) sketchFillKernel(SketchDev const *__restrict__ blks,
                                                        FillTileDesc const *__restrict__ tiles,
                                                        PointsDev src, KernelParams kp,
                                                        double2 *scratch) {
  FillTileDesc const t = tiles[blockIdx.x];
  SketchDev const b = blks[t.blk];
  kp.k = b.k;
  int const p = b.p;
  double const scaleP = kTwoPiDev / (double)p;
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;
  double2 *out = scratch + (t.what == 0 ? b.oZ : t.what == 1 ? b.oB0 : b.oZo);
  for (int q = threadIdx.x; q < t.cnt; q += blockDim.x) {
    int64_t const e = t.e0 + q;
    if (t.what == 1) {
      out[e] = gaussianAt(b.seed, e);
      continue;
    }
    int const i = (int)(e % p);
    int64_t const j = e / p;
    double s, c;
    sincos(scaleP * i, &s, &c);
    double const tx = b.cchk[2] * c + b.cchk[0], ty = b.cchk[2] * s + b.cchk[1];
    double sx, sy, snx, sny;
    if (t.what == 0) {
      double s2, c2;
      sincos(scaleP * (int)j, &s2, &c2);
      sx = b.ceq[2] * c2 + b.ceq[0];
      sy = b.ceq[2] * s2 + b.ceq[1];
      snx = c2;
      sny = s2;
    } else if (b.kind == kFirst) {
      int64_t const sj = b.s0 + j;
      sx = src.x[sj];
      sy = src.y[sj];
      snx = (useSrcN && src.nx) ? src.nx[sj] : 0.0;
      sny = (useSrcN && src.ny) ? src.ny[sj] : 0.0;
    } else {
      double s2, c2;
      sincos((kTwoPiDev / (double)b.n) * (int)j, &s2, &c2);
      sx = b.corig[2] * c2 + b.corig[0];
      sy = b.corig[2] * s2 + b.corig[1];
      snx = c2;
      sny = s2;
    }
    out[e] = kernelValue(kp, tx, ty, 0.0, 0.0, sx, sy, snx, sny);
  }
}

// ---------------------------------------------------------------------------
// Batched complex FP64 GEMM, C = diag(rowScale) op(A) B, one 64 x 64 tile
// per CTA (tiles of all problems in one launch).  16 x 16 threads, each a
// 4 x 4 register tile (rows ty + 16 r, columns tx + 16 c); A and B staged
// through shared memory in chunks of 16 along K.  GB300's FP64 units (about
// 2 FMA per clock per SM) bound it; the staging is not the limit.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) zgemmKernel(GemmDesc const *__restrict__ descs,
                                                   int4 const *__restrict__ tiles) {
  int4 const t = tiles[blockIdx.x];
  GemmDesc const g = descs[t.x];
  int const i0 = t.y * kGT, j0 = t.z * kGT;
  __shared__ double2 As[kGK][kGT + 1];
  __shared__ double2 Bs[kGK][kGT + 1];
  int const tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double2 acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < g.K; k0 += kGK) {
    if (g.opA == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int const i = tid & 63, kk = (tid >> 6) + 4 * q;
        int const gi = i0 + i, gk = k0 + kk;
        As[kk][i] = (gi < g.M && gk < g.K) ? g.A[gi + (int64_t)gk * g.lda] : make_double2(0.0, 0.0);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int const kk = tid & 15, i = (tid >> 4) + 16 * q;
        int const gi = i0 + i, gk = k0 + kk;
        As[kk][i] = (gi < g.M && gk < g.K) ? conjD(g.A[gk + (int64_t)gi * g.lda])
                                           : make_double2(0.0, 0.0);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const kk = tid & 15, j = (tid >> 4) + 16 * q;
      int const gj = j0 + j, gk = k0 + kk;
      Bs[kk][j] = (gj < g.N && gk < g.K) ? g.B[gk + (int64_t)gj * g.ldb] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kGK; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          acc[r][c].x = fma(a[r].x, b[c].x, fma(-a[r].y, b[c].y, acc[r][c].x));
          acc[r][c].y = fma(a[r].x, b[c].y, fma(a[r].y, b[c].x, acc[r][c].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int const gi = i0 + ty + 16 * r;
    if (gi >= g.M) continue;
    double const sc = g.rowScale ? g.rowScale[gi] : 1.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int const gj = j0 + tx + 16 * c;
      if (gj < g.N) {
        double const scc = g.colScale ? sc * g.colScale[gj] : sc;
        g.C[gi + (int64_t)gj * g.ldc] = make_double2(scc * acc[r][c].x, scc * acc[r][c].y);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Householder QR (LAPACK zgeqr2 / zlarfg conventions: H = I - tau v v^H,
// v_0 = 1, H^H [alpha; x] = [beta; 0] with beta real) and the explicit Q
// (zung2r), one block per CTA (mode 1) or per cluster of kSketchCluster
// CTAs (mode 2).  Every CTA forms the reflector of column k itself (same
// sums, same bits); warps across the cluster update the trailing columns;
// CTA 0 stores the scaled reflector of column k while the others work on
// step k + 1, which no longer reads it, so each step ends at one barrier.
// ---------------------------------------------------------------------------
template <int kMode>
__global__ void __launch_bounds__(512) hqrKernel(HqrDesc const *__restrict__ descs) {
  using Mem = SMem<kMode>;
  int const ctas = kMode == 2 ? kSketchCluster : 1;
  int const blk = kMode == 2 ? (int)(blockIdx.x / kSketchCluster) : (int)blockIdx.x;
  int const rank = kMode == 2 ? (int)(blockIdx.x % kSketchCluster) : 0;
  HqrDesc const d = descs[blk];
  int const m = d.rows, nc = d.cols;
  int const tid = threadIdx.x, nthr = blockDim.x;
  int const lane = tid & 31, warp = tid >> 5, nWarps = nthr >> 5;
  int const gWarp = rank * nWarps + warp, gWarps = ctas * nWarps;
  __shared__ double red[32];
  double2 *A = d.A;

  double2 prevSc = make_double2(0.0, 0.0), prevTau = make_double2(0.0, 0.0);
  double prevBeta = 0.0;
  for (int k = 0; k < nc; ++k) {
    double2 const *col = A + (int64_t)k * m;
    double s = 0.0;
    for (int i = k + 1 + tid; i < m; i += nthr) {
      double2 const v = Mem::ld(col + i);
      s += v.x * v.x + v.y * v.y;
    }
    s = blockSumAll(s, red);
    double2 const alpha = Mem::ld(col + k);
    if (rank == 0 && k > 0) {
      double2 *pc = A + (int64_t)(k - 1) * m;
      for (int i = k + tid; i < m; i += nthr) Mem::st(pc + i, cmul(prevSc, Mem::ld(pc + i)));
      if (tid == 0) {
        Mem::st(pc + (k - 1), make_double2(prevBeta, 0.0));
        Mem::st(d.tau + (k - 1), prevTau);
      }
    }
    double2 tau, sc;
    double beta;
    if (s == 0.0 && alpha.y == 0.0) {
      tau = make_double2(0.0, 0.0);
      sc = make_double2(0.0, 0.0);
      beta = alpha.x;
    } else {
      beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + s), alpha.x);
      tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      double2 const den = make_double2(alpha.x - beta, alpha.y);   // sc = 1 / (alpha - beta)
      double const dd = den.x * den.x + den.y * den.y;
      sc = make_double2(den.x / dd, -den.y / dd);
    }
    // a_j -= conj(tau) v (v^H a_j) for j > k, v = [1; sc x]
    for (int j = k + 1 + gWarp; j < nc; j += gWarps) {
      double2 *cj = A + (int64_t)j * m;
      double sr = 0.0, si = 0.0;
      for (int i = k + 1 + lane; i < m; i += 32) {
        double2 const x = Mem::ld(col + i), a = Mem::ld(cj + i);
        sr = fma(x.x, a.x, fma(x.y, a.y, sr));
        si = fma(x.x, a.y, fma(-x.y, a.x, si));
      }
      sr = warpSum(sr);
      si = warpSum(si);
      double2 const akj = Mem::ld(cj + k);
      double2 const cs = cmul(conjD(sc), make_double2(sr, si));
      double2 const w = make_double2(akj.x + cs.x, akj.y + cs.y);
      double2 const tw = cmul(conjD(tau), w);
      double2 const f = cmul(sc, tw);
      __syncwarp();
      if (lane == 0) Mem::st(cj + k, make_double2(akj.x - tw.x, akj.y - tw.y));
      for (int i = k + 1 + lane; i < m; i += 32) {
        double2 const x = Mem::ld(col + i), a = Mem::ld(cj + i);
        double2 const u = cmul(f, x);
        Mem::st(cj + i, make_double2(a.x - u.x, a.y - u.y));
      }
    }
    Mem::sync();
    prevSc = sc;
    prevTau = tau;
    prevBeta = beta;
  }
  if (rank == 0 && nc > 0) {
    double2 *pc = A + (int64_t)(nc - 1) * m;
    for (int i = nc + tid; i < m; i += nthr) Mem::st(pc + i, cmul(prevSc, Mem::ld(pc + i)));
    if (tid == 0) {
      Mem::st(pc + (nc - 1), make_double2(prevBeta, 0.0));
      Mem::st(d.tau + (nc - 1), prevTau);
    }
  }
  Mem::sync();

  // R^H (lower triangular) and the identity below it
  if (d.Rt) {
    int64_t const ldR = 2 * (int64_t)nc, total = ldR * nc;
    for (int64_t e = (int64_t)rank * nthr + tid; e < total; e += (int64_t)ctas * nthr) {
      int const a = (int)(e % ldR), b = (int)(e / ldR);
      double2 v = make_double2(0.0, 0.0);
      if (a < nc) {
        if (a >= b) v = conjD(Mem::ld(A + b + (int64_t)a * m));
      } else if (a - nc == b) {
        v = make_double2(1.0, 0.0);
      }
      Mem::st(d.Rt + e, v);
    }
  }
  // Q = H_0 ... H_{nc-1} [I ; 0]
  double2 *Q = d.Q;
  {
    int64_t const total = (int64_t)m * nc;
    for (int64_t e = (int64_t)rank * nthr + tid; e < total; e += (int64_t)ctas * nthr)
      Mem::st(Q + e, make_double2((e % m) == (e / m) ? 1.0 : 0.0, 0.0));
  }
  Mem::sync();
  for (int i = nc - 1; i >= 0; --i) {
    double2 const t = Mem::ld(d.tau + i);
    double2 const *v = A + (int64_t)i * m;
    for (int j = i + gWarp; j < nc; j += gWarps) {
      double2 *qj = Q + (int64_t)j * m;
      double sr = 0.0, si = 0.0;
      for (int r = i + 1 + lane; r < m; r += 32) {
        double2 const x = Mem::ld(v + r), a = Mem::ld(qj + r);
        sr = fma(x.x, a.x, fma(x.y, a.y, sr));
        si = fma(x.x, a.y, fma(-x.y, a.x, si));
      }
      sr = warpSum(sr);
      si = warpSum(si);
      double2 const qij = Mem::ld(qj + i);
      double2 const w = make_double2(qij.x + sr, qij.y + si);
      double2 const tw = cmul(t, w);
      __syncwarp();
      if (lane == 0) Mem::st(qj + i, make_double2(qij.x - tw.x, qij.y - tw.y));
      for (int r = i + 1 + lane; r < m; r += 32) {
        double2 const x = Mem::ld(v + r), a = Mem::ld(qj + r);
        double2 const u = cmul(tw, x);
        Mem::st(qj + r, make_double2(a.x - u.x, a.y - u.y));
      }
    }
    Mem::sync();
  }
}

// ---------------------------------------------------------------------------
// One-sided Jacobi (Hestenes) on the columns of M, FP64: a round-robin pair
// schedule, one warp per column pair, rotation when |<x, y>| > eps sqrt(n)
// |x| |y|; sweeps until none rotates (cap kSketchMaxSweeps).  Then the
// squared column norms over the first rowsDot rows.
// ---------------------------------------------------------------------------
template <int kMode>
__global__ void __launch_bounds__(512) sketchJacobiKernel(JacobiDesc const *__restrict__ descs,
                                                          int32_t *status) {
  using Mem = SMem<kMode>;
  int const ctas = kMode == 2 ? kSketchCluster : 1;
  int const blk = kMode == 2 ? (int)(blockIdx.x / kSketchCluster) : (int)blockIdx.x;
  int const rank = kMode == 2 ? (int)(blockIdx.x % kSketchCluster) : 0;
  JacobiDesc const d = descs[blk];
  int const nc = d.cols, rd = d.rowsDot, LD = d.ld;
  int const tid = threadIdx.x, nthr = blockDim.x;
  int const lane = tid & 31, warp = tid >> 5, nWarps = nthr >> 5;
  int const gWarp = rank * nWarps + warp, gWarps = ctas * nWarps;
  double2 *M = d.M;
  __shared__ int sRotated;

  int const P = nc + (nc & 1), nPairs = P / 2;
  double const tolRot = kEpsS * sqrt((double)rd);
  bool converged = nc < 2;
  for (int sweep = 0; sweep < kSketchMaxSweeps && !converged; ++sweep) {
    if (tid == 0) sRotated = 0;
    __syncthreads();
    for (int round = 0; round < P - 1; ++round) {
      for (int pr = gWarp; pr < nPairs; pr += gWarps) {
        int i, j;
        if (pr == 0) {
          i = round;
          j = P - 1;
        } else {
          i = (round + pr) % (P - 1);
          j = (round - pr + (P - 1)) % (P - 1);
        }
        if (i >= nc || j >= nc) continue;
        double2 *ci = M + (int64_t)i * LD, *cj = M + (int64_t)j * LD;
        double al = 0, be = 0, gr = 0, gi = 0;
        for (int r = lane; r < rd; r += 32) {
          double2 const x = Mem::ld(ci + r), y = Mem::ld(cj + r);
          al = fma(x.x, x.x, fma(x.y, x.y, al));
          be = fma(y.x, y.x, fma(y.y, y.y, be));
          gr = fma(x.x, y.x, fma(x.y, y.y, gr));
          gi = fma(x.x, y.y, fma(-x.y, y.x, gi));
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
          double const er = gr / ag, ei = -gi / ag;
          __syncwarp();
          for (int r = lane; r < LD; r += 32) {
            double2 const x = Mem::ld(ci + r), y = Mem::ld(cj + r);
            double const ytr = y.x * er - y.y * ei, yti = y.x * ei + y.y * er;
            Mem::st(ci + r, make_double2(c * x.x - s * ytr, c * x.y - s * yti));
            Mem::st(cj + r, make_double2(s * x.x + c * ytr, s * x.y + c * yti));
          }
          if (lane == 0) sRotated = 1;
        }
      }
      Mem::sync();
    }
    int rotated = sRotated;
    if (kMode == 2) {
      if (tid == 0) __stcg(d.flags + rank, rotated);
      Mem::sync();
      rotated = 0;
      for (int q = 0; q < kSketchCluster; ++q) rotated |= __ldcg(d.flags + q);
      Mem::sync();   // the flags are rewritten by the next sweep
    }
    __syncthreads();
    if (!rotated) converged = true;
  }
  if (!converged && tid == 0 && rank == 0) atomicOr(status, kStatusJacobiNotConverged);
  for (int a = gWarp; a < nc; a += gWarps) {
    double2 const *ca = M + (int64_t)a * LD;
    double s2 = 0;
    for (int r = lane; r < rd; r += 32) {
      double2 const v = Mem::ld(ca + r);
      s2 += v.x * v.x + v.y * v.y;
    }
    s2 = warpSum(s2);
    if (lane == 0) d.s2[a] = s2;
  }
}

// pseudo-inverse weights with the reference's cut rule
// (mat_dense_complex.c:1797-1808: sigma < max(m,n) eps sigma0 + eps) or the
// relative cut sigma < tol sigma0 (linalg.c:26-36), and the capture test
__global__ void __launch_bounds__(256) sketchWeightsKernel(WeightDesc const *__restrict__ descs,
                                                           int32_t cutMode, double cutTol,
                                                           double capture, int32_t *fail) {
  WeightDesc const d = descs[blockIdx.x];
  __shared__ double rmax[32], rmin[32];
  double mx = 0.0, mn = INFINITY;
  for (int a = threadIdx.x; a < d.cols; a += blockDim.x) {
    mx = fmax(mx, d.s2[a]);
    mn = fmin(mn, d.s2[a]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  }
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    rmax[warp] = mx;
    rmin[warp] = mn;
  }
  __syncthreads();
  mx = 0.0;
  mn = INFINITY;
  for (int w = 0; w < nw; ++w) {
    mx = fmax(mx, rmax[w]);
    mn = fmin(mn, rmin[w]);
  }
  double const smax = sqrt(mx);
  double const cut = cutMode == 0 ? (double)d.p * kEpsS * smax + kEpsS : cutTol * smax;
  for (int a = threadIdx.x; a < d.cols; a += blockDim.x) {
    double const sa = sqrt(d.s2[a]);
    d.w[a] = (sa < cut || sa == 0.0) ? 0.0 : 1.0 / d.s2[a];
  }
  if (threadIdx.x == 0) fail[blockIdx.x] = sqrt(mn) > capture * smax ? 1 : 0;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Buf {
  void *p = nullptr;
  size_t bytes = 0;
  ~Buf() {
    if (p) cudaFree(p);
  }
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
};

template <typename T>
cudaError_t put(Buf &b, std::vector<T> const &v, cudaStream_t s) {
  cudaError_t e = b.ensure(std::max<size_t>(1, v.size()) * sizeof(T));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

uint64_t splitmixHost(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}


// modes of the HQR / Jacobi launches: a whole cluster for large blocks
bool hqrCluster(int64_t p, int64_t l) { return p * l >= (int64_t)1 << 17; }
bool jacobiCluster(int64_t l) { return l >= 160; }

cudaError_t launchGemms(std::vector<GemmDesc> const &g, Buf &dDesc, Buf &dTiles,
                        cudaStream_t s) {
  if (g.empty()) return cudaSuccess;
  std::vector<int4> tiles;
  // longest K first, so that the longest tiles start in the first wave
  std::vector<int> order(g.size());
  for (size_t i = 0; i < g.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g[a].K > g[b].K; });
  for (int i : order) {
    int const tm = (g[i].M + kGT - 1) / kGT, tn = (g[i].N + kGT - 1) / kGT;
    for (int a = 0; a < tm; ++a)
      for (int c = 0; c < tn; ++c) tiles.push_back(make_int4(i, a, c, 0));
  }
  if (tiles.empty()) return cudaSuccess;
  cudaError_t e = put(dDesc, g, s);
  if (e != cudaSuccess) return e;
  e = put(dTiles, tiles, s);
  if (e != cudaSuccess) return e;
  // grids are limited to 2^31 - 1 CTAs in x; one launch per 2^30 tiles
  size_t const step = (size_t)1 << 30;
  for (size_t t0 = 0; t0 < tiles.size(); t0 += step) {
    size_t const cnt = std::min(step, tiles.size() - t0);
    zgemmKernel<<<(unsigned)cnt, 256, 0, s>>>(static_cast<GemmDesc const *>(dDesc.p),
                                              static_cast<int4 const *>(dTiles.p) + t0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <int kMode>
cudaError_t launchHqr(std::vector<HqrDesc> const &v, Buf &d, cudaStream_t s) {
  if (v.empty()) return cudaSuccess;
  cudaError_t e = put(d, v, s);
  if (e != cudaSuccess) return e;
  if (kMode == 1) {
    hqrKernel<1><<<(unsigned)v.size(), 512, 0, s>>>(static_cast<HqrDesc const *>(d.p));
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(v.size() * kSketchCluster));
  cfg.blockDim = dim3(512);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kSketchCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, hqrKernel<2>, static_cast<HqrDesc const *>(d.p));
}

template <int kMode>
cudaError_t launchJacobi(std::vector<JacobiDesc> const &v, Buf &d, int32_t *status,
                         cudaStream_t s) {
  if (v.empty()) return cudaSuccess;
  cudaError_t e = put(d, v, s);
  if (e != cudaSuccess) return e;
  if (kMode == 1) {
    sketchJacobiKernel<1><<<(unsigned)v.size(), 512, 0, s>>>(
        static_cast<JacobiDesc const *>(d.p), status);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(v.size() * kSketchCluster));
  cfg.blockDim = dim3(512);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kSketchCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, sketchJacobiKernel<2>, static_cast<JacobiDesc const *>(d.p),
                            status);
}

}  // namespace

int32_t sketchWidth(FillDesc const &d, double widthScale, int32_t widthPad) {
  double const R = std::hypot(d.ceq[0] - d.cchk[0], d.ceq[1] - d.cchk[1]);
  double const est = R > 0.0 ? d.k * d.ceq[2] * d.cchk[2] / R : (double)d.m;
  double l = std::ceil((widthScale * est + widthPad) / 32.0) * 32.0;
  if (!(l < (double)d.m)) return d.m;
  return std::max<int32_t>(32, (int32_t)l);
}

cudaError_t runSketchReexpansion(std::vector<SketchInput> const &in, PointsDev src,
                                 KernelParams kp, int32_t cutMode, double cutTol, double capture,
                                 double2 *arena, int64_t budgetEntries, cudaStream_t s,
                                 std::vector<FillDesc> *fallback, SketchReport *rep) {
  *rep = SketchReport{};
  if (in.empty()) return cudaSuccess;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaEventCreate(&e0);
  if (err != cudaSuccess) return err;
  err = cudaEventCreate(&e1);
  if (err != cudaSuccess) {
    cudaEventDestroy(e0);
    return err;
  }
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } evs{e0, e1};
  cudaEventRecord(e0, s);

  // phase boundaries of each batch (timed after the batch's final sync)
  struct PhaseEvents {
    cudaEvent_t e[9] = {};
    ~PhaseEvents() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } pev;
  for (cudaEvent_t &x : pev.e)
    if ((err = cudaEventCreate(&x)) != cudaSuccess) return err;
  auto mark = [&](int i) { cudaEventRecord(pev.e[i], s); };

  // blocks with the same Z_equiv (rank, equivalent and check circles,
  // wavenumber) form one group: one sketch, QR and SVD; every member its own
  // Z_orig and Z_shift
  struct Group {
    std::vector<FillDesc> mem;
    int32_t l, fullOk;
  };
  std::vector<Group> queue;
  {
    std::map<std::array<double, 8>, size_t> key;
    for (SketchInput const &x : in) {
      std::array<double, 8> const k8 = {(double)x.d.m, x.d.ceq[0], x.d.ceq[1], x.d.ceq[2],
                                        x.d.cchk[0], x.d.cchk[1], x.d.cchk[2], x.d.k};
      auto it = key.find(k8);
      if (it == key.end()) {
        key.emplace(k8, queue.size());
        queue.push_back(Group{{x.d}, x.l, x.fullOk});
      } else {
        Group &g = queue[it->second];
        g.mem.push_back(x.d);
        g.l = std::max(g.l, x.l);
        g.fullOk = g.fullOk && x.fullOk;
      }
    }
  }
  // largest first, so that the longest groups start in the first wave
  auto cost = [](Group const &g) {
    double n = 0;
    for (auto const &d : g.mem) n += d.n;
    return (double)g.mem[0].m * g.l * (g.l + g.mem[0].m) + (double)g.l * g.mem[0].m * n;
  };
  std::stable_sort(queue.begin(), queue.end(),
                   [&](Group const &a, Group const &b) { return cost(a) > cost(b); });
  Buf scratch, dBlk, dTiles, dDesc, dHqr1, dHqr2, dJac1, dJac2, dW, dFail, dStatus;
  err = dStatus.ensure(sizeof(int32_t));
  if (err != cudaSuccess) return err;
  err = cudaMemsetAsync(dStatus.p, 0, sizeof(int32_t), s);
  if (err != cudaSuccess) return err;
  int32_t *status = static_cast<int32_t *>(dStatus.p);
  uint64_t seedCounter = 0x5EED5EEDull;

  size_t q0 = 0;
  while (q0 < queue.size()) {
    // a batch of groups within the scratch budget (at least one): descs
    // holds the groups' leaders (the sketch, QRs and SVD), then their
    // members (Z_orig and the output products), memberOf[i] the leader of
    // member nb + i
    std::vector<SketchDev> blks, mems;
    std::vector<size_t> memberOf;
    int64_t total = 0;
    size_t q1 = q0;
    while (q1 < queue.size()) {
      Group const &gr = queue[q1];
      int64_t const p = gr.mem[0].m, l = gr.l;
      int64_t e = p * p + 3 * p * l + 2 * l * l + l + l + 4;
      for (auto const &d : gr.mem) e += p * d.n + 2 * l * d.n;
      if (q1 > q0 && total + e > budgetEntries) break;
      FillDesc const &d0 = gr.mem[0];
      SketchDev b{};
      b.kind = d0.kind;
      b.p = d0.m;
      b.n = d0.n;
      b.l = gr.l;
      b.arenaOff = d0.arenaOff;
      b.s0 = d0.s0;
      for (int c = 0; c < 3; ++c) {
        b.corig[c] = d0.corig[c];
        b.ceq[c] = d0.ceq[c];
        b.cchk[c] = d0.cchk[c];
      }
      b.k = d0.k;
      b.seed = splitmixHost(seedCounter++);
      int64_t o = total;
      b.oZ = o; o += p * p;
      b.oB0 = o; o += p * l;
      b.oB1 = o; o += p * l;
      b.oB2 = o; o += p * l;
      b.oM = o; o += 2 * l * l;
      b.oTau = o; o += l;
      b.oSW = o; o += l;
      b.oFlags = o; o += 4;
      for (auto const &d : gr.mem) {
        SketchDev m = b;
        m.kind = d.kind;
        m.n = d.n;
        m.arenaOff = d.arenaOff;
        m.s0 = d.s0;
        for (int c = 0; c < 3; ++c) m.corig[c] = d.corig[c];
        m.oZo = o; o += p * d.n;
        m.oC = o; o += l * d.n;
        m.oD = o; o += l * d.n;
        mems.push_back(m);
        memberOf.push_back(blks.size());
      }
      total = o;
      blks.push_back(b);
      ++q1;
    }
    err = scratch.ensure((size_t)total * sizeof(double2));
    if (err != cudaSuccess) return err;
    double2 *S = static_cast<double2 *>(scratch.p);
    size_t const nb = blks.size();
    std::vector<SketchDev> descs = blks;
    descs.insert(descs.end(), mems.begin(), mems.end());

    // fill: Z_equiv and Omega per group, Z_orig per member
    mark(0);
    std::vector<FillTileDesc> tiles;
    auto addTiles = [&](size_t di, int w, int64_t cnt) {
      for (int64_t e0 = 0; e0 < cnt; e0 += kFillTile) {
        FillTileDesc t{};
        t.blk = (int32_t)di;
        t.what = w;
        t.e0 = e0;
        t.cnt = (int32_t)std::min<int64_t>(kFillTile, cnt - e0);
        tiles.push_back(t);
      }
    };
    for (size_t i = 0; i < nb; ++i) {
      addTiles(i, 0, (int64_t)blks[i].p * blks[i].p);
      addTiles(i, 1, (int64_t)blks[i].p * blks[i].l);
    }
    for (size_t i = 0; i < mems.size(); ++i)
      addTiles(nb + i, 2, (int64_t)mems[i].p * mems[i].n);
    if ((err = put(dBlk, descs, s)) != cudaSuccess) return err;
    if ((err = put(dTiles, tiles, s)) != cudaSuccess) return err;
    for (size_t t0 = 0; t0 < tiles.size(); t0 += ((size_t)1 << 30)) {
      size_t const cnt = std::min<size_t>((size_t)1 << 30, tiles.size() - t0);
      sketchFillKernel<<<(unsigned)cnt, 256, 0, s>>>(
          static_cast<SketchDev const *>(dBlk.p), static_cast<FillTileDesc const *>(dTiles.p) + t0,
          src, kp, S);
      if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }

    // Y = Z Omega
    mark(1);
    std::vector<GemmDesc> g;
    for (auto const &b : blks)
      g.push_back(GemmDesc{S + b.oZ, S + b.oB0, S + b.oB1, nullptr, b.p, b.p, b.p, b.p, b.l, b.p, 0});
    if ((err = launchGemms(g, dDesc, dTiles, s)) != cudaSuccess) return err;
    // Q = qr(Y) into B0
    mark(2);
    std::vector<HqrDesc> h1, h2;
    for (auto const &b : blks) {
      HqrDesc h{S + b.oB1, S + b.oB0, S + b.oTau, nullptr, b.p, b.l};
      (hqrCluster(b.p, b.l) ? h2 : h1).push_back(h);
    }
    if ((err = launchHqr<1>(h1, dHqr1, s)) != cudaSuccess) return err;
    if ((err = launchHqr<2>(h2, dHqr2, s)) != cudaSuccess) return err;
    // G = Z^H Q into B1
    mark(3);
    g.clear();
    for (auto const &b : blks)
      g.push_back(GemmDesc{S + b.oZ, S + b.oB0, S + b.oB1, nullptr, b.p, b.p, b.p, b.p, b.l, b.p, 1});
    if ((err = launchGemms(g, dDesc, dTiles, s)) != cudaSuccess) return err;
    // G = Q2 R2: Q2 into B2, [R2^H ; I] into M
    mark(4);
    h1.clear();
    h2.clear();
    for (auto const &b : blks) {
      HqrDesc h{S + b.oB1, S + b.oB2, S + b.oTau, S + b.oM, b.p, b.l};
      (hqrCluster(b.p, b.l) ? h2 : h1).push_back(h);
    }
    if ((err = launchHqr<1>(h1, dHqr1, s)) != cudaSuccess) return err;
    if ((err = launchHqr<2>(h2, dHqr2, s)) != cudaSuccess) return err;
    // Jacobi on [R2^H ; I]
    mark(5);
    std::vector<JacobiDesc> j1, j2;
    for (auto const &b : blks) {
      JacobiDesc j{};
      j.M = S + b.oM;
      j.s2 = reinterpret_cast<double *>(S + b.oSW);
      j.flags = reinterpret_cast<int32_t *>(S + b.oFlags);
      j.cols = b.l;
      j.rowsDot = b.l;
      j.ld = 2 * b.l;
      (jacobiCluster(b.l) ? j2 : j1).push_back(j);
    }
    if ((err = launchJacobi<1>(j1, dJac1, status, s)) != cudaSuccess) return err;
    if ((err = launchJacobi<2>(j2, dJac2, status, s)) != cudaSuccess) return err;
    // weights and capture
    mark(6);
    std::vector<WeightDesc> wd;
    for (auto const &b : blks) {
      double *sw = reinterpret_cast<double *>(S + b.oSW);
      wd.push_back(WeightDesc{sw, sw + b.l, b.l, b.p});
    }
    if ((err = put(dW, wd, s)) != cudaSuccess) return err;
    if ((err = dFail.ensure(nb * sizeof(int32_t))) != cudaSuccess) return err;
    sketchWeightsKernel<<<(unsigned)nb, 256, 0, s>>>(static_cast<WeightDesc const *>(dW.p),
                                                     cutMode, cutTol, capture,
                                                     static_cast<int32_t *>(dFail.p));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    std::vector<int32_t> failed(nb, 0);
    if ((err = cudaMemcpyAsync(failed.data(), dFail.p, nb * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               s)) != cudaSuccess)
      return err;
    if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return err;

    // accepted groups: X = Q2 (W (diag(w) (T^H (Q^H Z_orig)))) per member.
    // A group whose members have more columns in all than Z_equiv has rows
    // forms E = Q2 W and F^H = Q T diag(w) once (in the free Z and G
    // buffers), and each member then takes X = E (F Z_orig): two products
    // per member instead of four
    std::vector<GemmDesc> gc, gd, ge, gx, gE, gF;
    std::vector<char> fused(nb, 0);
    std::vector<Group> requeue;
    for (size_t i = 0; i < nb; ++i) {
      SketchDev const &b = blks[i];
      Group const &gr = queue[q0 + i];
      bool const full = b.l >= b.p;
      if (failed[i] && !full) {
        Group r = gr;
        r.l = std::min<int32_t>(b.p, 2 * b.l);
        rep->retries += (int64_t)gr.mem.size();
        if (r.fullOk && r.l > (int32_t)(0.8 * b.p)) {
          fallback->insert(fallback->end(), r.mem.begin(), r.mem.end());
          rep->fallbacks += (int64_t)gr.mem.size();
        } else {
          requeue.push_back(r);
        }
        continue;
      }
      rep->groups += 1;
      int64_t sumN = 0;
      for (auto const &d : gr.mem) sumN += d.n;
      if (sumN > b.p) {
        fused[i] = 1;
        double const *w = reinterpret_cast<double const *>(S + b.oSW) + b.l;
        gE.push_back(GemmDesc{S + b.oB2, S + b.oM + b.l, S + b.oZ, nullptr, b.p, 2 * b.l, b.p, b.p,
                              b.l, b.l, 0, nullptr});
        gF.push_back(GemmDesc{S + b.oB0, S + b.oM, S + b.oB1, nullptr, b.p, 2 * b.l, b.p, b.p, b.l,
                              b.l, 0, w});
      }
    }
    for (size_t mi = 0; mi < mems.size(); ++mi) {
      size_t const i = memberOf[mi];
      SketchDev const &b = blks[i];
      if (failed[i] && b.l < b.p) continue;
      SketchDev const &m = mems[mi];
      double const *w = reinterpret_cast<double const *>(S + b.oSW) + b.l;
      if (fused[i]) {
        // Y1 = F Z_orig = (F^H)^H Z_orig into C, X = E Y1
        gc.push_back(GemmDesc{S + b.oB1, S + m.oZo, S + m.oC, nullptr, b.p, b.p, b.l, b.l, m.n,
                              b.p, 1, nullptr});
        gx.push_back(GemmDesc{S + b.oZ, S + m.oC, arena + m.arenaOff, nullptr, b.p, b.l, b.p, b.p,
                              m.n, b.l, 0, nullptr});
      } else {
        gc.push_back(GemmDesc{S + b.oB0, S + m.oZo, S + m.oC, nullptr, b.p, b.p, b.l, b.l, m.n,
                              b.p, 1, nullptr});
        gd.push_back(GemmDesc{S + b.oM, S + m.oC, S + m.oD, w, 2 * b.l, b.l, b.l, b.l, m.n, b.l, 1,
                              nullptr});
        ge.push_back(GemmDesc{S + b.oM + b.l, S + m.oD, S + m.oC, nullptr, 2 * b.l, b.l, b.l, b.l,
                              m.n, b.l, 0, nullptr});
        gx.push_back(GemmDesc{S + b.oB2, S + m.oC, arena + m.arenaOff, nullptr, b.p, b.l, b.p, b.p,
                              m.n, b.l, 0, nullptr});
      }
      ++rep->blocks;
      rep->maxWidth = std::max<int64_t>(rep->maxWidth, b.l);
      rep->sumWidth += b.l;
    }
    mark(7);
    if ((err = launchGemms(gE, dDesc, dTiles, s)) != cudaSuccess) return err;
    if ((err = launchGemms(gF, dDesc, dTiles, s)) != cudaSuccess) return err;
    if ((err = launchGemms(gc, dDesc, dTiles, s)) != cudaSuccess) return err;
    if ((err = launchGemms(gd, dDesc, dTiles, s)) != cudaSuccess) return err;
    if ((err = launchGemms(ge, dDesc, dTiles, s)) != cudaSuccess) return err;
    if ((err = launchGemms(gx, dDesc, dTiles, s)) != cudaSuccess) return err;
    mark(8);
    // descriptors and scratch are reused by the next batch
    if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return err;
    for (int i = 0; i < 8; ++i) {
      float pm = 0.f;
      cudaEventElapsedTime(&pm, pev.e[i], pev.e[i + 1]);
      rep->phaseMs[i] += pm;
    }
    queue.insert(queue.end(), requeue.begin(), requeue.end());
    q0 = q1;
  }
  int32_t hst = 0;
  if ((err = cudaMemcpy(&hst, dStatus.p, sizeof hst, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return err;
  rep->notConverged = (hst & kStatusJacobiNotConverged) ? 1 : 0;
  cudaEventRecord(e1, s);
  if ((err = cudaEventSynchronize(e1)) != cudaSuccess) return err;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  rep->ms = ms;
  return cudaSuccess;
}

}  // namespace bfg
