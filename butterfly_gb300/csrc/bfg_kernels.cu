// CUDA kernels of the butterfly Helmholtz path (sm_103a).
//
//  * fillBlocksKernel      evaluation (LAST) and dense blocks: fused
//                          points -> distance -> H0/H1 -> complex entry,
//                          written column-major straight into the arena
//                          (helm2.c:93-319, fac_helm2.c:403-509, 741-775).
//  * reexpansionKernel     FIRST/MIDDLE blocks: both proxy kernel matrices
//                          (helm2.c:321-365) plus the pseudo-inverse
//                          least-squares solve (mat_dense_complex.c:1768-1849)
//                          by a one-sided Jacobi SVD (details at the kernel).
//  * applyGemvKernel /     one stage of the staged apply (single / many RHS),
//    applyTileKernel       each item a row chunk of one block row summing its
//                          blocks in order; no atomics, so results are
//                          reproducible bit for bit.
//  * applyReduceKernel     sums the per-product outputs into Y in a fixed
//                          order (the reference's block-dense accumulation,
//                          mat_block_dense.c:512-572), optionally scattering
//                          to original point order.
#include <cuda_runtime.h>

#include <cooperative_groups.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "bfg_device.cuh"
#include "bfg_kernels.cuh"
#include "hankel.cuh"

namespace bfg {

namespace {

constexpr double kTwoPiD = 6.283185307179586;   // const.h BF_TWO_PI
constexpr double kEps = 2.220446049250313e-16;
constexpr int kMaxSweeps = 60;

// ---------------------------------------------------------------------------
// LAST and DENSE blocks
// ---------------------------------------------------------------------------
__global__ void fillBlocksKernel(FillDesc const *__restrict__ descs, PointsDev src,
                                 PointsDev tgt, KernelParams kp, double2 *arena,
                                 int32_t *status) {
  extern __shared__ double proxy[];   // 4 * n for LAST blocks
  FillDesc const d = descs[blockIdx.x];
  kp.k = d.k;
  int const m = d.m, n = d.n;
  double2 *out = arena + d.arenaOff;
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;
  bool const useTgtN = kp.layerPot == kLpPvNormalDerivSingle;
  if (d.kind == kLast) {
    double const scale = kTwoPiD / (double)d.nTot;
    for (int b = threadIdx.x; b < n; b += blockDim.x) {
      double s, c;
      sincos(scale * (d.j0 + b), &s, &c);
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
//
// Z_shift = pinv(Z_equiv) Z_orig with Z_equiv p x p.  One-sided Jacobi on
// the columns of M = [Z_equiv^H ; I]: rotations Q make the top part
// T = Z_equiv^H Q column-orthogonal (T = V S) while the bottom part
// accumulates Q (= U).  Then pinv_k(Z_equiv) = T diag(w) Q^H with
// w_a = 1/s_a^2 for kept singular values, 0 otherwise, and every column of
// the output is x_j = T (w .* (Q^H z_j)), z_j = Z_orig[:, j] evaluated on
// the fly.  Modes: 0 = M in shared memory (one CTA), 1 = M in global
// scratch (one CTA), 2 = M in global scratch shared by a thread-block
// cluster of kClusterCtas CTAs that split every Jacobi round and meet at
// hardware cluster barriers.
// ---------------------------------------------------------------------------
constexpr int kClusterCtas = 8;

// ---- double-float arithmetic for the Jacobi sweeps (kDf): each complex
// entry of M held as FP32 pairs (re hi, re lo, im hi, im lo) in the same 16
// bytes, products by FMA error terms, sums by TwoSum (Dekker; Knuth TAOCP
// 4.2.2).  The _rn intrinsics are never contracted into FMAs, which would
// break the error-free steps.
__device__ __forceinline__ void jTwoSum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float const bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}
// (sh, sl) += (ah + al)(bh + bl), unnormalised
__device__ __forceinline__ void jMac(float ah, float al, float bh, float bl, float &sh, float &sl) {
  float const ph = __fmul_rn(ah, bh);
  float pl = fmaf(ah, bh, -ph);
  pl = fmaf(ah, bl, pl);
  pl = fmaf(al, bh, pl);
  float s, e;
  jTwoSum(sh, ph, s, e);
  sh = s;
  sl += e + pl;
}
__device__ __forceinline__ float2 jNorm(float h, float l) {
  float const s = __fadd_rn(h, l);
  return make_float2(s, __fsub_rn(l, __fsub_rn(s, h)));
}
__device__ __forceinline__ float2 jSplit(double d) {
  float const h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}
// the sum over the warp as a double; TwoSum is commutative, so every lane of
// the butterfly gets the same bits
__device__ __forceinline__ double jWarpSum(float h, float l) {
  for (int o = 16; o > 0; o >>= 1) {
    float const oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
    float s, e;
    jTwoSum(h, oh, s, e);
    h = s;
    l = __fadd_rn(e, __fadd_rn(l, ol));
  }
  return (double)h + (double)l;
}

template <int kMode, bool kDf>
struct ReexpMem {
  static __device__ __forceinline__ double2 ld(double2 const *p) {
    if (kMode == 2) return __ldcg(p);   // other SMs of the cluster write M
    return *p;
  }
  static __device__ __forceinline__ void st(double2 *p, double2 v) {
    if (kMode == 2) __stcg(p, v);
    else *p = v;
  }
  static __device__ __forceinline__ float4 ld4(double2 const *p) {
    float4 const *q = reinterpret_cast<float4 const *>(p);
    if (kMode == 2) return __ldcg(q);
    return *q;
  }
  static __device__ __forceinline__ void st4(double2 *p, float4 v) {
    float4 *q = reinterpret_cast<float4 *>(p);
    if (kMode == 2) __stcg(q, v);
    else *q = v;
  }
  // an entry of M as a complex double, whichever way it is held
  static __device__ __forceinline__ double2 ldC(double2 const *p) {
    if (!kDf) return ld(p);
    float4 const v = ld4(p);
    return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
  }
  static __device__ __forceinline__ void stC(double2 *p, double2 v) {
    if (!kDf) {
      st(p, v);
      return;
    }
    float2 const r = jSplit(v.x), i = jSplit(v.y);
    st4(p, make_float4(r.x, r.y, i.x, i.y));
  }
  static __device__ __forceinline__ void sync() {
    if (kMode == 2) cooperative_groups::this_cluster().sync();
    else __syncthreads();
  }
};

constexpr int kNoExp = -100000;   // no nonzero entry seen
constexpr int kColExpBias = 1100;  // makes ilogb of any positive double positive

// The double-float scale exponent s of a block: the largest e over its
// threads (|entry|^2 < 2^e) and the largest s with p^2 2^(e + 2s) <= 2^100,
// so that a column's squared norm stays below 2^100 / p (FP32 reaches 2^128)
// while its rounding-floor entries stay far above 2^-102, where the error
// terms of their products turn subnormal.  Mode 2 combines the cluster's
// CTAs through their flag slots (free until the first sweep ends); every
// thread of the block (or cluster) gets the same s.
template <int kMode>
__device__ int reexpScaleExp(int eTop, int p, int32_t *clusterFlags, int rank) {
  __shared__ int red[32];
  for (int o = 16; o > 0; o >>= 1) eTop = max(eTop, __shfl_xor_sync(0xffffffffu, eTop, o));
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nWarps = blockDim.x >> 5;
  if (lane == 0) red[warp] = eTop;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = kNoExp;
    for (int w = 0; w < nWarps; ++w) m = max(m, red[w]);
    red[0] = m;
    if (kMode == 2) __stcg(clusterFlags + rank, m);
  }
  if (kMode == 2) cooperative_groups::this_cluster().sync();
  else __syncthreads();
  int eMax = red[0];
  if (kMode == 2)
    for (int q = 0; q < kClusterCtas; ++q) eMax = max(eMax, __ldcg(clusterFlags + q));
  __syncthreads();   // red[] is read before any later use of the helper's storage
  if (eMax == kNoExp) return 0;
  int lp = 0;
  while ((1 << lp) < p) ++lp;
  int const t = 100 - 2 * lp - eMax;
  return t >= 0 ? t / 2 : -((1 - t) / 2);
}

// kDf: the Jacobi sweeps in double-float (~48 significant bits, FP32
// arithmetic, about 6x fewer FP64 instructions; the rotation angles, the
// singular values and the output stay FP64), else in FP64
// Blocks with the same Z_equiv (the same rank, equivalent and check circles
// and wavenumber) share one SVD: descriptor `blk` is a group's leader (its n
// the largest over the group), and with `members` non-null the group's
// blocks are members[groupStart[blk] .. groupStart[blk + 1]), each of which
// gets its own Z_shift from the one pseudo-inverse.
template <int kMode, bool kDf>
__global__ void __launch_bounds__(512) reexpansionKernel(
    FillDesc const *__restrict__ descs, PointsDev src, KernelParams kp, int32_t cutMode,
    double cutTol, double2 *arena, double2 *scratch, int64_t const *scratchOff,
    int32_t *flags, int32_t *status, FillDesc const *__restrict__ members,
    int32_t const *__restrict__ groupStart) {
  using Mem = ReexpMem<kMode, kDf>;
  extern __shared__ double2 smem2[];
  int const ctas = kMode == 2 ? kClusterCtas : 1;
  int const blk = kMode == 2 ? (int)(blockIdx.x / kClusterCtas) : (int)blockIdx.x;
  int const rank = kMode == 2 ? (int)(blockIdx.x % kClusterCtas) : 0;
  FillDesc const d = descs[blk];
  kp.k = d.k;
  int const p = d.m, n = d.n, LD = 2 * p;
  int const tid = threadIdx.x, nthr = blockDim.x;
  int const lane = tid & 31, warp = tid >> 5, nWarps = nthr >> 5;
  int const gWarp = rank * nWarps + warp, gWarps = ctas * nWarps;

  // working matrix M (LD x p), then per-warp vectors (2p each), then (in a
  // cluster) p shared squared singular values; see reexpansionScratchEntries
  double2 *M, *wscr;
  double *geo;
  if (kMode == 0) {
    M = smem2;
    wscr = smem2 + (int64_t)LD * p;
    geo = reinterpret_cast<double *>(wscr + (int64_t)2 * p * nWarps);
  } else {
    M = scratch + scratchOff[blk];
    wscr = M + (int64_t)LD * p;
    geo = reinterpret_cast<double *>(smem2);
  }
  double2 *myB = wscr + (int64_t)2 * p * (kMode == 0 ? warp : gWarp);
  double2 *myY = myB + p;
  double *chkX = geo, *chkY = geo + p;
  double *eqX = geo + 2 * p, *eqY = geo + 3 * p, *eqNx = geo + 4 * p, *eqNy = geo + 5 * p;
  double *orX = geo + 6 * p, *orY = orX + n, *orNx = orX + 2 * n, *orNy = orX + 3 * n;
  double *wgt = orX + 4 * n;
  __shared__ int sRotated;
  __shared__ unsigned long long sColMax;   // bits of a nonnegative double
  bool const useSrcN = kp.layerPot == kLpPvDouble || kp.layerPot == kLpCombinedField;

  // proxy geometry (every CTA of a cluster keeps its own copy); check points
  // on cchk and equivalent sources on ceq share theta_a = (2 pi / p) a
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
  }
  __syncthreads();

  // M[a*LD + r] = conj(K(chk_a, eq_r)) for r < p, identity below.
  // Double-float holds the top part scaled by 2^sExp (exact), sExp chosen
  // from the largest entry so that the sweeps' products stay far above
  // FP32's subnormal range: there the products' error terms lose their bits,
  // and pairs of columns at the rounding floor (sigma^2 ~ 1e-31 of the
  // largest) rotate on noise until the sweep cap.  FP64 keeps sExp = 0.
  int sExp = 0;
  {
    int64_t const total = (int64_t)LD * p;
    int eTop = kNoExp;   // exponent bound of the largest |entry|^2 this thread wrote
    for (int64_t e = (int64_t)rank * nthr + tid; e < total; e += (int64_t)ctas * nthr) {
      int const a = (int)(e / LD), r = (int)(e % LD);
      double2 v;
      if (r < p) {
        double2 k = kernelValue(kp, chkX[a], chkY[a], 0.0, 0.0, eqX[r], eqY[r], eqNx[r], eqNy[r]);
        v = make_double2(k.x, -k.y);
        double const m2 = v.x * v.x + v.y * v.y;
        if (kDf && m2 > 0.0) eTop = max(eTop, ilogb(m2) + 1);
      } else {
        v = make_double2(r - p == a ? 1.0 : 0.0, 0.0);
      }
      if (kDf) Mem::st(M + e, v);   // FP64 until the scale is known
      else Mem::stC(M + e, v);
    }
    if (kDf) {
      sExp = reexpScaleExp<kMode>(eTop, p, flags ? flags + (int64_t)blk * kClusterCtas : nullptr,
                                  rank);
      // every thread converts the entries it wrote
      for (int64_t e = (int64_t)rank * nthr + tid; e < total; e += (int64_t)ctas * nthr) {
        double2 v = Mem::ld(M + e);
        if ((int)(e % LD) < p) v = make_double2(ldexp(v.x, sExp), ldexp(v.y, sExp));
        Mem::stC(M + e, v);
      }
    }
  }
  Mem::sync();

  // one-sided Jacobi, round-robin pair schedule
  int const P = p + (p & 1);
  int const nPairs = P / 2;
  // rotation threshold: FP64 eps, or (double-float) 2^-44, well above the
  // rounding noise of the pair sums (2^-46 left a large block cycling to the
  // sweep cap)
  double const tolRot = (kDf ? 5.684341886080802e-14 : kEps) * sqrt((double)p);
  // double-float: columns far under the pseudo-inverse cut carry the
  // rounding noise (2^-48 of the largest columns) that every rotation of a
  // large column injects, and rotations on that noise would go on to the
  // sweep cap.  Measured against the previous sweep's largest column norm^2
  // (a lower bound of sigma_max^2): a pair whose columns both lie below
  // 1e-4 cut^2 is not rotated (only rotations with larger columns, which
  // still run, could lift them toward the cut), and one whose columns both
  // lie below 1e-2 cut^2 is rotated without holding the sweeps open --
  // neither can change the kept part of the pseudo-inverse.
  // The second band keeps a column just above the first from cycling against
  // the unrotated noise columns until the cap.
  double const cutRel = cutMode == 0 ? (double)p * kEps : cutTol;
  double skipBelow = 0.0, quietBelow = 0.0;
  bool converged = false;
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    if (tid == 0) {
      sRotated = 0;
      sColMax = 0ull;
    }
    __syncthreads();
    double colMax = 0.0;   // this warp's largest column norm^2 of the sweep
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
        if (i >= p || j >= p) continue;
        double2 *ci = M + (int64_t)i * LD, *cj = M + (int64_t)j * LD;
        double al = 0, be = 0, gr = 0, gi = 0;
        if (kDf) {
          float alh = 0, all = 0, beh = 0, bel = 0, grh = 0, grl = 0, gih = 0, gil = 0;
          for (int r = lane; r < p; r += 32) {
            float4 const x = Mem::ld4(ci + r), y = Mem::ld4(cj + r);
            jMac(x.x, x.y, x.x, x.y, alh, all);
            jMac(x.z, x.w, x.z, x.w, alh, all);
            jMac(y.x, y.y, y.x, y.y, beh, bel);
            jMac(y.z, y.w, y.z, y.w, beh, bel);
            jMac(x.x, x.y, y.x, y.y, grh, grl);      // conj(x) y
            jMac(x.z, x.w, y.z, y.w, grh, grl);
            jMac(x.x, x.y, y.z, y.w, gih, gil);
            jMac(-x.z, -x.w, y.x, y.y, gih, gil);
          }
          al = jWarpSum(alh, all);
          be = jWarpSum(beh, bel);
          gr = jWarpSum(grh, grl);
          gi = jWarpSum(gih, gil);
        } else {
          for (int r = lane; r < p; r += 32) {
            double2 x = Mem::ld(ci + r), y = Mem::ld(cj + r);
            al = fma(x.x, x.x, fma(x.y, x.y, al));
            be = fma(y.x, y.x, fma(y.y, y.y, be));
            gr = fma(x.x, y.x, fma(x.y, y.y, gr));     // conj(x) y
            gi = fma(x.x, y.y, fma(-x.y, y.x, gi));
          }
          al = warpSum(al);
          be = warpSum(be);
          gr = warpSum(gr);
          gi = warpSum(gi);
        }
        double const ag = sqrt(gr * gr + gi * gi);
        // double-float: a column below 1e-14 of its partner in norm lies far
        // under the pseudo-inverse cut; rotating it only cycles on rounding
        if (kDf) colMax = fmax(colMax, fmax(al, be));
        bool const negligible =
            kDf && (fmin(al, be) <= 1e-28 * fmax(al, be) || fmax(al, be) < skipBelow);
        if (!negligible && ag > tolRot * sqrt(al * be) && ag > 0.0) {
          double const zeta = (be - al) / (2.0 * ag);
          double const t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          double const c = 1.0 / sqrt(1.0 + t * t), s = c * t;
          double const er = gr / ag, ei = -gi / ag;   // exp(-i phi) = conj(gamma)/|gamma|
          if (kDf) {
            float2 const cD = jSplit(c), sD = jSplit(s), erD = jSplit(er), eiD = jSplit(ei);
            for (int r = lane; r < LD; r += 32) {
              float4 const x = Mem::ld4(ci + r), y = Mem::ld4(cj + r);
              float h, l;
              // yt = y exp(-i phi)
              h = 0.f, l = 0.f;
              jMac(y.x, y.y, erD.x, erD.y, h, l);
              jMac(-y.z, -y.w, eiD.x, eiD.y, h, l);
              float2 const ytr = jNorm(h, l);
              h = 0.f, l = 0.f;
              jMac(y.x, y.y, eiD.x, eiD.y, h, l);
              jMac(y.z, y.w, erD.x, erD.y, h, l);
              float2 const yti = jNorm(h, l);
              // x' = c x - s yt, y' = s x + c yt
              h = 0.f, l = 0.f;
              jMac(cD.x, cD.y, x.x, x.y, h, l);
              jMac(-sD.x, -sD.y, ytr.x, ytr.y, h, l);
              float2 const xr = jNorm(h, l);
              h = 0.f, l = 0.f;
              jMac(cD.x, cD.y, x.z, x.w, h, l);
              jMac(-sD.x, -sD.y, yti.x, yti.y, h, l);
              float2 const xi = jNorm(h, l);
              h = 0.f, l = 0.f;
              jMac(sD.x, sD.y, x.x, x.y, h, l);
              jMac(cD.x, cD.y, ytr.x, ytr.y, h, l);
              float2 const yr = jNorm(h, l);
              h = 0.f, l = 0.f;
              jMac(sD.x, sD.y, x.z, x.w, h, l);
              jMac(cD.x, cD.y, yti.x, yti.y, h, l);
              float2 const yi = jNorm(h, l);
              Mem::st4(ci + r, make_float4(xr.x, xr.y, xi.x, xi.y));
              Mem::st4(cj + r, make_float4(yr.x, yr.y, yi.x, yi.y));
            }
          } else {
            for (int r = lane; r < LD; r += 32) {
              double2 x = Mem::ld(ci + r), y = Mem::ld(cj + r);
              double const ytr = y.x * er - y.y * ei, yti = y.x * ei + y.y * er;
              Mem::st(ci + r, make_double2(c * x.x - s * ytr, c * x.y - s * yti));
              Mem::st(cj + r, make_double2(s * x.x + c * ytr, s * x.y + c * yti));
            }
          }
          if (lane == 0 && (!kDf || fmax(al, be) >= quietBelow)) sRotated = 1;
        }
      }
      Mem::sync();
    }
    if (kDf) {
      if (lane == 0) atomicMax(&sColMax, (unsigned long long)__double_as_longlong(colMax));
      __syncthreads();
    }
    int rotated = sRotated;
    // the largest column norm^2 as a biased exponent (2^(colExp - bias) <= it)
    int colExp = 0;
    if (kDf) {
      double const cm = __longlong_as_double((long long)sColMax);
      colExp = cm > 0.0 ? ilogb(cm) + kColExpBias : 0;
    }
    if (kMode == 2) {
      // cluster-wide OR of the CTAs' flags (and maximum of their exponents),
      // read after a barrier so every CTA takes the same decisions
      if (tid == 0) __stcg(flags + (int64_t)blk * kClusterCtas + rank, rotated | (colExp << 1));
      Mem::sync();
      rotated = 0;
      colExp = 0;
      for (int q = 0; q < kClusterCtas; ++q) {
        int const v = __ldcg(flags + (int64_t)blk * kClusterCtas + q);
        rotated |= v & 1;
        colExp = max(colExp, v >> 1);
      }
    }
    __syncthreads();
    if (!rotated) {
      converged = true;
      break;
    }
    if (kDf && colExp > 0) {
      double const colMaxLow = ldexp(cutRel * cutRel, colExp - kColExpBias);
      skipBelow = 1e-4 * colMaxLow;
      quietBelow = 1e-2 * colMaxLow;
    }
  }
  if (!converged && tid == 0 && rank == 0) atomicOr(status, kStatusJacobiNotConverged);

  // singular values and the pseudo-inverse cut (mat_dense_complex.c:1797-1808)
  double2 *wg = kMode == 2 ? wscr + (int64_t)2 * p * gWarps : nullptr;   // shared sigma^2
  for (int a = gWarp; a < p; a += gWarps) {
    double2 const *ca = M + (int64_t)a * LD;
    double s2 = 0;
    for (int r = lane; r < p; r += 32) {
      double2 v = Mem::ldC(ca + r);
      s2 += v.x * v.x + v.y * v.y;
    }
    s2 = warpSum(s2);
    if (kDf) s2 = ldexp(s2, -2 * sExp);   // sigma^2 of the unscaled block
    if (lane == 0) {
      if (kMode == 2) Mem::st(wg + a, make_double2(s2, 0.0));
      else wgt[a] = s2;
    }
  }
  Mem::sync();
  if (kMode == 2)
    for (int a = tid; a < p; a += nthr) wgt[a] = Mem::ld(wg + a).x;
  __syncthreads();
  if (tid == 0) {
    double smax = 0;
    for (int a = 0; a < p; ++a) smax = fmax(smax, sqrt(wgt[a]));
    double const cut = cutMode == 0 ? (double)p * kEps * smax + kEps : cutTol * smax;
    for (int a = 0; a < p; ++a) {
      double const sa = sqrt(wgt[a]);
      // (double-float: T holds 2^sExp of its columns, so 2^-sExp goes here)
      wgt[a] = (sa < cut || sa == 0.0) ? 0.0 : ldexp(1.0 / wgt[a], -sExp);
    }
  }
  __syncthreads();

  // every block of the group: its source points (Z_orig's columns), then
  // x_j = T (w .* (Q^H z_j)), one warp per output column
  int const g0 = members ? groupStart[blk] : 0, g1 = members ? groupStart[blk + 1] : 1;
  for (int gm = g0; gm < g1; ++gm) {
  FillDesc const dm = members ? members[gm] : d;
  int const nm = dm.n;
  if (dm.kind == kFirst) {
    for (int b = tid; b < nm; b += nthr) {
      int64_t const sj = dm.s0 + b;
      orX[b] = src.x[sj];
      orY[b] = src.y[sj];
      orNx[b] = (useSrcN && src.nx) ? src.nx[sj] : 0.0;
      orNy[b] = (useSrcN && src.ny) ? src.ny[sj] : 0.0;
    }
  } else {
    double const scale2 = kTwoPiD / (double)nm;
    for (int b = tid; b < nm; b += nthr) {
      double s, c;
      sincos(scale2 * b, &s, &c);
      orX[b] = dm.corig[2] * c + dm.corig[0];
      orY[b] = dm.corig[2] * s + dm.corig[1];
      orNx[b] = c;
      orNy[b] = s;
    }
  }
  __syncthreads();
  double2 *out = arena + dm.arenaOff;
  for (int j = gWarp; j < nm; j += gWarps) {
    for (int r = lane; r < p; r += 32) {
      double2 z = kernelValue(kp, chkX[r], chkY[r], 0.0, 0.0, orX[j], orY[j], orNx[j], orNy[j]);
      myB[r] = z;
    }
    __syncwarp();
    for (int a = 0; a < p; ++a) {
      double const w = wgt[a];
      if (w == 0.0) {
        if (lane == 0) myY[a] = make_double2(0.0, 0.0);
        continue;
      }
      double2 const *qa = M + (int64_t)a * LD + p;
      double yr = 0, yi = 0;
      for (int r = lane; r < p; r += 32) {
        double2 q = Mem::ldC(qa + r), z = myB[r];
        yr = fma(q.x, z.x, fma(q.y, z.y, yr));        // conj(q) z
        yi = fma(q.x, z.y, fma(-q.y, z.x, yi));
      }
      yr = warpSum(yr);
      yi = warpSum(yi);
      if (lane == 0) myY[a] = make_double2(w * yr, w * yi);
    }
    __syncwarp();
    for (int i = lane; i < p; i += 32) {
      double sr = 0, si = 0;
      for (int a = 0; a < p; ++a) {
        double2 const y = myY[a];
        if (y.x == 0.0 && y.y == 0.0) continue;
        double2 const t = Mem::ldC(M + (int64_t)a * LD + i);
        cmacc(sr, si, t, y);
      }
      out[(int64_t)j * p + i] = make_double2(sr, si);
    }
    __syncwarp();
  }
  __syncthreads();   // the next member's points overwrite these
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
        cmacc(accr[c], acci[c], kv, xv);
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

// FP64 fused multiply-add throughput: 8 independent chains per thread, the
// result written so that nothing is optimised away
__global__ void __launch_bounds__(256) fp64RateKernel(int32_t iters, double seed, double *out) {
  double a[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) a[c] = seed + 1e-3 * (threadIdx.x + 8 * c);
  double const b = 0.9999999, d = 1e-9;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = fma(a[c], b, d);
  double t = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) t += a[c];
  if (t == 12345.678) out[blockIdx.x] = t;   // never true for these inputs
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
                                float2 *b, int64_t ldb, int64_t bTile, int64_t bTileStride) {
  int64_t const total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / cols, j = e % cols;
    double2 v = a[i * lda + j];
    int64_t const o = bTile ? (j / bTile) * bTileStride + i * bTile + j % bTile : i * ldb + j;
    b[o] = make_float2((float)v.x, (float)v.y);
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

// R == 1: one CTA of 8 warps per item; lane = output row, warp w takes the
// columns j = w, w + 8, ... of every block in the row, four columns in
// flight at once; the 8 partial sums are reduced in shared memory in a
// fixed order.
constexpr int kGemvWarps = 8;

template <typename T2>
__global__ void __launch_bounds__(32 * kGemvWarps)
applyGemvKernel(ApplyItem const *__restrict__ items, ApplyContrib const *__restrict__ contribs,
                T2 const *__restrict__ arena, T2 const *__restrict__ X, int64_t ldx,
                T2 *__restrict__ W) {
  using T = typename Real<T2>::T;
  __shared__ T2 part[kGemvWarps][32];
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ApplyItem const it = items[blockIdx.x];
  bool const active = lane < it.rows;
  T accr = 0, acci = 0;
  for (int c = 0; c < it.nContrib; ++c) {
    ApplyContrib const cb = contribs[it.contrib0 + c];
    T2 const *a = arena + cb.aOff + lane;
    T2 const *x = cb.inIsX ? X + cb.inRow * ldx : W + cb.inRow;
    int64_t const xs = cb.inIsX ? ldx : 1;
    int const n = cb.n;
    int64_t const lda = cb.lda;
    int j = warp;
    constexpr int S = kGemvWarps;
    for (; j + 3 * S < n; j += 4 * S) {
      T2 a0, a1, a2, a3;
      if (active) {
        a0 = a[(int64_t)(j + 0 * S) * lda];
        a1 = a[(int64_t)(j + 1 * S) * lda];
        a2 = a[(int64_t)(j + 2 * S) * lda];
        a3 = a[(int64_t)(j + 3 * S) * lda];
      } else {
        a0 = a1 = a2 = a3 = mk2<T2>(0, 0);
      }
      T2 const x0 = x[(j + 0 * S) * xs], x1 = x[(j + 1 * S) * xs];
      T2 const x2 = x[(j + 2 * S) * xs], x3 = x[(j + 3 * S) * xs];
      cmacc(accr, acci, a0, x0);
      cmacc(accr, acci, a1, x1);
      cmacc(accr, acci, a2, x2);
      cmacc(accr, acci, a3, x3);
    }
    for (; j < n; j += S) {
      T2 const a0 = active ? a[(int64_t)j * lda] : mk2<T2>(0, 0);
      T2 const x0 = x[j * xs];
      cmacc(accr, acci, a0, x0);
    }
  }
  part[warp][lane] = mk2<T2>(accr, acci);
  __syncthreads();
  if (warp == 0 && active) {
    T sr = 0, si = 0;
#pragma unroll
    for (int w = 0; w < kGemvWarps; ++w) {
      sr += part[w][lane].x;
      si += part[w][lane].y;
    }
    W[it.outRow + lane] = mk2<T2>(sr, si);
  }
}

// two adjacent complex values from shared memory (16-byte aligned)
__device__ __forceinline__ void load2(float2 const *p, float2 &a, float2 &b) {
  float4 const v = *reinterpret_cast<float4 const *>(p);
  a = make_float2(v.x, v.y);
  b = make_float2(v.z, v.w);
}
__device__ __forceinline__ void load2(double2 const *p, double2 &a, double2 &b) {
  a = p[0];
  b = p[1];
}

// Asynchronous global -> shared copies (LDGSTS) of one complex entry; the
// 16-byte form bypasses L1 (stored blocks are read once per launch).
__device__ __forceinline__ void cpAsyncEntry(float2 *dst, float2 const *src) {
  unsigned const d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncEntry(double2 *dst, double2 const *src) {
  unsigned const d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// R > 1, pipelined: one CTA of NW warps per (item, tile of 16 RHS).  The
// item's contributions are walked in chunks of up to KC columns; each chunk's
// A panel (rows x columns) and X panel (columns x 16 RHS) are copied into
// shared memory with cp.async, one chunk ahead of the one being multiplied,
// so every load of a chunk is in flight at once instead of one column per
// round trip.  Warp w multiplies the columns w, w+NW, ... of each chunk; a
// lane owns 4 rows x 4 RHS of the 32 x 16 tile (4 vector shared loads per
// 16 complex MACs) in 16 register accumulators; the NW partial 32 x 16 tiles
// are summed in shared memory in a fixed order.  Rows >= item rows and RHS
// >= R are never copied: they only reach accumulators that are not stored.
template <typename T2>
struct PipeShape {
  static constexpr int KC = 32;   // 12 KB (FP32) / 24 KB (FP64) per stage
  static constexpr int RT = 16;
  static constexpr size_t stageBytes = (size_t)KC * (32 + RT) * sizeof(T2);
};
constexpr int kPipeWarps = 4;

template <typename T2, int NW, int S>
__global__ void __launch_bounds__(32 * NW, sizeof(T2) == 8 ? 8 : 4) applyPipeKernel(
    ApplyItem const *__restrict__ items, ApplyContrib const *__restrict__ contribs,
    T2 const *__restrict__ arena, T2 const *__restrict__ X, int64_t ldx,
    T2 *__restrict__ W, int64_t R) {
  using T = typename Real<T2>::T;
  constexpr int KC = PipeShape<T2>::KC, RT = PipeShape<T2>::RT, TH = 32 * NW;
  static_assert((size_t)NW * RT * 32 <= (size_t)S * KC * 32, "partials must fit in sA");
  extern __shared__ __align__(16) unsigned char pipeSmem[];
  T2 *const sA = reinterpret_cast<T2 *>(pipeSmem);   // [S][KC][32]
  T2 *const sX = sA + S * KC * 32;                   // [S][KC][RT]
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int const rg = lane & 7, cg = lane >> 3;   // lane's rows 4rg.., RHS 4cg..
  ApplyItem const it = items[blockIdx.x];
  int64_t const r0 = (int64_t)blockIdx.y * RT;
  int const nr = (R - r0) < RT ? (int)(R - r0) : RT;
  int const rows = it.rows;

  // issue cursor over (contribution, first column); uniform across the CTA
  int ci = 0, cj = 0;
  ApplyContrib icb{};
  if (it.nContrib > 0) icb = contribs[it.contrib0];
  int ncBuf[S];
  int issued = 0;
  // copies the next chunk (if any) into stage `slot`, then commits a group
  // (an empty one at the end, so that group counts stay in step)
  auto tryIssue = [&](int slot) {
    if (ci < it.nContrib) {
      int const nc = min(KC, icb.n - cj);
      T2 const *a = arena + icb.aOff + (int64_t)cj * icb.lda;
      int64_t const lda = icb.lda;
      for (int e = threadIdx.x; e < nc * 32; e += TH) {
        int const col = e >> 5, row = e & 31;
        if (row < rows) cpAsyncEntry(&sA[(slot * KC + col) * 32 + row], a + col * lda + row);
      }
      int64_t const xld = icb.inIsX ? ldx : R;
      T2 const *x =
          (icb.inIsX ? X + icb.inRow * ldx : W + icb.inRow * R) + r0 + (int64_t)cj * xld;
      for (int e = threadIdx.x; e < nc * RT; e += TH) {
        int const col = e / RT, q = e % RT;
        if (q < nr) cpAsyncEntry(&sX[(slot * KC + col) * RT + q], x + col * xld + q);
      }
      ncBuf[slot] = nc;
      ++issued;
      cj += nc;
      if (cj >= icb.n) {
        ++ci;
        cj = 0;
        if (ci < it.nContrib) icb = contribs[it.contrib0 + ci];
      }
    }
    cpAsyncCommit();
  };

  T accr[RT], acci[RT];
#pragma unroll
  for (int q = 0; q < RT; ++q) accr[q] = acci[q] = 0;

#pragma unroll
  for (int sl = 0; sl < S - 1; ++sl) tryIssue(sl);
  for (int i = 0; i < issued; ++i) {
    tryIssue((i + S - 1) % S);   // the stage multiplied in the previous pass
    cpAsyncWait<S - 1>();         // chunk i has landed
    __syncthreads();
    int const slot = i % S;
    int const nc = ncBuf[slot];
    T2 const *pa = sA + slot * KC * 32 + 4 * rg;
    T2 const *px = sX + slot * KC * RT + 4 * cg;
    for (int col = warp; col < nc; col += NW) {
      T2 a[4], x[4];
      load2(pa + col * 32, a[0], a[1]);
      load2(pa + col * 32 + 2, a[2], a[3]);
      load2(px + col * RT, x[0], x[1]);
      load2(px + col * RT + 2, x[2], x[3]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          cmacc(accr[4 * u + q], acci[4 * u + q], a[u], x[q]);
        }
    }
    __syncthreads();
  }
  cpAsyncWait<0>();

  T2 *const part = sA;   // [NW][RT][32], reuses the drained stage buffers
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int q = 0; q < 4; ++q)
      part[(warp * RT + 4 * cg + q) * 32 + 4 * rg + u] =
          mk2<T2>(accr[4 * u + q], acci[4 * u + q]);
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * RT; e += TH) {
    int const row = e & 31, q = e >> 5;
    if (row >= rows || q >= nr) continue;
    T sr = 0, si = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      T2 const v = part[(w * RT + q) * 32 + row];
      sr += v.x;
      si += v.y;
    }
    W[(it.outRow + row) * R + r0 + q] = mk2<T2>(sr, si);
  }
}

// R > 1: one CTA per (item, RHS tile of RT columns); 32 rows x RT outputs,
// A and X staged through shared memory in chunks of KC columns.
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
          cmacc(accr[q], acci[q], a, b);
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
                                  int64_t const *__restrict__ outPerm, int64_t wTile,
                                  int64_t wTileStride) {
  using T = typename Real<T2>::T;
  int64_t const total = nRows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / R, r = e % R;
    int const s = rowSeg[i];
    int64_t const di = i - segStart[s];
    // W row-major (ld R), or tile-major: panels of wTile columns
    T2 const *Wc = wTile ? W + (r / wTile) * wTileStride + r % wTile : W + r;
    int64_t const ldw = wTile ? wTile : R;
    T sr = 0, si = 0;
    for (int64_t c = segContrib0[s]; c < segContrib0[s + 1]; ++c) {
      T2 const v = Wc[(segBase[c] + di) * ldw];
      sr += v.x;
      si += v.y;
    }
    int64_t const oi = outPerm ? outPerm[i] : i;
    Y[oi * ldy + r] = mk2<T2>(sr, si);
  }
}

template <typename T2>
__global__ void gatherRowsKernel(T2 const *X, int64_t ldx, int64_t const *perm,
                                 int64_t nRows, int64_t R, T2 *out, int64_t outTile,
                                 int64_t outTileStride) {
  int64_t const total = nRows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / R, r = e % R;
    int64_t const o = outTile ? (r / outTile) * outTileStride + i * outTile + r % outTile : e;
    out[o] = X[(perm ? perm[i] : i) * ldx + r];
  }
}

// Multi-RHS kernel choice: the pipelined kernel above 8 RHS, the shared-memory
// tile kernel up to 8 (the pipelined kernel computes 16 RHS per CTA); the
// environment variable BFG_APPLY_KERNEL=tile forces the tile kernel for every
// R > 1 (for A/B measurements).
bool forceTileKernel() {
  static bool v = [] {
    char const *e = std::getenv("BFG_APPLY_KERNEL");
    return e && std::strcmp(e, "tile") == 0;
  }();
  return v;
}

int gridFor(int64_t total, int threads) {
  int64_t g = (total + threads - 1) / threads;
  if (g > 152 * 64) g = 152 * 64;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

int64_t reexpansionSmemBytes(int32_t m, int32_t n, int32_t warps) {
  return (int64_t)16 * (2 * (int64_t)m * m + 2 * (int64_t)m * warps) +
         reexpansionGeoBytes(m, n);
}

int64_t reexpansionGeoBytes(int32_t m, int32_t n) {
  return (int64_t)8 * (7 * (int64_t)m + 4 * (int64_t)n);
}

int64_t reexpansionScratchEntries(int32_t m, int32_t warps) {
  // M (2m x m), 2m per warp, m shared squared singular values
  int64_t e = 2 * (int64_t)m * m + 2 * (int64_t)m * warps + m;
  return (e + 15) & ~int64_t(15);
}

int32_t reexpansionClusterCtas() { return kClusterCtas; }

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

template <bool kDf>
cudaError_t launchReexpansionT(FillDesc const *descs, int32_t nDesc, PointsDev src,
                               KernelParams kp, int32_t cutMode, double cutTol,
                               double2 *arena, double2 *scratch, int64_t const *scratchOff,
                               int32_t *flags, int32_t *status, int32_t mode,
                               int32_t smemBytes, int32_t threads, cudaStream_t stream,
                               FillDesc const *members, int32_t const *groupStart) {
  if (nDesc == 0) return cudaSuccess;
  cudaError_t e;
  if (mode == 0) {
    e = cudaFuncSetAttribute(reexpansionKernel<0, kDf>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smemBytes);
    if (e != cudaSuccess) return e;
    reexpansionKernel<0, kDf><<<nDesc, threads, smemBytes, stream>>>(
        descs, src, kp, cutMode, cutTol, arena, scratch, scratchOff, flags, status, members,
        groupStart);
  } else if (mode == 1) {
    e = cudaFuncSetAttribute(reexpansionKernel<1, kDf>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smemBytes);
    if (e != cudaSuccess) return e;
    reexpansionKernel<1, kDf><<<nDesc, threads, smemBytes, stream>>>(
        descs, src, kp, cutMode, cutTol, arena, scratch, scratchOff, flags, status, members,
        groupStart);
  } else {
    e = cudaFuncSetAttribute(reexpansionKernel<2, kDf>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smemBytes);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)nDesc * kClusterCtas, 1, 1);
    cfg.blockDim = dim3((unsigned)threads, 1, 1);
    cfg.dynamicSmemBytes = (size_t)smemBytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, reexpansionKernel<2, kDf>, descs, src, kp, cutMode, cutTol,
                           arena, scratch, scratchOff, flags, status, members, groupStart);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t launchReexpansion(FillDesc const *descs, int32_t nDesc, PointsDev src,
                              KernelParams kp, int32_t cutMode, double cutTol,
                              double2 *arena, double2 *scratch, int64_t const *scratchOff,
                              int32_t *flags, int32_t *status, int32_t mode,
                              int32_t smemBytes, int32_t threads, int32_t doubleFloat,
                              cudaStream_t stream, FillDesc const *members,
                              int32_t const *groupStart) {
  if (doubleFloat)
    return launchReexpansionT<true>(descs, nDesc, src, kp, cutMode, cutTol, arena, scratch,
                                    scratchOff, flags, status, mode, smemBytes, threads, stream,
                                    members, groupStart);
  return launchReexpansionT<false>(descs, nDesc, src, kp, cutMode, cutTol, arena, scratch,
                                   scratchOff, flags, status, mode, smemBytes, threads, stream,
                                   members, groupStart);
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

cudaError_t launchFp64Rate(int32_t blocks, int32_t iters, double *out, cudaStream_t stream) {
  fp64RateKernel<<<(unsigned)blocks, 256, 0, stream>>>(iters, 0.5, out);
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
                            float2 *b, int64_t ldb, cudaStream_t stream, int64_t bTile,
                            int64_t bTileStride) {
  if (rows * cols == 0) return cudaSuccess;
  c128ToC64Kernel<<<gridFor(rows * cols, 256), 256, 0, stream>>>(a, lda, rows, cols, b, ldb,
                                                                 bTile, bTileStride);
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
    applyGemvKernel<T2><<<(unsigned)nItems, 32 * kGemvWarps, 0, stream>>>(items, contribs,
                                                                          arena, X, ldx, W);
  } else if (R > 8 && !forceTileKernel()) {
    size_t const smem = 2 * PipeShape<T2>::stageBytes;
    // the shared-memory limit is a per-device function attribute: set it once
    // per device, so that applies enqueue nothing else (stream capture)
    static std::atomic<uint64_t> attrSet{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    uint64_t const bit = 1ull << (dev & 63);
    if (!(attrSet.load() & bit)) {
      e = cudaFuncSetAttribute(applyPipeKernel<T2, kPipeWarps, 2>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      attrSet.fetch_or(bit);
    }
    dim3 grid((unsigned)nItems, (unsigned)((R + 15) / 16));
    applyPipeKernel<T2, kPipeWarps, 2><<<grid, 32 * kPipeWarps, smem, stream>>>(
        items, contribs, arena, X, ldx, W, R);
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
                              cudaStream_t stream, int64_t wTile, int64_t wTileStride) {
  applyReduceKernel<T2><<<gridFor(nRows * R, 256), 256, 0, stream>>>(
      rowSeg, segStart, segContrib0, segBase, W, R, Y, ldy, nRows, outPerm, wTile, wTileStride);
  return cudaGetLastError();
}

template <typename T2>
cudaError_t launchGatherRows(T2 const *X, int64_t ldx, int64_t const *perm,
                             int64_t nRows, int64_t R, T2 *out, cudaStream_t stream,
                             int64_t outTile, int64_t outTileStride) {
  gatherRowsKernel<T2><<<gridFor(nRows * R, 256), 256, 0, stream>>>(X, ldx, perm, nRows, R,
                                                                    out, outTile, outTileStride);
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
                                                cudaStream_t, int64_t, int64_t);
template cudaError_t launchApplyReduce<float2>(int32_t const *, int64_t const *, int64_t const *,
                                               int64_t const *, float2 const *, int64_t, float2 *,
                                               int64_t, int64_t, int64_t const *, cudaStream_t,
                                               int64_t, int64_t);
template cudaError_t launchGatherRows<double2>(double2 const *, int64_t, int64_t const *, int64_t,
                                               int64_t, double2 *, cudaStream_t, int64_t, int64_t);
template cudaError_t launchGatherRows<float2>(float2 const *, int64_t, int64_t const *, int64_t,
                                              int64_t, float2 *, cudaStream_t, int64_t, int64_t);

}  // namespace bfg
