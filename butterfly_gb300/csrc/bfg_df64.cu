// Double-float ("df64") apply: the FP64 factors and vectors carried as
// pairs of FP32 numbers (hi + lo, ~48 significant bits) and multiplied with
// FP32 FMAs and their exact error terms.  GB300 runs FP64 at 1/64 of the
// FP32 rate, so the plain FP64 single-vector apply is bound by its FP64
// units (~1.2 TFLOP/s) rather than by HBM; with double-float arithmetic the
// same 16 bytes per stored entry stream at HBM speed and the result stays
// within ~1e-13 of FP64.  Same apply program as the other precisions
// (mat_block_dense.c:512-572, mat_product.c:211-245, one item = rows of one
// block row summing its blocks in order), no atomics, reproducible.
//
// Arithmetic (error-free transformations, Dekker 1971 / Knuth TAOCP 4.2.2;
// the FMA form of the product and the double-word sums of Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", 2017):
//   TwoSum(a, b)   = (s, e), s = fl(a + b), e = a + b - s exactly
//   TwoProd(a, b)  = (p, e), p = fl(a b),   e = fma(a, b, -p) exactly
//   (ah + al)(bh + bl) ~ ah bh + [fma(ah, bh, -ah bh) + ah bl + al bh]
// Each lane keeps its running sum unnormalised as (s, t): the high parts
// pass through TwoSum and every low-order term is added to t.
#include <cuda_runtime.h>

#include <cstdint>

#include "bfg_kernels.cuh"

namespace bfg {
namespace {

constexpr int kDfWarps = 8;

// The _rn intrinsics are never contracted into FMAs, which would break the
// error-free transformations.
__device__ __forceinline__ void twoSum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float const bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}
__device__ __forceinline__ void fastTwoSum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// (sh, sl) += (ah + al)(bh + bl), unnormalised
__device__ __forceinline__ void dfMac(float ah, float al, float bh, float bl, float &sh,
                                      float &sl) {
  float const ph = __fmul_rn(ah, bh);
  float pl = fmaf(ah, bh, -ph);
  pl = fmaf(ah, bl, pl);
  pl = fmaf(al, bh, pl);
  float s, e;
  twoSum(sh, ph, s, e);
  sh = s;
  sl += e + pl;
}
// (sh, sl) += (bh, bl)
__device__ __forceinline__ void dfAdd(float &sh, float &sl, float bh, float bl) {
  float s, e;
  twoSum(sh, bh, s, e);
  sh = s;
  sl += e + bl;
}
// a double as hi + lo
__device__ __forceinline__ float2 dfSplit(double d) {
  float const h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}
// complex entry: (re hi, re lo, im hi, im lo)
__device__ __forceinline__ float4 dfSplit(double2 v) {
  float2 const r = dfSplit(v.x), i = dfSplit(v.y);
  return make_float4(r.x, r.y, i.x, i.y);
}

__global__ void arenaToDfKernel(double2 const *__restrict__ a, float4 *__restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = dfSplit(a[i]);
}

// out (nRows x R, leading dimension R) = X rows (perm[i] or i), split
__global__ void gatherToDfKernel(double2 const *__restrict__ X, int64_t ldx,
                                 int64_t const *__restrict__ perm, int64_t nRows, int64_t R,
                                 float4 *__restrict__ out) {
  int64_t const total = nRows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / R, r = e % R;
    out[e] = dfSplit(X[(perm ? perm[i] : i) * ldx + r]);
  }
}

// One CTA per (item, RHS): lane = item row, the 8 warps take every 8th
// column with 4 entries in flight each; the warps' sums are combined in a
// fixed order.  X and W hold double-float rows with leading dimension R.
__global__ void __launch_bounds__(32 * kDfWarps)
applyGemvDfKernel(ApplyItem const *__restrict__ items, ApplyContrib const *__restrict__ contribs,
                  float4 const *__restrict__ arena, float4 const *__restrict__ X,
                  float4 *__restrict__ W, int64_t R) {
  __shared__ float4 part[kDfWarps][32];
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t const r = blockIdx.y;
  ApplyItem const it = items[blockIdx.x];
  bool const active = lane < it.rows;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  auto mac = [&](float4 a, float4 x) {
    // re += ar xr - ai xi, im += ar xi + ai xr
    dfMac(a.x, a.y, x.x, x.y, rh, rl);
    dfMac(-a.z, -a.w, x.z, x.w, rh, rl);
    dfMac(a.x, a.y, x.z, x.w, ih, il);
    dfMac(a.z, a.w, x.x, x.y, ih, il);
  };
  for (int c = 0; c < it.nContrib; ++c) {
    ApplyContrib const cb = contribs[it.contrib0 + c];
    float4 const *a = arena + cb.aOff + lane;
    float4 const *x = (cb.inIsX ? X : W) + cb.inRow * R + r;
    int const n = cb.n;
    int64_t const lda = cb.lda;
    constexpr int S = kDfWarps;
    int j = warp;
    for (; j + 3 * S < n; j += 4 * S) {
      float4 a0, a1, a2, a3;
      if (active) {
        a0 = a[(int64_t)(j + 0 * S) * lda];
        a1 = a[(int64_t)(j + 1 * S) * lda];
        a2 = a[(int64_t)(j + 2 * S) * lda];
        a3 = a[(int64_t)(j + 3 * S) * lda];
      } else {
        a0 = a1 = a2 = a3 = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      float4 const x0 = x[(int64_t)(j + 0 * S) * R], x1 = x[(int64_t)(j + 1 * S) * R];
      float4 const x2 = x[(int64_t)(j + 2 * S) * R], x3 = x[(int64_t)(j + 3 * S) * R];
      mac(a0, x0);
      mac(a1, x1);
      mac(a2, x2);
      mac(a3, x3);
    }
    for (; j < n; j += S) {
      float4 const a0 = active ? a[(int64_t)j * lda] : make_float4(0.f, 0.f, 0.f, 0.f);
      mac(a0, x[(int64_t)j * R]);
    }
  }
  part[warp][lane] = make_float4(rh, rl, ih, il);
  __syncthreads();
  if (warp == 0 && active) {
    float sh = 0.f, sl = 0.f, th = 0.f, tl = 0.f;
#pragma unroll
    for (int w = 0; w < kDfWarps; ++w) {
      float4 const v = part[w][lane];
      dfAdd(sh, sl, v.x, v.y);
      dfAdd(th, tl, v.z, v.w);
    }
    float a, b, c, d;
    fastTwoSum(sh, sl, a, b);
    fastTwoSum(th, tl, c, d);
    W[(it.outRow + lane) * R + r] = make_float4(a, b, c, d);
  }
}

// Y row i (outPerm[i] if given) = sum over the row's segment terms, in FP64
__global__ void applyReduceDfKernel(int32_t const *__restrict__ rowSeg,
                                    int64_t const *__restrict__ segStart,
                                    int64_t const *__restrict__ segContrib0,
                                    int64_t const *__restrict__ segBase,
                                    float4 const *__restrict__ W, int64_t R,
                                    double2 *__restrict__ Y, int64_t ldy, int64_t nRows,
                                    int64_t const *__restrict__ outPerm) {
  int64_t const total = nRows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t const i = e / R, r = e % R;
    int const s = rowSeg[i];
    int64_t const di = i - segStart[s];
    double sr = 0, si = 0;
    for (int64_t c = segContrib0[s]; c < segContrib0[s + 1]; ++c) {
      float4 const v = W[(segBase[c] + di) * R + r];
      sr += (double)v.x + (double)v.y;
      si += (double)v.z + (double)v.w;
    }
    int64_t const oi = outPerm ? outPerm[i] : i;
    Y[oi * ldy + r] = make_double2(sr, si);
  }
}

int gridDf(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

}  // namespace

cudaError_t launchArenaToDf(double2 const *a64, float4 *adf, int64_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  arenaToDfKernel<<<gridDf(n), 256, 0, stream>>>(a64, adf, n);
  return cudaGetLastError();
}

cudaError_t launchGatherToDf(double2 const *X, int64_t ldx, int64_t const *perm, int64_t nRows,
                             int64_t R, float4 *out, cudaStream_t stream) {
  if (nRows * R == 0) return cudaSuccess;
  gatherToDfKernel<<<gridDf(nRows * R), 256, 0, stream>>>(X, ldx, perm, nRows, R, out);
  return cudaGetLastError();
}

cudaError_t launchApplyStageDf(ApplyItem const *items, int64_t nItems,
                               ApplyContrib const *contribs, float4 const *arena,
                               float4 const *X, float4 *W, int64_t R, cudaStream_t stream) {
  if (nItems == 0) return cudaSuccess;
  if (R > 65535) return cudaErrorInvalidConfiguration;   // one grid row per RHS
  dim3 grid((unsigned)nItems, (unsigned)R);
  applyGemvDfKernel<<<grid, 32 * kDfWarps, 0, stream>>>(items, contribs, arena, X, W, R);
  return cudaGetLastError();
}

cudaError_t launchApplyReduceDf(int32_t const *rowSeg, int64_t const *segStart,
                                int64_t const *segContrib0, int64_t const *segBase,
                                float4 const *W, int64_t R, double2 *Y, int64_t ldy,
                                int64_t nRows, int64_t const *outPerm, cudaStream_t stream) {
  applyReduceDfKernel<<<gridDf(nRows * R), 256, 0, stream>>>(rowSeg, segStart, segContrib0,
                                                             segBase, W, R, Y, ldy, nRows,
                                                             outPerm);
  return cudaGetLastError();
}

}  // namespace bfg
