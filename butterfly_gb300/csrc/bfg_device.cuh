// Device helpers shared by the CUDA sources of the factorization: complex
// product, the kernel value of each layer potential, warp sums.
#pragma once

#include <cuda_runtime.h>

#include "bfg_kernels.cuh"
#include "hankel.cuh"

namespace bfg {

constexpr double kTwoPiDev = 6.283185307179586;   // const.h BF_TWO_PI

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

// (accr, acci) += a x as four fused multiply-adds: written out, the compiler
// forms a multiply, an FMA and an add per part (six instructions), and the
// FP64 forms are bound by GB300's FP64 pipe
__device__ __forceinline__ void cmacc(float &accr, float &acci, float2 a, float2 x) {
  accr = fmaf(a.x, x.x, accr);
  accr = fmaf(-a.y, x.y, accr);
  acci = fmaf(a.x, x.y, acci);
  acci = fmaf(a.y, x.x, acci);
}
__device__ __forceinline__ void cmacc(double &accr, double &acci, double2 a, double2 x) {
  accr = fma(a.x, x.x, accr);
  accr = fma(-a.y, x.y, accr);
  acci = fma(a.x, x.y, acci);
  acci = fma(a.y, x.x, acci);
}

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace bfg
