// The boundary-integral system object shared by the solver (bfg_solver.cu)
// and the two-level preconditioner (bfg_coarse.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bfg.h"
#include "bfg_kernels.cuh"

namespace bfg {

// an owned device allocation that only grows
struct Dev {
  void *p = nullptr;
  size_t bytes = 0;
  Dev() = default;
  Dev(Dev const &) = delete;
  Dev &operator=(Dev const &) = delete;
  ~Dev() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 16));
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

}  // namespace bfg

struct bfgSystem_s {
  using Dev = bfg::Dev;
  bfgContext ctx = nullptr;
  bfgFac fac = nullptr;
  int64_t n = 0, numCurves = 0;
  int32_t order = 0;
  double shift = 0.5;
  bfgPrecision applyPrec = BFG_PRECISION_FP64;   // of the butterfly part
  bfg::KernelParams kp{};
  std::vector<int64_t> offsets;
  std::vector<double> weights;                   // host copy (coarse mode counts)
  Dev dOffsets, dCurveOf, dX, dW, dKrVal, dKrCol;
  Dev tmpXw, tmpK;
  // block-Jacobi
  bool haveBj = false, haveBj64 = false;   // the FP32 inverses; the FP64 ones (on first use)
  std::vector<int64_t> blkOff;
  Dev dBlkOff, dInv, dInv32, dWork, dColBuf, dPerm, dFlag;
  // learned preconditioner: chunks of consecutive points of a curve
  bfgMlp mlp = nullptr;
  int32_t chunk = 0;
  int64_t nChunks = 0;
  Dev dChunkStart, dChunkLen, dFeat, dOut, dScale, dZbj;
  // two-level preconditioner: per-curve Fourier coarse space Phi (curve b's
  // modes at coarse rows cStart[b] .. cStart[b+1], its basis table
  // n_b x M_b row-major complex64 at tabOff[b]), A_c = Phi^H A Phi and its
  // inverse (complex64, row-major)
  bool haveCoarse = false;
  int64_t coarseDim = 0;
  std::vector<int64_t> cStart, tabOff;
  Dev dCStart, dTabOff, dTab, dAc, dAcInv, dCoarseIn, dCoarseOut, dZ1, dT1, dT2;
  std::string err;
  cudaStream_t stream() const;
};

namespace bfg {
// A X for one device complex128 vector with the butterfly part in `prec`
bfgStatus systemApplyPrec(bfgSystem sys, bfgPrecision prec, void const *X, void *Y);
// z = M_bj r from the FP32 block inverses (block-Jacobi built)
void applyBlockJacobi32(bfgSystem sys, double2 const *r, double2 *z, cudaStream_t s);
// the two-level preconditioner z = z1 + M_bj (r - A z1), z1 = Phi A_c^-1 Phi^H r
bfgStatus applyTwoLevel(bfgSystem sys, double2 const *r, double2 *z);
// kernels shared with bfg_coarse.cu
void launchSubFrom(int64_t n, double2 const *x, double2 *y, cudaStream_t s);   // y = x - y
}  // namespace bfg
