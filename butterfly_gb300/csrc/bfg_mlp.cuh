// Launchers of the MLP kernels (bfg_mlp.cu): FP32 GEMM with fused
// epilogues, deterministic column sums, the squared-error gradient and Adam.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace bfg {

// GEMM epilogues: none, relu, or zero where mask <= 0 (relu's derivative)
constexpr int kEpiNone = 0, kEpiRelu = 1, kEpiMask = 2;

// C (M x N, ldc) = op(A) (M x K) op(B) (K x N) [+ bias] [epilogue]; row-major
cudaError_t launchGemm(bool transA, bool transB, int M, int N, int K, float const *A, int lda,
                       float const *B, int ldb, float *C, int ldc, float const *bias, int epi,
                       float const *mask, int ldm, cudaStream_t s);
// floats of scratch launchColSum needs
int64_t colSumScratch(int rows, int N);
// out[n] = sum_r G[r N + n], in a fixed order
cudaError_t launchColSum(int rows, int N, float const *G, float *scratch, float *out,
                         cudaStream_t s);
// dY = (Y - T) / rows, rowLoss[r] = 0.5 ||Y_r - T_r||^2
cudaError_t launchMseGrad(int rows, int N, float const *Y, float const *T, float *dY,
                          float *rowLoss, cudaStream_t s);
// one Adam step (t = step >= 1) on n parameters
cudaError_t launchAdam(int64_t n, float *w, float const *g, float *m, float *v, float lr,
                       float b1, float b2, float eps, int64_t step, cudaStream_t s);

}  // namespace bfg

struct bfgMlp_s;
namespace bfg {
// bfgMlpForward on the given stream (the learned preconditioner runs it on
// its system's stream, whatever context the network was created on)
int mlpForwardOnStream(bfgMlp_s *mlp, float const *X, int64_t batch, float *Y,
                       cudaStream_t stream);

}  // namespace bfg
