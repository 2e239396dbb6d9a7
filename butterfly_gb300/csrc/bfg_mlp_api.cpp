// C ABI of the MLP (bfgMlp*): parameters, forward pass, gradients and Adam
// steps on the GPU through the hand-written kernels of bfg_mlp.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bfg.h"
#include "bfg_mlp.cuh"

struct bfgMlp_s {
  bfgContext ctx = nullptr;
  int32_t nIn = 0, nHid = 0, nOut = 0;
  int64_t nParams = 0;
  int64_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  int64_t step = 0;
  // per-batch scratch: H1, H2 (batch x nHid), Y, dY (batch x nOut), dH2, dH1
  // (batch x nHid), row losses (batch), column-sum scratch
  float *scratch = nullptr;
  int64_t scratchBatch = 0;
  std::vector<float> hostLoss;
  ~bfgMlp_s() {
    for (float *p : {params, grads, m, v, scratch})
      if (p) cudaFree(p);
  }
  cudaStream_t stream() const {
    void *s = nullptr;
    bfgContextGetStream(ctx, &s);
    return static_cast<cudaStream_t>(s);
  }
  int64_t perRow() const { return 4 * (int64_t)nHid + 2 * (int64_t)nOut + 1; }
  bool ensureScratch(int64_t batch) {
    if (batch <= scratchBatch) return true;
    if (scratch) cudaFree(scratch);
    scratch = nullptr;
    scratchBatch = 0;
    int64_t const cs = bfg::colSumScratch((int)batch, std::max(nHid, nOut));
    if (cudaMalloc(&scratch, (size_t)(batch * perRow() + cs) * sizeof(float)) != cudaSuccess)
      return false;
    scratchBatch = batch;
    return true;
  }
  float *H1() const { return scratch; }
  float *H2() const { return H1() + scratchBatch * nHid; }
  float *Y() const { return H2() + scratchBatch * nHid; }
  float *dY() const { return Y() + scratchBatch * nOut; }
  float *dH2() const { return dY() + scratchBatch * nOut; }
  float *dH1() const { return dH2() + scratchBatch * nHid; }
  float *rowLoss() const { return dH1() + scratchBatch * nHid; }
  float *colScratch() const { return rowLoss() + scratchBatch; }
};

namespace {

#define MLP_CK(expr)                              \
  do {                                            \
    if ((expr) != cudaSuccess) return BFG_ERROR_CUDA; \
  } while (0)

bfgStatus forwardOn(bfgMlp n, float const *X, int64_t batch, float *Y, cudaStream_t s) {
  int const B = (int)batch;
  float const *p = n->params;
  MLP_CK(bfg::launchGemm(false, false, B, n->nHid, n->nIn, X, n->nIn, p + n->oW1, n->nHid, n->H1(),
                         n->nHid, p + n->ob1, bfg::kEpiRelu, nullptr, 0, s));
  MLP_CK(bfg::launchGemm(false, false, B, n->nHid, n->nHid, n->H1(), n->nHid, p + n->oW2, n->nHid,
                         n->H2(), n->nHid, p + n->ob2, bfg::kEpiRelu, nullptr, 0, s));
  MLP_CK(bfg::launchGemm(false, false, B, n->nOut, n->nHid, n->H2(), n->nHid, p + n->oW3, n->nOut,
                         Y, n->nOut, p + n->ob3, bfg::kEpiNone, nullptr, 0, s));
  return BFG_OK;
}
bfgStatus forward(bfgMlp n, float const *X, int64_t batch, float *Y) {
  return forwardOn(n, X, batch, Y, n->stream());
}

// gradients of mean_b 0.5 ||y_b - t_b||^2 into n->grads; loss to *loss
bfgStatus backward(bfgMlp n, float const *X, float const *T, int64_t batch, double *loss) {
  cudaStream_t s = n->stream();
  int const B = (int)batch;
  float const *p = n->params;
  float *g = n->grads;
  bfgStatus st = forward(n, X, batch, n->Y());
  if (st != BFG_OK) return st;
  MLP_CK(bfg::launchMseGrad(B, n->nOut, n->Y(), T, n->dY(), n->rowLoss(), s));
  // layer 3: dW3 = H2^T dY, db3 = colsum dY, dH2 = (dY W3^T) * [H2 > 0]
  MLP_CK(bfg::launchGemm(true, false, n->nHid, n->nOut, B, n->H2(), n->nHid, n->dY(), n->nOut,
                         g + n->oW3, n->nOut, nullptr, bfg::kEpiNone, nullptr, 0, s));
  MLP_CK(bfg::launchColSum(B, n->nOut, n->dY(), n->colScratch(), g + n->ob3, s));
  MLP_CK(bfg::launchGemm(false, true, B, n->nHid, n->nOut, n->dY(), n->nOut, p + n->oW3, n->nOut,
                         n->dH2(), n->nHid, nullptr, bfg::kEpiMask, n->H2(), n->nHid, s));
  // layer 2
  MLP_CK(bfg::launchGemm(true, false, n->nHid, n->nHid, B, n->H1(), n->nHid, n->dH2(), n->nHid,
                         g + n->oW2, n->nHid, nullptr, bfg::kEpiNone, nullptr, 0, s));
  MLP_CK(bfg::launchColSum(B, n->nHid, n->dH2(), n->colScratch(), g + n->ob2, s));
  MLP_CK(bfg::launchGemm(false, true, B, n->nHid, n->nHid, n->dH2(), n->nHid, p + n->oW2, n->nHid,
                         n->dH1(), n->nHid, nullptr, bfg::kEpiMask, n->H1(), n->nHid, s));
  // layer 1
  MLP_CK(bfg::launchGemm(true, false, n->nIn, n->nHid, B, X, n->nIn, n->dH1(), n->nHid,
                         g + n->oW1, n->nHid, nullptr, bfg::kEpiNone, nullptr, 0, s));
  MLP_CK(bfg::launchColSum(B, n->nHid, n->dH1(), n->colScratch(), g + n->ob1, s));
  n->hostLoss.resize((size_t)B);
  MLP_CK(cudaMemcpyAsync(n->hostLoss.data(), n->rowLoss(), (size_t)B * sizeof(float),
                         cudaMemcpyDeviceToHost, s));
  MLP_CK(cudaStreamSynchronize(s));
  double sum = 0;
  for (float v : n->hostLoss) sum += v;
  if (loss) *loss = sum / (double)B;
  return BFG_OK;
}

}  // namespace

int bfg::mlpForwardOnStream(bfgMlp_s *n, float const *X, int64_t batch, float *Y,
                            cudaStream_t stream) {
  if (!n || !X || !Y || batch < 0 || batch > (1 << 30)) return BFG_ERROR_INVALID_ARGUMENTS;
  if (batch == 0) return BFG_OK;
  if (!n->ensureScratch(batch)) return BFG_ERROR_MEMORY;
  return forwardOn(n, X, batch, Y, stream);
}

extern "C" {

bfgStatus bfgMlpCreate(bfgContext ctx, int32_t nIn, int32_t nHidden, int32_t nOut, uint64_t seed,
                       bfgMlp *out) {
  if (!ctx || !out || nIn < 1 || nHidden < 1 || nOut < 1) return BFG_ERROR_INVALID_ARGUMENTS;
  *out = nullptr;
  auto *n = new (std::nothrow) bfgMlp_s;
  if (!n) return BFG_ERROR_MEMORY;
  n->ctx = ctx;
  n->nIn = nIn;
  n->nHid = nHidden;
  n->nOut = nOut;
  n->oW1 = 0;
  n->ob1 = n->oW1 + (int64_t)nIn * nHidden;
  n->oW2 = n->ob1 + nHidden;
  n->ob2 = n->oW2 + (int64_t)nHidden * nHidden;
  n->oW3 = n->ob2 + nHidden;
  n->ob3 = n->oW3 + (int64_t)nHidden * nOut;
  n->nParams = n->ob3 + nOut;
  size_t const bytes = (size_t)n->nParams * sizeof(float);
  for (float **p : {&n->params, &n->grads, &n->m, &n->v})
    if (cudaMalloc(p, bytes) != cudaSuccess) {
      delete n;
      return BFG_ERROR_MEMORY;
    }
  // He-uniform weights (ReLU layers), the output layer scaled by 0.1 so the
  // initial correction is small; zero biases
  std::vector<float> h((size_t)n->nParams, 0.f);
  bfgRng rng;
  bfgRngSeed(&rng, seed);
  auto fill = [&](int64_t off, int64_t count, int fanIn, double scale) {
    double const a = scale * std::sqrt(6.0 / fanIn);
    for (int64_t i = 0; i < count; ++i) h[(size_t)(off + i)] = (float)(a * (2 * bfgRngUniform1(&rng) - 1));
  };
  fill(n->oW1, (int64_t)nIn * nHidden, nIn, 1.0);
  fill(n->oW2, (int64_t)nHidden * nHidden, nHidden, 1.0);
  fill(n->oW3, (int64_t)nHidden * nOut, nHidden, 0.1);
  cudaStream_t s = n->stream();
  if (cudaMemcpyAsync(n->params, h.data(), bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(n->m, 0, bytes, s) != cudaSuccess ||
      cudaMemsetAsync(n->v, 0, bytes, s) != cudaSuccess ||
      cudaMemsetAsync(n->grads, 0, bytes, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    delete n;
    return BFG_ERROR_CUDA;
  }
  *out = n;
  return BFG_OK;
}

bfgStatus bfgMlpDestroy(bfgMlp n) {
  if (!n) return BFG_ERROR_INVALID_ARGUMENTS;
  cudaStreamSynchronize(n->stream());
  delete n;
  return BFG_OK;
}

bfgStatus bfgMlpGetShape(bfgMlp n, int32_t *nIn, int32_t *nHidden, int32_t *nOut) {
  if (!n || !nIn || !nHidden || !nOut) return BFG_ERROR_INVALID_ARGUMENTS;
  *nIn = n->nIn;
  *nHidden = n->nHid;
  *nOut = n->nOut;
  return BFG_OK;
}

bfgStatus bfgMlpNumParams(bfgMlp n, int64_t *count) {
  if (!n || !count) return BFG_ERROR_INVALID_ARGUMENTS;
  *count = n->nParams;
  return BFG_OK;
}

bfgStatus bfgMlpGetParams(bfgMlp n, float *params) {
  if (!n || !params) return BFG_ERROR_INVALID_ARGUMENTS;
  cudaStream_t s = n->stream();
  MLP_CK(cudaMemcpyAsync(params, n->params, (size_t)n->nParams * sizeof(float),
                         cudaMemcpyDeviceToHost, s));
  MLP_CK(cudaStreamSynchronize(s));
  return BFG_OK;
}

bfgStatus bfgMlpSetParams(bfgMlp n, float const *params) {
  if (!n || !params) return BFG_ERROR_INVALID_ARGUMENTS;
  cudaStream_t s = n->stream();
  MLP_CK(cudaMemcpyAsync(n->params, params, (size_t)n->nParams * sizeof(float),
                         cudaMemcpyHostToDevice, s));
  MLP_CK(cudaStreamSynchronize(s));
  n->step = 0;
  MLP_CK(cudaMemsetAsync(n->m, 0, (size_t)n->nParams * sizeof(float), s));
  MLP_CK(cudaMemsetAsync(n->v, 0, (size_t)n->nParams * sizeof(float), s));
  return BFG_OK;
}

bfgStatus bfgMlpForward(bfgMlp n, void const *X, int64_t batch, void *Y) {
  if (!n || !X || !Y || batch < 0 || batch > (1 << 30)) return BFG_ERROR_INVALID_ARGUMENTS;
  if (batch == 0) return BFG_OK;
  if (!n->ensureScratch(batch)) return BFG_ERROR_MEMORY;
  return forward(n, static_cast<float const *>(X), batch, static_cast<float *>(Y));
}

bfgStatus bfgMlpGradients(bfgMlp n, void const *X, void const *T, int64_t batch, float *grad,
                          double *loss) {
  if (!n || !X || !T || batch < 1 || batch > (1 << 30)) return BFG_ERROR_INVALID_ARGUMENTS;
  if (!n->ensureScratch(batch)) return BFG_ERROR_MEMORY;
  bfgStatus st = backward(n, static_cast<float const *>(X), static_cast<float const *>(T), batch, loss);
  if (st != BFG_OK) return st;
  if (grad) {
    cudaStream_t s = n->stream();
    MLP_CK(cudaMemcpyAsync(grad, n->grads, (size_t)n->nParams * sizeof(float),
                           cudaMemcpyDeviceToHost, s));
    MLP_CK(cudaStreamSynchronize(s));
  }
  return BFG_OK;
}

bfgStatus bfgMlpTrainStep(bfgMlp n, void const *X, void const *T, int64_t batch, float lr,
                          double *loss) {
  if (!n || !X || !T || batch < 1 || batch > (1 << 30) || !(lr > 0))
    return BFG_ERROR_INVALID_ARGUMENTS;
  if (!n->ensureScratch(batch)) return BFG_ERROR_MEMORY;
  bfgStatus st = backward(n, static_cast<float const *>(X), static_cast<float const *>(T), batch, loss);
  if (st != BFG_OK) return st;
  ++n->step;
  MLP_CK(bfg::launchAdam(n->nParams, n->params, n->grads, n->m, n->v, lr, 0.9f, 0.999f, 1e-8f,
                         n->step, n->stream()));
  return BFG_OK;
}

}  // extern "C"
