// A small multilayer perceptron, trained and evaluated by hand-written FP32
// kernels: the learned right preconditioner of flexible GMRES on the
// multiple-scattering operator (a GB300 addition; the reference preconditions
// with block-Jacobi only, multiple_scattering_context.c:545-634).
//
// Network: x (nIn) -> relu(x W1 + b1) (nHidden) -> relu(. W2 + b2) (nHidden)
// -> . W3 + b3 (nOut), W_l row-major [in x out].  Loss: the mean over the
// batch of 0.5 ||y - t||^2.  Gradients by back-propagation, Adam updates.
// Every reduction runs in a fixed order (no atomics): the same batch gives
// the same gradients bit for bit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "bfg_mlp.cuh"

namespace bfg {
namespace {

// C (M x N, ldc) = op(A) op(B) [+ bias] [relu | * (mask > 0)], FP32.
// op(A) is M x K: A[m lda + k], or A[k lda + m] when transA; op(B) is K x N:
// B[k ldb + n], or B[n ldb + k] when transB.  64 x 64 tiles, K in steps of
// 16 through shared memory, 4 x 4 outputs per thread.
constexpr int kTile = 64, kTileK = 16;
template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
gemmKernel(int M, int N, int K, float const *__restrict__ A, int lda, float const *__restrict__ B,
           int ldb, float *__restrict__ C, int ldc, float const *__restrict__ bias, int epi,
           float const *__restrict__ mask, int ldm) {
  __shared__ float As[kTileK][kTile + 4];
  __shared__ float Bs[kTileK][kTile + 4];
  int const tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  int const m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTileK) {
    // 64 x 16 of op(A) and 16 x 64 of op(B): 4 elements per thread each
    for (int e = threadIdx.x; e < kTile * kTileK; e += 256) {
      int mm, kk;
      if (TA) {   // consecutive threads along m (contiguous in memory)
        mm = e % kTile;
        kk = e / kTile;
      } else {    // consecutive threads along k
        kk = e % kTileK;
        mm = e / kTileK;
      }
      int const gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = TA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
      As[kk][mm] = v;
    }
    for (int e = threadIdx.x; e < kTile * kTileK; e += 256) {
      int nn, kk;
      if (TB) {
        kk = e % kTileK;
        nn = e / kTileK;
      } else {
        nn = e % kTile;
        kk = e / kTile;
      }
      int const gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < K) v = TB ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTileK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int const gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int const gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (bias) v += bias[gn];
      if (epi == kEpiRelu) v = v > 0.f ? v : 0.f;
      if (epi == kEpiMask && !(mask[(int64_t)gm * ldm + gn] > 0.f)) v = 0.f;
      C[(int64_t)gm * ldc + gn] = v;
    }
  }
}

// out[n] = sum over rows of G (rows x N) in two fixed-order steps
constexpr int kColRows = 256;
__global__ void colSumPartKernel(int rows, int N, float const *__restrict__ G,
                                 float *__restrict__ part) {
  int const n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  int const r0 = blockIdx.y * kColRows, r1 = min(rows, r0 + kColRows);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += G[(int64_t)r * N + n];
  part[(int64_t)blockIdx.y * N + n] = s;
}
__global__ void colSumFinishKernel(int chunks, int N, float const *__restrict__ part,
                                   float *__restrict__ out) {
  int const n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int c = 0; c < chunks; ++c) s += part[(int64_t)c * N + n];
  out[n] = s;
}

// dY = (Y - T) / batch; per-row squared error to rowLoss
__global__ void mseGradKernel(int rows, int N, float const *__restrict__ Y,
                              float const *__restrict__ T, float *__restrict__ dY,
                              float *__restrict__ rowLoss) {
  int const r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  float s = 0.f;
  float const inv = 1.f / (float)rows;
  for (int n = 0; n < N; ++n) {
    float const d = Y[(int64_t)r * N + n] - T[(int64_t)r * N + n];
    s += d * d;
    dY[(int64_t)r * N + n] = d * inv;
  }
  rowLoss[r] = 0.5f * s;
}

__global__ void adamKernel(int64_t n, float *__restrict__ w, float const *__restrict__ g,
                           float *__restrict__ m, float *__restrict__ v, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float const gi = g[i];
    float const mi = b1 * m[i] + (1.f - b1) * gi;
    float const vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

int gridN(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

}  // namespace

cudaError_t launchGemm(bool transA, bool transB, int M, int N, int K, float const *A, int lda,
                       float const *B, int ldb, float *C, int ldc, float const *bias, int epi,
                       float const *mask, int ldm, cudaStream_t s) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  dim3 grid((unsigned)((N + kTile - 1) / kTile), (unsigned)((M + kTile - 1) / kTile));
  if (grid.y > 65535) return cudaErrorInvalidConfiguration;
  if (!transA && !transB)
    gemmKernel<false, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, epi, mask, ldm);
  else if (transA && !transB)
    gemmKernel<true, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, epi, mask, ldm);
  else if (!transA && transB)
    gemmKernel<false, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, epi, mask, ldm);
  else
    gemmKernel<true, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, epi, mask, ldm);
  return cudaGetLastError();
}

int64_t colSumScratch(int rows, int N) { return (int64_t)((rows + kColRows - 1) / kColRows) * N; }

cudaError_t launchColSum(int rows, int N, float const *G, float *scratch, float *out,
                         cudaStream_t s) {
  int const chunks = (rows + kColRows - 1) / kColRows;
  if (chunks == 0) return cudaMemsetAsync(out, 0, (size_t)N * sizeof(float), s);
  dim3 grid((unsigned)((N + 127) / 128), (unsigned)chunks);
  colSumPartKernel<<<grid, 128, 0, s>>>(rows, N, G, scratch);
  colSumFinishKernel<<<(N + 127) / 128, 128, 0, s>>>(chunks, N, scratch, out);
  return cudaGetLastError();
}

cudaError_t launchMseGrad(int rows, int N, float const *Y, float const *T, float *dY,
                          float *rowLoss, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  mseGradKernel<<<(rows + 255) / 256, 256, 0, s>>>(rows, N, Y, T, dY, rowLoss);
  return cudaGetLastError();
}

cudaError_t launchAdam(int64_t n, float *w, float const *g, float *m, float *v, float lr,
                       float b1, float b2, float eps, int64_t step, cudaStream_t s) {
  float const c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  adamKernel<<<gridN(n), 256, 0, s>>>(n, w, g, m, v, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace bfg
