// Kernel launchers shared between the C-ABI layer and the CUDA sources.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "bfg_plan.hpp"

namespace bfg {

// Layer potentials, numbered as the reference's BfLayerPotential
// (layer_pot.h:52-65).
enum LayerPot : int32_t {
  kLpSingle = 1,
  kLpPvDouble = 2,
  kLpPvNormalDerivSingle = 3,
  kLpCombinedField = 5,
};

struct KernelParams {
  double k;
  int32_t layerPot;        // layer potential of this fill
  int32_t pad;
  double alphaRe, alphaIm, betaRe, betaIm;
};

struct PointsDev {
  double const *x = nullptr, *y = nullptr;    // tree order
  double const *nx = nullptr, *ny = nullptr;  // unit normals or null
};

// status word bits written by the kernels
enum : int32_t {
  kStatusJacobiNotConverged = 1,
  kStatusBadDescriptor = 2,
};

// Fills LAST and DENSE blocks (plain kernel evaluation).
// maxProxyN bounds n over the LAST blocks of the launch (shared memory).
cudaError_t launchFillBlocks(FillDesc const *descs, int32_t nDesc, PointsDev src,
                             PointsDev tgt, KernelParams kp, double2 *arena,
                             int32_t maxProxyN, int32_t *status, cudaStream_t stream);

// Fills FIRST/MIDDLE blocks: proxy kernel matrices + pseudo-inverse
// re-expansion.  With `members`, descriptor i leads a group of blocks with
// the same Z_equiv (members[groupStart[i] .. groupStart[i + 1]), its n the
// largest of theirs): one SVD, every member's Z_shift.  mode 0: working matrix in shared memory (smemBytes =
// reexpansionSmemBytes); mode 1: in global `scratch` at scratchOff[block],
// one CTA per block; mode 2: in global scratch, one thread-block cluster of
// reexpansionClusterCtas() CTAs per block, `flags` holding one int per CTA.
// Modes 1 and 2 take smemBytes = reexpansionGeoBytes of the largest block.
cudaError_t launchReexpansion(FillDesc const *descs, int32_t nDesc, PointsDev src,
                              KernelParams kp, int32_t cutMode, double cutTol,
                              double2 *arena, double2 *scratch, int64_t const *scratchOff,
                              int32_t *flags, int32_t *status, int32_t mode,
                              int32_t smemBytes, int32_t threads, int32_t doubleFloat,
                              cudaStream_t stream, FillDesc const *members = nullptr,
                              int32_t const *groupStart = nullptr);

int64_t reexpansionSmemBytes(int32_t m, int32_t n, int32_t warps);
int64_t reexpansionGeoBytes(int32_t m, int32_t n);
// complex entries of global scratch one block needs; `warps` = all warps
// working on it (threads/32 times the CTAs per block)
int64_t reexpansionScratchEntries(int32_t m, int32_t warps);
int32_t reexpansionClusterCtas();

// FIRST/MIDDLE blocks by the randomized range finder (bfg_sketch.cu): one
// input per block with its initial sketch width l (<= m) and whether the
// full-Jacobi kernels could take it instead.
struct SketchInput {
  FillDesc d;
  int32_t l;
  int32_t fullOk;
};
struct SketchReport {
  int64_t blocks = 0;      // blocks computed by this path
  int64_t groups = 0;      // their distinct Z_equiv (one sketch and SVD each)
  int64_t retries = 0;     // sketches redone with a wider l
  int64_t fallbacks = 0;   // blocks handed back to the full path
  int64_t maxWidth = 0, sumWidth = 0;
  int32_t notConverged = 0;
  double ms = 0.0;         // device time of the whole path
  // device time per phase: fill, Y = Z Omega, qr(Y), G = Z^H Q, qr(G),
  // Jacobi, weights (+ capture check), output GEMMs
  double phaseMs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};
// initial sketch width: widthScale * k r1 r2 / R + widthPad rounded up to 32,
// at most m (R: distance of the equivalent and check circles' centres)
int32_t sketchWidth(FillDesc const &d, double widthScale, int32_t widthPad);
// Computes the blocks of `in` into the arena.  A block whose sketch missed
// part of Z_equiv's numerical rank (smallest sigma above capture * sigma0) is
// sketched again with twice the width, or, when that width passes 0.8 m and
// the full path can take it, appended to *fallback.  Scratch is allocated per
// batch of blocks within budgetEntries complex entries (at least one block).
cudaError_t runSketchReexpansion(std::vector<SketchInput> const &in, PointsDev src,
                                 KernelParams kp, int32_t cutMode, double cutTol, double capture,
                                 double2 *arena, int64_t budgetEntries, cudaStream_t stream,
                                 std::vector<FillDesc> *fallback, SketchReport *rep);

// Dense kernel rows: out[s*ldo + r] = sum_j K(t_rows[s], src_j) x[j*ldx + r]
cudaError_t launchDenseRows(PointsDev src, int64_t nSrc, PointsDev tgt,
                            int64_t const *rows, int64_t nRows, KernelParams kp,
                            double2 const *x, int64_t ldx, int64_t R, double2 *out,
                            int64_t ldo, cudaStream_t stream);

// Kernel matrix K(tgt_i, src_j), row-major m x n, points given directly.
cudaError_t launchKernelMatrix(PointsDev src, int64_t n, PointsDev tgt, int64_t m,
                               KernelParams kp, double2 *out, cudaStream_t stream);

// FP64 FMA throughput probe: blocks x 256 threads x iters x 8 FMAs
cudaError_t launchFp64Rate(int32_t blocks, int32_t iters, double *out, cudaStream_t stream);

// H0, H1 at x[i]: out[4i..4i+3] = J0, Y0, J1, Y1
cudaError_t launchBessel01(double const *x, int64_t n, double *out, cudaStream_t stream);

// FP64 -> FP32 arena conversion (same layout)
cudaError_t launchArenaToF32(double2 const *a64, float2 *a32, int64_t n, cudaStream_t stream);
// double-float apply (bfg_df64.cu): arena split, input split (and gather),
// stage, final sum into complex128
cudaError_t launchArenaToDf(double2 const *a64, float4 *adf, int64_t n, cudaStream_t stream);
cudaError_t launchGatherToDf(double2 const *X, int64_t ldx, int64_t const *perm, int64_t nRows,
                             int64_t R, float4 *out, cudaStream_t stream);
cudaError_t launchApplyStageDf(ApplyItem const *items, int64_t nItems,
                               ApplyContrib const *contribs, float4 const *arena,
                               float4 const *X, float4 *W, int64_t R, cudaStream_t stream);
cudaError_t launchApplyReduceDf(int32_t const *rowSeg, int64_t const *segStart,
                                int64_t const *segContrib0, int64_t const *segBase,
                                float4 const *W, int64_t R, double2 *Y, int64_t ldy,
                                int64_t nRows, int64_t const *outPerm, cudaStream_t stream);

// complex128 <-> complex64 matrix conversion (row-major, leading dims)
// (bTile > 0: b tile-major, panel t of bTile columns at b + t bTileStride,
// leading dimension bTile)
cudaError_t launchC128ToC64(double2 const *a, int64_t lda, int64_t rows, int64_t cols,
                            float2 *b, int64_t ldb, cudaStream_t stream, int64_t bTile = 0,
                            int64_t bTileStride = 0);
cudaError_t launchC64ToC128(float2 const *a, int64_t lda, int64_t rows, int64_t cols,
                            double2 *b, int64_t ldb, cudaStream_t stream);

// Apply: one stage of items, element type T2 (double2 or float2).
template <typename T2>
cudaError_t launchApplyStage(ApplyItem const *items, int64_t nItems,
                             ApplyContrib const *contribs, T2 const *arena,
                             T2 const *X, int64_t ldx, T2 *W, int64_t R,
                             cudaStream_t stream);

// W row-major with leading dimension R, or (wTile > 0) tile-major: panel t
// of wTile columns at W + t wTileStride, leading dimension wTile
template <typename T2>
cudaError_t launchApplyReduce(int32_t const *rowSeg, int64_t const *segStart,
                              int64_t const *segContrib0, int64_t const *segBase,
                              T2 const *W, int64_t R, T2 *Y, int64_t ldy,
                              int64_t nRows, int64_t const *outPerm,
                              cudaStream_t stream, int64_t wTile = 0, int64_t wTileStride = 0);

// Split-BF16 tensor-core apply (terms = 2 or 3 bf16 planes).
// sets the kernels' shared-memory limit; returns resident CTAs per SM
cudaError_t tcPrepare(int32_t terms, int32_t *ctasPerSm);
cudaError_t launchTcFill(int32_t terms, TcFill const *fills, int64_t nFills,
                         double2 const *arena64, uint8_t *tarena, cudaStream_t stream);
// one stage: `ctas` chunk streams times ceil(R / rt) RHS tiles of rt = 16
// or 32 right-hand sides, one persistent CTA each, the tiles of a stream
// adjacent in the grid; stream c runs chunks [ctaChunk0[c], ctaChunk0[c+1]);
// status bit 4 = a bounded wait expired.
// the default tile: 16 RHS for R <= 16, else 32
int32_t tcRhsTile(int64_t R);
// every mbarrier wait of the kernel gives up after waitLimitNs (then the CTA
// drains what it has in flight, frees its tensor memory and sets status bit 4)
constexpr uint64_t kTcWaitLimitNs = 1000000000ull;
// X (inputs) and W (intermediates and outputs) are each row-major (ld >= R,
// tile stride rt) or, with more than one tile, tile-major: one panel of rt
// columns per tile (ld = rt, tile stride >= rows x rt), which lets every
// full tile's rows arrive by one bulk copy per chunk.
cudaError_t launchApplyTc(int32_t terms, int32_t rt, TcChunk const *chunks,
                          int64_t const *ctaChunk0, int32_t ctas, uint8_t const *tarena,
                          float2 const *X, int64_t ldx, int64_t xTs, float2 *W, int64_t ldw,
                          int64_t wTs, int64_t R, int32_t *status, cudaStream_t stream,
                          uint64_t waitLimitNs = kTcWaitLimitNs);
enum : int32_t { kStatusTcTimeout = 4 };

// X_tree[i] = X[perm[i]] (row gather, R columns; no perm: X[i]) into out row-major
// (leading dimension R) or (outTile > 0) tile-major: panel t of outTile
// columns at out + t outTileStride, leading dimension outTile
template <typename T2>
cudaError_t launchGatherRows(T2 const *X, int64_t ldx, int64_t const *perm,
                             int64_t nRows, int64_t R, T2 *out, cudaStream_t stream,
                             int64_t outTile = 0, int64_t outTileStride = 0);

}  // namespace bfg
