/* bfg -- GB300-native butterfly factorization of the 2-D Helmholtz kernel.
 *
 * C ABI of libbfg.so.  Plain pointers and sizes only.  Every entry point
 * returns a bfgStatus; the message of the last failure on a context is
 * available from bfgGetErrorString.  Nothing here aborts the process and
 * no kernel traps: failures come back as status codes.
 *
 * Complex numbers are interleaved (re, im) pairs: complex128 = two doubles,
 * complex64 = two floats.  Matrices are row-major with a leading dimension
 * in elements, as the reference's BfMatDenseComplex (rowStride = numCols,
 * mat_dense_complex.c:2069-2087).
 *
 * Each declaration names the reference interface it replaces.
 */
#ifndef BFG_H
#define BFG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  0..8 carry the reference's BfError numbering
 * (error.h:3-16) so an adapter can forward them unchanged. */
typedef enum bfgStatus {
  BFG_OK = 0,                       /* BF_ERROR_NONE */
  BFG_ERROR_INVALID_ARGUMENTS = 1,  /* BF_ERROR_INVALID_ARGUMENTS */
  BFG_ERROR_RUNTIME = 2,            /* BF_ERROR_RUNTIME_ERROR */
  BFG_ERROR_NOT_IMPLEMENTED = 3,    /* BF_ERROR_NOT_IMPLEMENTED */
  BFG_ERROR_MEMORY = 4,             /* BF_ERROR_MEMORY_ERROR */
  BFG_ERROR_OUT_OF_RANGE = 5,       /* BF_ERROR_OUT_OF_RANGE */
  BFG_ERROR_INCOMPATIBLE_SHAPES = 8,/* BF_ERROR_INCOMPATIBLE_SHAPES */
  BFG_ERROR_CUDA = 32,              /* a CUDA runtime call failed */
  BFG_ERROR_TIMEOUT = 33,           /* a bounded device wait ran out */
  BFG_ERROR_NUMERICAL = 34          /* e.g. an SVD that did not converge */
} bfgStatus;

/* Layer potentials, numbered as BfLayerPotential (layer_pot.h:52-65). */
typedef enum bfgLayerPotential {
  BFG_LAYER_POTENTIAL_SINGLE = 1,
  BFG_LAYER_POTENTIAL_PV_DOUBLE = 2,
  BFG_LAYER_POTENTIAL_PV_NORMAL_DERIV_SINGLE = 3,
  BFG_LAYER_POTENTIAL_COMBINED_FIELD = 5
} bfgLayerPotential;

/* Arithmetic of an apply. */
typedef enum bfgPrecision {
  BFG_PRECISION_FP64 = 0,   /* complex128 factors and vectors */
  BFG_PRECISION_FP32 = 1,   /* complex64 factors and vectors, FP32 accumulate */
  /* Tensor-core products with complex64 vectors: factors and right-hand sides
   * split into bf16 planes (hi + lo, or hi + lo + lo2), FP32 accumulate.
   * BF16X2 stores 8 bytes per complex entry and keeps ~16 significant bits;
   * BF16X3 stores 12 bytes and keeps ~24 bits (FP32-like).  The reference
   * computes in complex128 only; these are GB300 additions. */
  BFG_PRECISION_BF16X2 = 2,
  BFG_PRECISION_BF16X3 = 3,
  /* complex128 vectors in and out, factors and intermediates as pairs of
   * FP32 numbers (hi + lo, ~48 significant bits, 16 bytes per complex
   * entry) with error-free FP32 products: within ~1e-13 of FP64 at FP32
   * rates.  A GB300 addition (its FP64 units run at 1/64 of FP32). */
  BFG_PRECISION_DF64 = 4
} bfgPrecision;

typedef struct bfgContext_s *bfgContext;
typedef struct bfgFac_s *bfgFac;

/* BfHelm2 (helm2.h:10-15) with its complex scalars split into parts. */
typedef struct bfgHelm2 {
  double k;
  int32_t layerPot;           /* bfgLayerPotential */
  int32_t reserved;
  double alphaRe, alphaIm;    /* combined field: alpha S + beta D */
  double betaRe, betaIm;
} bfgHelm2;

/* Knobs of the factorization.  bfgFacOptionsDefault gives the reference's
 * behaviour exactly. */
typedef struct bfgFacOptions {
  int64_t leafSize;   /* split nodes with more points (reference: 1,
                         quadtree_node.c:17) */
  double rankEps;     /* eps in the rank estimate p = ceil(k r1 r2 / d -
                         log10 eps) (reference: 1e-15, fac_helm2.c:102,
                         291-296, 523; helm2.c:14-36) */
  int32_t pinvCut;    /* 0: keep sigma >= max(m,n) eps sigma0 + eps
                         (mat_dense_complex.c:1797-1808); 1: keep
                         sigma >= pinvTol * sigma0 (linalg.c:26-36) */
  int32_t treeOnGpu;  /* 1: build the quadtrees on the GPU (the same trees
                         as the host build, which is the default, 0) */
  double pinvTol;
  int32_t jacobiArith; /* arithmetic of the re-expansion SVDs' Jacobi sweeps:
                          0 FP64 (default), 1 double-float (FP32 pairs,
                          ~48 bits; several times faster on GB300, whose FP64
                          units run at 1/64 of FP32).  Double-float carries
                          rounding noise at ~1e-14 of the largest singular
                          value, so it requires pinvCut = 1 with
                          pinvTol >= 1e-10 */
  int32_t sketch;     /* 1 (default): a FIRST/MIDDLE block of rank estimate
                         p >= 128 whose Z_equiv has a numerical rank well
                         below p (about k r1 r2 / R against the estimate's
                         k r1 r2 / (R - r1 - r2)) takes the randomized range
                         finder instead of the p x p Jacobi SVD, when
                         pinvCut = 1 and pinvTol >= 1e-10: the same cut on
                         the same singular values, to within Z_equiv's
                         rounding floor (~1e-14 sigma0), at a fraction of the
                         work.  A block too large for the shared-memory
                         working set of the full path takes it whatever the
                         cut.  0: the full path only (such blocks are then
                         refused with BFG_ERROR_NOT_IMPLEMENTED).  No
                         counterpart in the reference. */
} bfgFacOptions;

typedef struct bfgFacStats {
  int64_t numRows, numCols;
  int64_t numBlocks, numFirst, numMiddle, numLast, numDense;
  int64_t numProducts;
  int64_t arenaEntries;       /* complex entries over all stored blocks */
  int64_t numStages;          /* apply launches before the final sum */
  int64_t numItems;           /* apply work items over all stages */
  int64_t maxRank;
  int64_t jacobiNotConverged; /* 1 if any block's Jacobi SVD hit the sweep cap */
  double factorMs;            /* device time of the factorization kernels */
  double flopsPerRhs;         /* 8 * sum over blocks of m*n */
  double fillMs;              /* evaluation and dense blocks */
  double reexpSmemMs;         /* re-expansions held in shared memory */
  double reexpGlobalMs;       /* re-expansions held in global memory */
  int64_t numSketched;        /* re-expansions by the randomized path */
  int64_t sketchRetries;      /* sketches redone wider (rank not captured) */
  int64_t sketchFallbacks;    /* blocks handed back to the full path */
  int64_t sketchMaxWidth;     /* widest accepted sketch */
  double sketchMs;            /* device time of the randomized path */
  double sketchMeanWidth;     /* mean accepted sketch width */
  int64_t applyBufferBytes;   /* device bytes the allocating applies have
                                 allocated so far (workspace and gather
                                 buffers; bfgFacApplyNoAlloc adds none) */
  double sketchPhaseMs[8];    /* randomized path by phase: fills, Z Omega,
                                 qr(Y), Z^H Q, qr(G), Jacobi, weights and
                                 capture test, output products */
  int64_t reexpSvds;          /* SVDs of the full path: its blocks with the
                                 same Z_equiv share one */
  int64_t sketchGroups;       /* SVDs of the randomized path, shared the same
                                 way */
} bfgFacStats;

/* Contexts: one CUDA device and one stream; calls on a context are
 * serialised by the caller. */
bfgStatus bfgContextCreate(int32_t device, bfgContext *ctx);
bfgStatus bfgContextDestroy(bfgContext ctx);
/* Launch on the caller's cudaStream_t (passed as void*; NULL is CUDA's
 * legacy default stream).  A context starts on a non-blocking stream of its
 * own; bfgContextGetStream returns the stream in use. */
bfgStatus bfgContextSetStream(bfgContext ctx, void *cudaStream);
bfgStatus bfgContextGetStream(bfgContext ctx, void **cudaStream);
/* Waits for all work the context has launched. */
bfgStatus bfgContextSynchronize(bfgContext ctx);
char const *bfgGetErrorString(bfgContext ctx);

void bfgFacOptionsDefault(bfgFacOptions *opts);

/* Replaces bfQuadtreeInit for both point sets (quadtree.c:80-98) followed by
 * bfFacHelm2MakeMultilevel (fac_helm2.h:18, fac_helm2.c:943-1002).
 * Points are host arrays of (x, y) pairs in original order; normals may be
 * NULL.  The factorization runs on the GPU and stays resident there. */
bfgStatus bfgFacHelm2MakeMultilevel(bfgContext ctx, bfgHelm2 const *helm,
                                    double const *srcXy, double const *srcNormals,
                                    int64_t numSrc, double const *tgtXy,
                                    double const *tgtNormals, int64_t numTgt,
                                    bfgFacOptions const *opts, bfgFac *fac);
/* Many independent problems of uneven size in one factorization: problem p
 * has sources srcXy[2*srcOffsets[p] .. 2*srcOffsets[p+1]) (normals alike),
 * targets alike, wavenumber k[p], and helm's layer potential and alpha/beta.
 * Every kernel launch covers the blocks of all problems.  The result is the
 * block-diagonal operator diag(A_0, ..., A_{P-1}): its rows and columns are
 * the problems' tree orders back to back (bfgFacGetPerms maps them into the
 * concatenated point arrays), so one apply serves every problem.  No
 * counterpart call in the reference; each A_p equals
 * bfFacHelm2MakeMultilevel of problem p (fac_helm2.c:943-1002). */
bfgStatus bfgFacHelm2MakeBatched(bfgContext ctx, bfgHelm2 const *helm, double const *k,
                                 int64_t numProblems, double const *srcXy,
                                 double const *srcNormals, int64_t const *srcOffsets,
                                 double const *tgtXy, double const *tgtNormals,
                                 int64_t const *tgtOffsets, bfgFacOptions const *opts,
                                 bfgFac *fac);
/* Writes the factorization to `path`: its inputs (points, normals,
 * wavenumbers, options, problem offsets) and its FP64 factors.  The
 * reference's dumps (bfMatDump, mat.c:67-73; bf_one_block.c:166-258) store
 * block values without what rebuilds the operator, so there is no
 * counterpart; this caches factorizations that take minutes to build.
 * Synchronises the context's stream.  Little-endian; files move between the
 * x86-64 and aarch64 builds. */
bfgStatus bfgFacSave(bfgFac fac, char const *path);
/* Rebuilds a factorization saved by bfgFacSave on ctx's device without
 * factorizing again: the plan (trees, ranks, block order) is rebuilt on the
 * host from the stored inputs -- it is a deterministic function of them --
 * and must account for exactly the stored number of factor entries; the
 * factors are then uploaded.  BFG_ERROR_INVALID_ARGUMENTS for a file of
 * another format or version or with inconsistent contents,
 * BFG_ERROR_RUNTIME for I/O failures. */
bfgStatus bfgFacLoad(bfgContext ctx, char const *path, bfgFac *fac);
/* bfMatDelete on the factorization (mat.h:57). */
bfgStatus bfgFacDestroy(bfgFac fac);
/* bfMatGetNumRows / bfMatGetNumCols (mat.c). */
bfgStatus bfgFacGetShape(bfgFac fac, int64_t *numRows, int64_t *numCols);
/* BfTree.perm of both quadtrees: tree position -> original index. */
bfgStatus bfgFacGetPerms(bfgFac fac, int64_t *srcPerm, int64_t *tgtPerm);
/* bfMatNumBytes (mat.h:56): bytes of the stored complex128 blocks. */
bfgStatus bfgFacNumBytes(bfgFac fac, int64_t *numBytes);
bfgStatus bfgFacGetStats(bfgFac fac, bfgFacStats *stats);
/* The block structure in the grammar of the oracle's plan dump. */
bfgStatus bfgFacDescribe(bfgFac fac, char *buf, int64_t capacity, int64_t *length);
/* Host copy of every stored block, plan order, each column-major m x n
 * complex128; `table` receives (kind, m, n, arena offset) per block. */
bfgStatus bfgFacCopyBlocks(bfgFac fac, double *entries, int64_t capacityEntries,
                           int64_t *table, int64_t capacityBlocks);

/* Flags of the applies. */
#define BFG_APPLY_ORIGINAL_ORDER 1u  /* X and Y rows in original point order */

/* Builds the precision's copy of the factors now, as the first apply in that
 * precision would (allocates and synchronises). */
bfgStatus bfgFacPrepare(bfgFac fac, bfgPrecision precision);
/* Test hook (no counterpart in the reference): the time after which every
 * bounded wait of the tensor-core apply (BFG_PRECISION_BF16X2/X3) gives up,
 * 1 s by default.  A wait that gives up makes each CTA drain its copies and
 * tensor-core products in flight, free its tensor memory and end; the apply
 * then returns BFG_ERROR_TIMEOUT and the factorization stays usable.  0
 * makes every wait that is not already satisfied give up at once, which is
 * how the tests drive that path. */
bfgStatus bfgFacSetTcWaitLimit(bfgFac fac, uint64_t waitLimitNs);

/* Autotuner of the tensor-core apply (BF16X2, BF16X3) for numRhs
 * right-hand sides.  It tries both RHS tile widths (16 and 32 right-hand
 * sides per CTA) and, for each, deals every stage's chunks to the
 * persistent CTAs under several cost models; it times every stage of every
 * candidate on the GPU (best of 5).  Per width it takes each stage's
 * fastest dealing, and it keeps the width whose stages sum to less (the
 * default width and model are candidates, so the apply gets no slower).
 * Later applies of numRhs right-hand sides use the choice.
 * stageMs[2 s], stageMs[2 s + 1]: stage s with the default width and
 * schedule, and with the chosen ones (up to `capacity` values);
 * *numStages the number of stages.  Within one tile width the results do
 * not change, only which CTA runs which chunk; the two widths sum the
 * plane products in different groupings, so a change of width changes
 * results by rounding. */
bfgStatus bfgFacAutotune(bfgFac fac, bfgPrecision precision, int64_t numRhs, double *stageMs,
                         int32_t capacity, int32_t *numStages);

/* The RHS tile width (16 or 32) the tensor-core apply of numRhs right-hand
 * sides uses in this precision: bfgFacAutotune's choice for that count,
 * else the default (16 up to 16 right-hand sides, else 32). */
bfgStatus bfgFacGetRhsTile(bfgFac fac, bfgPrecision precision, int64_t numRhs,
                           int32_t *rhsTile);

/* Waits for the context's stream and reports what the tensor-core applies
 * enqueued since the last check left in their status word:
 * BFG_ERROR_TIMEOUT when a bounded device wait ran out (the factorization
 * stays usable).  The synchronising calls (bfgFacApplyHost,
 * bfgFacApplyTimed, bfgFacAutotune) check it themselves; after
 * asynchronous bfgFacApply calls, this is the check.  No counterpart in the
 * reference (whose applies are synchronous host code). */
bfgStatus bfgFacSynchronize(bfgFac fac);

/* Y = A X -- bfMatMul (mat.c:183-185) with A the factorization.  X (numCols
 * x numRhs) and Y (numRows x numRhs) are DEVICE pointers: complex128 for
 * FP64, complex64 for FP32, BF16X2 and BF16X3.  The first apply in a
 * precision other than FP64 builds that precision's copy of the factors
 * (allocates and synchronises once).  Rows are in tree order unless
 * BFG_APPLY_ORIGINAL_ORDER is set.  Runs on the context's stream; returns
 * without synchronising.  Every apply of one factorization uses its one
 * workspace: applies issued on different streams must be ordered by the
 * caller (events), as must the writes of X and reads of Y on other streams. */
bfgStatus bfgFacApply(bfgFac fac, bfgPrecision precision, void const *X, int64_t ldx,
                      int64_t numRhs, void *Y, int64_t ldy, uint32_t flags);

/* The same product with HOST complex128 X and Y (the reference's contract
 * for bfMatMul on BfMatDenseComplex operands); copies both ways and
 * synchronises.  The precision selects the device arithmetic. */
bfgStatus bfgFacApplyHost(bfgFac fac, bfgPrecision precision, double const *X,
                          int64_t ldx, int64_t numRhs, double *Y, int64_t ldy,
                          uint32_t flags);
/* The same, enqueued: returns at once, the copies run on streams of their
 * own so that one call's upload and download overlap another call's
 * compute (two calls in flight per factorization; a third waits on the
 * device for the first).  X must stay unchanged and Y unread until
 * bfgFacApplyHostWait returns; X and Y should be pinned host memory
 * (pageable memory makes the copies synchronous). */
bfgStatus bfgFacApplyHostAsync(bfgFac fac, bfgPrecision precision, double const *X,
                               int64_t ldx, int64_t numRhs, double *Y, int64_t ldy,
                               uint32_t flags);
/* Waits for every enqueued host-operand apply of the factorization. */
bfgStatus bfgFacApplyHostWait(bfgFac fac);

/* No counterpart in the reference.  The FP64 product of bfgFacApply (device
 * complex128 X and Y, same flags and contract) for callers that cannot
 * allocate GPU memory -- their device memory is reserved up front by another
 * allocator, or cudaMalloc's possible device synchronisation is not
 * acceptable on their path.  The workspace is a static 32 MiB device array
 * inside the library (held by every GPU that loads it); calls whose
 * workspace would exceed it fail with BFG_ERROR_OUT_OF_RANGE.  The first
 * call on a device looks up the array's address and should come before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * race. */
bfgStatus bfgFacApplyNoAlloc(bfgFac fac, void const *X, int64_t ldx, int64_t numRhs,
                             void *Y, int64_t ldy, uint32_t flags);

/* bfgFacApply with a CUDA event around every launch; launchMs[i] receives
 * the device time of launch i (stages in order, then the final sum).
 * Synchronises. */
bfgStatus bfgFacApplyTimed(bfgFac fac, bfgPrecision precision, void const *X,
                           int64_t ldx, int64_t numRhs, void *Y, int64_t ldy,
                           uint32_t flags, float *launchMs, int32_t capacity,
                           int32_t *numLaunches);

/* Algorithmic work of each launch of a device-operand apply (bfgFacApply)
 * in this precision with numRhs right-hand sides and these flags, in the
 * order of bfgFacApplyTimed: info[3i..3i+2] = stored complex entries read,
 * vector rows read, vector rows written (per right-hand side).  The
 * launches: the input's gather (original order) or, for a tensor-core
 * apply of more than one RHS tile, its tile-major copy; the stages; the
 * final sum. */
bfgStatus bfgFacGetApplyLaunches(bfgFac fac, bfgPrecision precision, int64_t numRhs,
                                 uint32_t flags, int64_t *info, int32_t capacity,
                                 int32_t *numLaunches);

/* bfgFacGetApplyLaunches for the applies whose launches do not depend on
 * the precision or the right-hand-side count: FP64, FP32, DF64, and the
 * tensor-core applies of one RHS tile. */
bfgStatus bfgFacGetLaunchInfo(bfgFac fac, uint32_t flags, int64_t *info,
                              int32_t capacity, int32_t *numLaunches);

/* Rows `rows` (tree order) of the dense FP64 product K X, evaluated on the
 * GPU kernel by kernel -- bfHelm2GetKernelMatrix (helm2.c:282-319) times X
 * without forming K.  X: device complex128, tree order; out: device
 * complex128 (numRowsSel x numRhs, leading dimension ldo). */
bfgStatus bfgFacDenseRows(bfgFac fac, int64_t const *rows, int64_t numRowsSel,
                          void const *X, int64_t ldx, int64_t numRhs, void *out,
                          int64_t ldo);

/* bfHelm2GetKernelMatrix (helm2.c:282-319): host arrays in and out,
 * out = row-major m x n complex128, rows = targets. */
bfgStatus bfgHelm2KernelMatrix(bfgContext ctx, bfgHelm2 const *helm,
                               double const *srcXy, double const *srcNormals,
                               int64_t numSrc, double const *tgtXy,
                               double const *tgtNormals, int64_t numTgt,
                               double *out);

/* bf_H0 / bf_H1 (bessel.c:294-308) evaluated on the GPU:
 * out[4i..4i+3] = J0, Y0, J1, Y1 at x[i] > 0 (host arrays). */
bfgStatus bfgBessel01(bfgContext ctx, double const *x, int64_t n, double *out);

/* The device's FP64 fused multiply-add rate in TFLOP/s (2 flops per FMA),
 * measured with CUDA events on a kernel of independent FMA chains over all
 * SMs (~100 ms): the FP64 roof of the FP64 apply and the factorization.  No
 * counterpart in the reference. */
bfgStatus bfgMeasureFp64Rate(bfgContext ctx, double *tflops);

/* ---------------------------------------------------------------------
 * Boundary-integral systems and GMRES
 * --------------------------------------------------------------------- */
typedef struct bfgSystem_s *bfgSystem;

/* A = diagShift I + (K + C) diag(w): the operator assembleButterfliedK
 * builds (multiple_scattering_context.c:457-507; diagShift = 1/2 there).
 * K is `fac`, built on the same points (original order) and layer
 * potential as given here; C the Kapur-Rokhlin correction of order krOrder
 * (2, 6, 10; 0 = none) inside each closed curve [curveOffsets[b],
 * curveOffsets[b+1]) (bfQuadKrApplyBlockCorrectionTree, quadrature.c:222-269)
 * with the reference's kernel callback (multiple_scattering_context.c:
 * 27-42); w the quadrature weights.  `ctx` is the context of `fac`.
 * Vectors of the system are in original point order. */
bfgStatus bfgSystemCreate(bfgContext ctx, bfgFac fac, bfgHelm2 const *helm,
                          double const *xy, double const *normals,
                          double const *weights, int64_t const *curveOffsets,
                          int64_t numCurves, int32_t krOrder, double diagShift,
                          bfgSystem *sys);
bfgStatus bfgSystemDestroy(bfgSystem sys);
char const *bfgSystemGetErrorString(bfgSystem sys);
/* Y = A X for one device complex128 vector (bfMatMul on the assembled
 * operator). */
bfgStatus bfgSystemApply(bfgSystem sys, void const *X, void *Y);
/* Arithmetic of the butterfly part of bfgSystemApply, and so of the GMRES
 * iterations: BFG_PRECISION_FP64 (the default) or BFG_PRECISION_DF64.
 * bfgSolveGmres computes its final true residual in FP64 either way. */
bfgStatus bfgSystemSetApplyPrecision(bfgSystem sys, bfgPrecision precision);
/* Block-Jacobi preconditioner: dense diagonal block of A per curve, inverted
 * on the GPU (assemblePreconditioner, multiple_scattering_context.c:545-634;
 * the reference factors them with zgetrf, lu_dense_complex.c:185-232). */
bfgStatus bfgSystemBuildBlockJacobi(bfgSystem sys);
bfgStatus bfgSystemApplyBlockJacobi(bfgSystem sys, void const *R, void *Z);

#define BFG_PRECOND_NONE 0
#define BFG_PRECOND_BLOCK_JACOBI 1
#define BFG_PRECOND_USER 2
#define BFG_PRECOND_LEARNED 3
#define BFG_PRECOND_TWO_LEVEL 4

/* ---- Two-level preconditioner (a GB300 addition; the reference
 * preconditions with block-Jacobi only) ----
 * A coarse space of every curve's discrete Fourier modes: with the points
 * j = 0 .. n_b - 1 of curve b equispaced in its parameter (as the
 * reference's circles are, ellipse.c), Phi_b[j, m] = e^{i mu 2 pi j / n_b} /
 * sqrt(n_b) for mu = -q_b .. q_b, q_b = min(ceil(k L_b / 2 pi) + extraModes,
 * (n_b - 1) / 2) with L_b the sum of the curve's quadrature weights (its
 * length: the modes that radiate, plus extraModes).  Builds A_c = Phi^H A
 * Phi from one apply of the system to all coarse basis vectors (butterfly
 * part in split-BF16 on the tensor cores) and inverts it by block
 * Gauss-Jordan elimination over the curves' mode blocks (pivoting inside a
 * block), in FP32; at most 128 modes per curve.  With
 * BFG_PRECOND_TWO_LEVEL, bfgSolveGmres applies the multiplicative
 * two-level preconditioner z1 = Phi A_c^-1 Phi^H r, z = z1 + M_bj (r - A z1)
 * (block-Jacobi built; the system apply in the iterations' precision).
 * *dim: the coarse dimension (may be NULL). */
bfgStatus bfgSystemBuildCoarse(bfgSystem sys, int32_t extraModes, int64_t *dim);
/* A_c and A_c^-1 (device complex64, dim x dim row-major; either may be
 * NULL). */
bfgStatus bfgSystemCoarseMatrices(bfgSystem sys, void *Ac, void *AcInv);
/* z = Phi A_c^-1 Phi^H r (device complex128 vectors). */
bfgStatus bfgSystemApplyCoarse(bfgSystem sys, void const *R, void *Z);

/* ---- Learned preconditioner (a GB300 addition; the reference
 * preconditions with block-Jacobi only) ---- */
typedef struct bfgMlp_s *bfgMlp;
/* A perceptron nIn -> nHidden -> nHidden -> nOut with ReLU between the
 * layers, FP32 parameters on the context's GPU, He-uniform weights from
 * `seed` (the output layer scaled by 0.1) and zero biases.  Forward,
 * gradients and Adam run in hand-written kernels, in a fixed order (the
 * same batch gives the same gradients bit for bit). */
bfgStatus bfgMlpCreate(bfgContext ctx, int32_t nIn, int32_t nHidden, int32_t nOut,
                       uint64_t seed, bfgMlp *mlp);
bfgStatus bfgMlpDestroy(bfgMlp mlp);
bfgStatus bfgMlpGetShape(bfgMlp mlp, int32_t *nIn, int32_t *nHidden, int32_t *nOut);
/* The parameters as one FP32 array: W1 (nIn x nHidden, row-major), b1, W2
 * (nHidden x nHidden), b2, W3 (nHidden x nOut), b3.  Get/Set copy to/from
 * the host; Set also resets the optimiser. */
bfgStatus bfgMlpNumParams(bfgMlp mlp, int64_t *count);
bfgStatus bfgMlpGetParams(bfgMlp mlp, float *params);
bfgStatus bfgMlpSetParams(bfgMlp mlp, float const *params);
/* Y (batch x nOut) = network(X (batch x nIn)); device FP32, row-major. */
bfgStatus bfgMlpForward(bfgMlp mlp, void const *X, int64_t batch, void *Y);
/* The loss mean_b 0.5 ||y_b - t_b||^2 of one batch (device X, T) and its
 * gradient (host, parameter layout; may be NULL); no update. */
bfgStatus bfgMlpGradients(bfgMlp mlp, void const *X, void const *T, int64_t batch,
                          float *grad, double *loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8, learning rate lr) on one
 * batch; *loss = the loss before the step. */
bfgStatus bfgMlpTrainStep(bfgMlp mlp, void const *X, void const *T, int64_t batch, float lr,
                          double *loss);

/* BFG_PRECOND_LEARNED: z = M_bj r + s_c p_c mlp(features_c) on every chunk
 * c of `chunk` consecutive points of a curve, with M_bj the block-Jacobi
 * preconditioner (FP32 copy), s_c = ||r_c||, p_c the phase of sum_t |r_t|
 * r_t over the chunk and features_c = conj(p_c) (r_c, (M_bj r)_c) / s_c as
 * interleaved (re, im) pairs, zero-padded to `chunk` points (nIn = 4 chunk,
 * nOut = 2 chunk): the preconditioner commutes with complex scalings of r.
 * The network runs on the system's stream.  Requires the block-Jacobi inverses; `mlp`
 * must live as long as it is used. */
bfgStatus bfgSystemSetLearnedPreconditioner(bfgSystem sys, bfgMlp mlp, int32_t chunk);
bfgStatus bfgSystemLearnedNumChunks(bfgSystem sys, int64_t *numChunks);
/* Training pairs: for a residual R and its exact correction E = A^-1 R
 * (device complex128; E may be NULL), the chunk features (numChunks x 4
 * chunk) and targets conj(p_c) (E - M_bj R)_c / s_c (numChunks x 2 chunk),
 * device FP32. */
bfgStatus bfgSystemLearnedPairs(bfgSystem sys, void const *R, void const *E, void *features,
                                void *targets);
/* A right preconditioner z = M r on device complex128 vectors, launched on
 * `cudaStream`; may change from call to call (flexible GMRES). */
typedef bfgStatus (*bfgPrecondFn)(void *userData, void const *r, void *z, void *cudaStream);

typedef struct bfgGmresResult {
  int64_t iterations;
  double relResidual;       /* |g_{j+1}| / ||b|| from the Arnoldi process */
  double trueRelResidual;   /* ||b - A x|| / ||b|| recomputed at the end */
  double seconds;           /* wall time of the solve */
  int32_t converged;
  int32_t reserved;
} bfgGmresResult;

/* Solves A x = b with right-preconditioned flexible GMRES (no restart, at
 * most maxIter iterations), X holding x0 on entry and x on exit (device
 * complex128).  Arnoldi in FP64: classical Gram-Schmidt with a second pass
 * where the DGKS criterion asks for one; BFG_PRECOND_BLOCK_JACOBI applies
 * an FP32 copy of the block inverses (a flexible solver's preconditioner
 * needs no more).  Replaces bfSolveGMRES (linalg.c:47-317), which is
 * left-preconditioned: here the convergence test |g_{j+1}|/||b|| < tol is
 * on the true residual. */
bfgStatus bfgSolveGmres(bfgSystem sys, void const *B, void *X, double tol,
                        int64_t maxIter, int32_t precond, bfgPrecondFn userFn,
                        void *userData, bfgGmresResult *result);

/* Host-only (no GPU needed): the quadtrees and block structure that
 * bfgFacHelm2MakeMultilevel builds for the same inputs -- the permutations
 * and the plan text of bfgFacDescribe.  Either output may be NULL. */
bfgStatus bfgPlanHelm2(double k, double const *srcXy, int64_t numSrc,
                       double const *tgtXy, int64_t numTgt,
                       bfgFacOptions const *opts, int64_t *srcPerm,
                       int64_t *tgtPerm, char *buf, int64_t capacity,
                       int64_t *length);

/* Host-only self-check of the apply's work decomposition (no GPU; no
 * counterpart in the reference).  Plans these inputs as
 * bfgFacHelm2MakeMultilevel (numProblems = 1) or bfgFacHelm2MakeBatched
 * would, gives every stored block seeded pseudo-random entries and
 * evaluates A X for numRhs (1..64) seeded right-hand sides three ways in
 * FP64 on the host: from the plan's block structure directly, by the staged
 * program the device kernels execute (items, workspace regions, final sum),
 * and by the tensor-core chunk schedules dealt to `ctas` persistent CTAs
 * under every cost model bfgFacAutotune tries.  relErr[0] receives the
 * relative Frobenius difference of the staged program from the direct
 * evaluation, relErr[1] the largest over the chunk schedules.  A schedule
 * that reads a workspace row no earlier stage wrote gives a non-finite
 * difference; one that writes a row twice in a stage, or whose chunks do
 * not form whole items, returns BFG_ERROR_RUNTIME.  Only a difference is
 * returned, never an operator value. */
bfgStatus bfgPlanCheckApply(double const *k, int64_t numProblems, double const *srcXy,
                            int64_t const *srcOffsets, double const *tgtXy,
                            int64_t const *tgtOffsets, bfgFacOptions const *opts,
                            int32_t numRhs, int32_t ctas, uint64_t seed, double *relErr);

/* A quadtree node (BfQuadtreeNode, quadtree_node.h:22-39): bounding box,
 * split point, the node's points as a range of the tree order, children in
 * quadrant order (quadtree_node.h:31-37). */
typedef struct bfgQuadtreeNode {
  double xmin, ymin, xmax, ymax;
  double splitX, splitY;
  int64_t i0, i1;             /* tree-order range of the node's points */
  int32_t parent, depth;      /* parent -1 at the root */
  int32_t child[4];           /* -1: no points in that quadrant */
} bfgQuadtreeNode;

/* bfQuadtreeInit (quadtree.c:80-98) of numSets point sets at once: set t is
 * xy[2*setOffsets[t] .. 2*setOffsets[t+1]) (host array, setOffsets[0] = 0),
 * split while a node holds more than leafSize points.  onGpu = 1 builds all
 * sets on the context's GPU in one breadth-first pass (ctx required), 0 on
 * the host (ctx may be NULL); both give the same trees, node for node.
 * perm (setOffsets[numSets] entries) receives each set's tree order as
 * indices into that set; nodeOffsets (numSets + 1 entries) the range of each
 * set's nodes in `nodes`, numbered as the reference's recursive build
 * creates them.  nodes may be NULL to count only; else it has room for
 * nodeCapacity entries (BFG_ERROR_OUT_OF_RANGE when that is too few). */
bfgStatus bfgQuadtreeBuild(bfgContext ctx, double const *xy, int64_t const *setOffsets,
                           int64_t numSets, int64_t leafSize, int32_t onGpu, int64_t *perm,
                           bfgQuadtreeNode *nodes, int64_t nodeCapacity, int64_t *nodeOffsets);

/* Host-only: the device H0/H1 evaluator's source compiled for the CPU,
 * out[4i..4i+3] = J0, Y0, J1, Y1. */
bfgStatus bfgBessel01Host(double const *x, int64_t n, double *out);

/* The reference's seeded generator (rand.c:19-76): splitmix64 seeding
 * xoshiro256+.  State is explicit instead of process-global. */
typedef struct bfgRng {
  uint64_t s[4];
} bfgRng;
void bfgRngSeed(bfgRng *rng, uint64_t seed);               /* bfSeed */
double bfgRngUniform1(bfgRng *rng);                        /* bfRealUniform1 */
void bfgRngUniform(bfgRng *rng, int64_t n, double *out);   /* bfRealUniform */
void bfgRngComplexRandn(bfgRng *rng, int64_t n, double *out); /* bfComplexRandn, 2n doubles */

#ifdef __cplusplus
}
#endif

#endif /* BFG_H */
