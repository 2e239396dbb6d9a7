// Host-side structure of a butterfly factorization: quadtrees, the planner
// that walks node pairs exactly like the reference's bfFacHelm2MakeMultilevel
// (fac_helm2.c:551-1002), and the flat descriptor tables the GPU kernels
// consume (block fill, batched re-expansion, staged apply).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace bfg {

struct Circle {
  double cx = 0, cy = 0, r = 0;
};

// Quadtree over a point set, built with the reference's split rule and sift
// order (quadtree_node.c:123-306).  `perm[i]` is the original index of the
// point at tree position i (BfTree.perm).
struct QNode {
  double xmin, ymin, xmax, ymax;  // bounding box
  double sx, sy;                  // split point (box centre)
  int child[4] = {-1, -1, -1, -1};
  int parent = -1;
  int depth = 0;
  int64_t i0 = 0, i1 = 0;         // tree-order range of the node's points
  bool leaf() const { return child[0] < 0 && child[1] < 0 && child[2] < 0 && child[3] < 0; }
  int64_t numPoints() const { return i1 - i0; }
};

class Quadtree {
 public:
  // leafSize generalises LEAF_SIZE_THRESHOLD = 1 (quadtree_node.c:17): a
  // node with more than leafSize points is split.
  void build(double const *xy, int64_t n, int64_t leafSize);
  // the root's box from the points' bounding box (bbox.c:18-30) and a
  // child's box and split point (quadtree_node.c:196-282): the arithmetic
  // both the host and the GPU build use
  static QNode rootNode(double xmin, double xmax, double ymin, double ymax);
  static QNode childNode(QNode const &parent, int q);
  Circle circle(int node) const;  // quadtree_node.c:321-330
  std::vector<int> children(int node) const;
  // LR level order below `node`, grouped by depth (tree_level_iter.c:12-88)
  std::vector<std::vector<int>> levelsBelow(int node) const;

  std::vector<QNode> nodes;
  std::vector<int64_t> perm;
  int64_t leafSize = 1;

 private:
  void split(int node, double const *px, double const *py);
};

// Quadtrees of the point sets xy[2 setOff[t] .. 2 setOff[t+1]) built on the
// GPU (bfg_tree.cu): the same permutation and node table as Quadtree::build
// of each set.  Synchronises the stream.
// stream: a cudaStream_t.
void buildQuadtreesGpu(double const *xy, int64_t const *setOff, int64_t numSets, int64_t leafSize,
                       void *stream, std::vector<Quadtree> &out);

enum BlockKind : int32_t { kFirst = 0, kMiddle = 1, kLast = 2, kDense = 3 };

// One stored block of the factorization.  Geometry for the fill:
//   first : sources = source-tree range [s0,s1); equivalent sources on `ceq`
//           (m points), check points on `cchk` (m points)
//   middle: sources = n points on `corig`; equivalent sources on `ceq`
//           (m points); check points on `cchk` (m points)
//   last  : sources = n points on `ceq`; targets = target-tree range [t0,t1)
//   dense : sources [s0,s1), targets [t0,t1)
struct Block {
  int32_t kind;
  int32_t m, n;
  int32_t ri, ci;               // block row / column within its factor
  int64_t s0 = 0, s1 = 0, t0 = 0, t1 = 0;
  Circle corig, ceq, cchk;
  int64_t arenaOff = 0;         // complex entries, column-major m x n
  double k = 0;                 // wavenumber of the block's problem
};

struct Factor {
  int32_t kind;                 // 0 = block diagonal, 1 = block COO
  int32_t nbr, nbc;
  std::vector<int64_t> rowOff, colOff;
  std::vector<int32_t> blocks;  // indices into Plan::blocks, stored order
};

struct Product {
  std::vector<int32_t> factors; // stored order: [evaluation, ..., first]
  int64_t t0, t1, s0, s1;
};

// A node of the hierarchical (HODBF) structure.
struct PNode {
  int32_t type;                 // 0 = block dense, 1 = product, 2 = dense
  int32_t nr = 0, nc = 0;
  std::vector<int64_t> rowOff, colOff;
  std::vector<int32_t> children;
  int32_t product = -1, block = -1;
};

struct PlanParams {
  double k = 1;
  int64_t leafSize = 1;
  double rankEps = 1e-15;       // eps of the rank estimate (helm2.c:14-36)
};

struct Plan {
  Quadtree src, tgt;
  std::vector<Block> blocks;
  std::vector<Factor> factors;
  std::vector<Product> products;
  std::vector<PNode> pnodes;
  int32_t root = -1;
  // one HODBF root per problem with the tree-order row / column offsets of
  // that problem (a single problem has one root at (0, 0))
  struct Root {
    int32_t pnode;
    int64_t rowBase, colBase;
  };
  std::vector<Root> roots;
  int64_t arenaEntries = 0;
  // block indices in plan order (the order of the plan text); the arena
  // stores the blocks back to back in this order
  std::vector<int32_t> blockOrder;

  std::string text() const;     // the plan grammar of the oracle driver
};

// Independent problems in one plan: problem p has sources
// srcXy[2*srcOff[p] .. 2*srcOff[p+1]) and targets likewise, wavenumber k[p];
// the merged plan's rows and columns are the problems' tree orders back to
// back, and its perms index the concatenated point arrays.
// trees: null, or the 2 numProblems quadtrees already built (source tree of
// problem p at 2p, target tree at 2p+1).
void makePlanBatched(Plan &plan, PlanParams const &params, double const *k,
                     double const *srcXy, int64_t const *srcOff, double const *tgtXy,
                     int64_t const *tgtOff, int64_t numProblems,
                     std::vector<Quadtree> const *trees = nullptr);

// Builds trees (unless given) and the plan; throws std::runtime_error on
// geometry the reference cannot factor.
void makePlan(Plan &plan, PlanParams const &params, double const *srcXy,
              int64_t nSrc, double const *tgtXy, int64_t nTgt,
              Quadtree const *srcTree = nullptr, Quadtree const *tgtTree = nullptr);

// ---------------------------------------------------------------------------
// GPU descriptor tables
// ---------------------------------------------------------------------------

// One work item of an apply stage: up to kItemRows consecutive output rows of
// one block row, accumulating over the blocks in that row.
constexpr int kItemRows = 32;
// products whose last factors share one output region (and one item per
// row range) in an apply program
constexpr int kFinGroup = 8;

struct ApplyItem {
  int64_t outRow;               // first output row in the workspace
  int32_t rows;                 // <= kItemRows
  int32_t nContrib;
  int64_t contrib0;             // first contribution
};

struct ApplyContrib {
  int64_t aOff;                 // arena offset of (first item row, column 0)
  int64_t inRow;                // first input row
  int32_t lda;                  // column stride of the block (its m)
  int32_t n;                    // columns
  int32_t inIsX;                // 1: input rows are in X, 0: in the workspace
  int32_t pad;
};

struct ApplyProgram {
  std::vector<int64_t> stageItem0;        // item range per stage (+1)
  std::vector<ApplyItem> items;
  std::vector<ApplyContrib> contribs;
  int64_t wsRows = 0;                     // workspace rows
  // final reduction: target row i sums segBase[c] + (i - segStart[s]) over
  // contributions c of its segment s
  std::vector<int32_t> rowSeg;            // per tree-order target row
  std::vector<int64_t> segStart;          // first row of each segment
  std::vector<int64_t> segContrib0;       // contribution range (+1)
  std::vector<int64_t> segBase;           // workspace row of segment start
  int64_t numRows = 0, numCols = 0;
  double flopsPerRhs = 0;                 // 8 * sum m*n
  // algorithmic traffic per stage: stored entries read, vector rows read
  // and written (one RHS); the final sum reads sumRows and writes numRows
  std::vector<int64_t> stageEntries, stageRowsIn, stageRowsOut;
  int64_t sumRows = 0;
};

// itemRows: rows per work item (32 for the CUDA-core kernels, 128 for the
// tensor-core kernel, whose MMA tile is 128 rows high)
void makeApplyProgram(Plan const &plan, ApplyProgram &prog, int itemRows = kItemRows);

// ---------------------------------------------------------------------------
// Tensor-core (split-BF16) apply: chunks of an item's contributions, each
// stored as a pre-tiled bf16 A tile in the tensor arena.
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;          // MMA M: rows per item
constexpr int kTcChunkCols = 32;      // most complex columns per chunk (4 MMA k-steps)
// k-groups (4 complex columns) per chunk for an item of mg row groups: an A
// plane holds at most 64 cores (8 KB) and the B planes of a 32-RHS tile at
// most 8 k-groups; the count is even (whole k-steps)
inline int32_t tcMaxKGroups(int32_t mg) {
  int32_t k = 64 / (mg < 1 ? 1 : mg);
  if (k > kTcChunkCols / 4) k = kTcChunkCols / 4;
  return k & ~1;
}

// One chunk of the chunk stream of a persistent CTA.  The A tile of a chunk
// holds `terms` bf16 planes back to back, each kg x mg core matrices of
// 8 rows x 16 bytes, k-group-major: core (g, h) at (g * mg + h) * 128 bytes.
struct TcChunk {
  int64_t tileOff;              // bytes: plane 0 of the A tile
  int64_t inRow;                // first input row (X or workspace)
  int64_t outRow;               // first output row of the chunk's item
  int32_t nc;                   // complex columns (<= 4 tcMaxKGroups(mg))
  int32_t kg;                   // k-groups (4 complex columns each) = ceil(nc / 4)
  int32_t mg;                   // row groups (8 rows each) = ceil(rows / 8)
  int32_t rows;                 // rows of the item (<= kTcRows)
  int32_t inIsX;
  int32_t flags;                // bit 0: first chunk of its item, bit 1: last
};
constexpr int32_t kTcFirst = 1, kTcLast = 2;

// Conversion of one chunk of the FP64 arena into its A tile.
struct TcFill {
  int64_t srcOff;               // FP64 arena entry of (item row 0, chunk column 0)
  int64_t tileOff;
  int32_t lda, rows, nc, kg, mg, pad;
};

struct TcSchedule {
  int32_t ctas = 0;                       // persistent CTAs per RHS tile
  // per stage s: chunk range of CTA c is ctaChunk0[s * (ctas + 1) + c] ..
  // ctaChunk0[s * (ctas + 1) + c + 1]
  std::vector<int64_t> ctaChunk0;
  std::vector<TcChunk> chunks;
  std::vector<TcFill> fills;
  int64_t arenaBytes = 0;                 // bytes of all tiles (every plane)
  int32_t maxChunksPerCta = 0;
};

// Cost of a chunk for the longest-first dealing, in units of ~10 ns:
// max(perChunk + perKstep * terms * ksteps, bytesPct / 100 * kg * mg * terms).
// The defaults follow per-CTA durations measured on the GB300; the autotuner
// (bfgFacAutotune) times other settings per stage.
struct TcCostModel {
  int64_t perChunk = 60;
  int64_t perKstep = 1;
  int64_t bytesPct = 29;
};

// Splits the 128-row program's items into chunks and deals each stage's items
// to `ctas` CTAs, longest first to the least-loaded CTA.  Tile offsets are in
// bytes for `terms` planes per tile; they follow the item order, so every cost
// model gives the same tiles.
void makeTcSchedule(ApplyProgram const &prog128, int terms, int ctas, TcSchedule &sched,
                    TcCostModel const &model = TcCostModel());
// the cost models the autotuner times, the default first
std::vector<TcCostModel> tcCandidateModels();

// Fill descriptors for the kernel-evaluation and re-expansion kernels.
struct FillDesc {
  int32_t kind, m, n, pad;
  int64_t arenaOff;
  int64_t s0, t0;               // tree-order point offsets
  double corig[3], ceq[3], cchk[3];
  double k;                     // wavenumber
  // a LAST block filled in column pieces: this piece holds columns
  // [j0, j0 + n) of the block's nTot proxy points (arenaOff at column j0)
  int32_t j0, nTot;
};

}  // namespace bfg
