// Quadtree build on the GPU (bfQuadtreeInit, quadtree.c:80-98, with the node
// split of quadtreeNodeInitRecursive, quadtree_node.c:123-282), for a forest
// of point sets at once (the batched problems' trees).
//
// The host build (Quadtree::build) splits a node by three in-place "sifts"
// (quadtree_node.c:148-194): pass q moves the points of quadrant q to the
// front of what is left of the node's range.  A pass keeps its members in
// order, but its swaps rotate the non-members: scanning positions after the
// first non-member s, a member at write t = p - s takes the slot of the
// non-member window's front, which moves to the back.  With arr[0] = the
// element at s, write t copies its own element for a non-member and
// arr[r(t)] for a member, r(t) = members seen in (s, p); the window's final
// contents are arr[F .. F+K) (F members after s, K non-members).  So:
//   member at p          -> position a + (members before p in the range);
//   position p >= a + m  <- the element at resolve(p), where resolve follows
//                           p -> s + r(p - s) while p holds a member,
// with a the range start and m its members; resolve is computed by pointer
// doubling.  The levels run breadth first over every tree of the forest; the
// host numbers the nodes depth first as the recursive build does, so both
// builds give the same permutation and node table, bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "bfg_kernels.cuh"
#include "bfg_plan.hpp"

namespace bfg {
namespace {

constexpr int kScanThreads = 256, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__global__ void splitXyKernel(int64_t n, double const *__restrict__ xy, double *__restrict__ X,
                              double *__restrict__ Y, int32_t *__restrict__ I) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    X[p] = xy[2 * p];
    Y[p] = xy[2 * p + 1];
    I[p] = (int32_t)p;
  }
}

// per set: min/max of x and y (bfPoints2GetBoundingBox, points.c:415-430);
// fmin / fmax are exact, so the order of the reduction does not matter
__global__ void bboxKernel(int64_t const *__restrict__ setOff, double const *__restrict__ X,
                           double const *__restrict__ Y, double *__restrict__ box) {
  int64_t const a = setOff[blockIdx.x], b = setOff[blockIdx.x + 1];
  double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
  for (int64_t p = a + threadIdx.x; p < b; p += blockDim.x) {
    x0 = fmin(x0, X[p]);
    x1 = fmax(x1, X[p]);
    y0 = fmin(y0, Y[p]);
    y1 = fmax(y1, Y[p]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    x0 = fmin(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    x1 = fmax(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y0 = fmin(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    y1 = fmax(y1, __shfl_xor_sync(0xffffffffu, y1, o));
  }
  __shared__ double s[4][32];
  int const lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    s[0][w] = x0;
    s[1][w] = x1;
    s[2][w] = y0;
    s[3][w] = y1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
      x0 = fmin(x0, s[0][q]);
      x1 = fmax(x1, s[1][q]);
      y0 = fmin(y0, s[2][q]);
      y1 = fmax(y1, s[3][q]);
    }
    box[4 * blockIdx.x + 0] = x0;
    box[4 * blockIdx.x + 1] = x1;
    box[4 * blockIdx.x + 2] = y0;
    box[4 * blockIdx.x + 3] = y1;
  }
}

// active node of every position (-1 outside the nodes being split)
__global__ void nodeOfKernel(int nNodes, int32_t const *__restrict__ i0, int32_t const *__restrict__ i1,
                             int32_t *__restrict__ nodeOf) {
  for (int nd = blockIdx.x; nd < nNodes; nd += gridDim.x)
    for (int32_t p = i0[nd] + threadIdx.x; p < i1[nd]; p += blockDim.x) nodeOf[p] = nd;
}

__global__ void passInitKernel(int nNodes, int32_t const *__restrict__ i1, int32_t *__restrict__ s,
                               int32_t *__restrict__ m) {
  int const nd = blockIdx.x * blockDim.x + threadIdx.x;
  if (nd < nNodes) {
    s[nd] = i1[nd];   // no non-member yet
    m[nd] = 0;
  }
}

// membership in quadrant q of the node (quadtree_node.c:148-194) and the
// segment heads of the pass ranges [aq, i1)
__global__ void classifyKernel(int64_t n, int q, int32_t const *__restrict__ nodeOf,
                               int32_t const *__restrict__ aq, double const *__restrict__ sx,
                               double const *__restrict__ sy, double const *__restrict__ X,
                               double const *__restrict__ Y, int32_t *__restrict__ flag,
                               uint8_t *__restrict__ head) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    int32_t const nd = nodeOf[p];
    if (nd < 0 || p < aq[nd]) {
      flag[p] = 0;
      head[p] = 1;
      continue;
    }
    double const x = X[p], y = Y[p], cx = sx[nd], cy = sy[nd];
    bool in;
    if (q == 0) in = x <= cx && y <= cy;
    else if (q == 1) in = x <= cx && y > cy;
    else in = x > cx && y <= cy;
    flag[p] = in ? 1 : 0;
    head[p] = p == aq[nd] ? 1 : 0;
  }
}

// ---- segmented inclusive scan of int32 values with head flags ----
struct Seg {
  int32_t v;
  int32_t h;
};
__device__ __forceinline__ Seg segOp(Seg a, Seg b) { return Seg{b.h ? b.v : a.v + b.v, a.h | b.h}; }

// tile-local inclusive scan; tile aggregate to agg
__global__ void __launch_bounds__(kScanThreads) segScanTileKernel(int64_t n, int32_t const *__restrict__ val,
                                                                 uint8_t const *__restrict__ head,
                                                                 int32_t *__restrict__ out,
                                                                 Seg *__restrict__ agg) {
  __shared__ Seg warpTot[kScanThreads / 32];
  int64_t const base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  Seg it[kScanItems];
  Seg acc{0, 0};
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t const p = base + k;
    Seg e = p < n ? Seg{val[p], head[p]} : Seg{0, 1};
    acc = k == 0 ? e : segOp(acc, e);
    it[k] = acc;
  }
  // scan of the thread totals across the warp, then across warps
  int const lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Seg t = acc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    Seg u{__shfl_up_sync(0xffffffffu, t.v, o), __shfl_up_sync(0xffffffffu, t.h, o)};
    if (lane >= o) t = segOp(u, t);
  }
  if (lane == 31) warpTot[w] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    Seg r = warpTot[0];
    for (int q = 1; q < kScanThreads / 32; ++q) {
      r = segOp(r, warpTot[q]);
      warpTot[q] = r;
    }
  }
  __syncthreads();
  // exclusive prefix of this thread within the tile
  Seg ex{0, 0};
  bool have = false;
  Seg up{__shfl_up_sync(0xffffffffu, t.v, 1), __shfl_up_sync(0xffffffffu, t.h, 1)};
  if (lane > 0) {
    ex = up;
    have = true;
  }
  if (w > 0) {
    ex = have ? segOp(warpTot[w - 1], ex) : warpTot[w - 1];
    have = true;
  }
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t const p = base + k;
    Seg r = have ? segOp(ex, it[k]) : it[k];
    if (p < n) out[p] = r.v;
  }
  if (threadIdx.x == kScanThreads - 1) agg[blockIdx.x] = have ? segOp(ex, acc) : acc;
}

// exclusive scan of the tile aggregates: one CTA of 1024 threads walks them
// in chunks of 1024 with a running carry; agg[t] becomes the carry into t
__global__ void __launch_bounds__(1024) segScanAggKernel(int64_t nTiles, Seg *__restrict__ agg) {
  __shared__ Seg warpTot[32];
  int const lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Seg carry{0, 0};
  for (int64_t base = 0; base < nTiles; base += 1024) {
    int64_t const t = base + threadIdx.x;
    Seg const e = t < nTiles ? agg[t] : Seg{0, 0};
    Seg x = e;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      Seg u{__shfl_up_sync(0xffffffffu, x.v, o), __shfl_up_sync(0xffffffffu, x.h, o)};
      if (lane >= o) x = segOp(u, x);
    }
    if (lane == 31) warpTot[w] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      Seg r = warpTot[0];
      for (int q = 1; q < 32; ++q) {
        r = segOp(r, warpTot[q]);
        warpTot[q] = r;
      }
    }
    __syncthreads();
    // exclusive prefix within the chunk
    Seg up{__shfl_up_sync(0xffffffffu, x.v, 1), __shfl_up_sync(0xffffffffu, x.h, 1)};
    Seg ex{0, 0};
    if (lane > 0) ex = up;
    if (w > 0) ex = segOp(warpTot[w - 1], ex);
    if (t < nTiles) agg[t] = segOp(carry, ex);
    Seg const chunkTot = warpTot[31];
    __syncthreads();
    carry = segOp(carry, chunkTot);
  }
}

// add each tile's carry to its positions before the tile's first head; then
// exclusive member counts = inclusive - own value
__global__ void segScanFinishKernel(int64_t n, Seg const *__restrict__ agg,
                                    int32_t const *__restrict__ val, uint8_t const *__restrict__ head,
                                    int32_t *__restrict__ out) {
  int64_t const tile = blockIdx.x;
  int64_t const a = tile * kScanTile, b = min(n, a + kScanTile);
  int32_t const carry = tile > 0 ? agg[tile].v : 0;
  // first head of the tile
  __shared__ int32_t firstHead;
  if (threadIdx.x == 0) firstHead = (int32_t)kScanTile;
  __syncthreads();
  for (int64_t p = a + threadIdx.x; p < b; p += blockDim.x)
    if (head[p]) atomicMin(&firstHead, (int32_t)(p - a));
  __syncthreads();
  for (int64_t p = a + threadIdx.x; p < b; p += blockDim.x) {
    int32_t v = out[p];
    if (p - a < firstHead) v += carry;
    out[p] = v - val[p];
  }
}

// first non-member s and member count m of each node's pass range
__global__ void passStatsKernel(int64_t n, int32_t const *__restrict__ nodeOf,
                                int32_t const *__restrict__ aq, int32_t const *__restrict__ i1,
                                int32_t const *__restrict__ flag, int32_t const *__restrict__ excl,
                                int32_t *__restrict__ s, int32_t *__restrict__ m) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    int32_t const nd = nodeOf[p];
    if (nd < 0 || p < aq[nd]) continue;
    if (!flag[p]) atomicMin(&s[nd], (int32_t)p);
    if (p == i1[nd] - 1) m[nd] = excl[p] + flag[p];
  }
}

// ptr[p]: the position write p - s copies from (p itself for non-members,
// the first non-member and positions outside the chain)
__global__ void ptrInitKernel(int64_t n, int32_t const *__restrict__ nodeOf,
                              int32_t const *__restrict__ aq, int32_t const *__restrict__ s,
                              int32_t const *__restrict__ flag, int32_t const *__restrict__ excl,
                              int32_t *__restrict__ ptr) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    int32_t const nd = nodeOf[p];
    int32_t r = (int32_t)p;
    if (nd >= 0 && p >= aq[nd]) {
      int32_t const sn = s[nd];
      if (p > sn && flag[p]) r = sn + (excl[p] - (sn - aq[nd]));
    }
    ptr[p] = r;
  }
}

__global__ void ptrJumpKernel(int64_t n, int32_t const *__restrict__ a, int32_t *__restrict__ b) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x)
    b[p] = a[a[p]];
}

__global__ void scatterKernel(int64_t n, int32_t const *__restrict__ nodeOf,
                              int32_t const *__restrict__ aq, int32_t const *__restrict__ m,
                              int32_t const *__restrict__ flag, int32_t const *__restrict__ excl,
                              int32_t const *__restrict__ ptr, double const *__restrict__ X,
                              double const *__restrict__ Y, int32_t const *__restrict__ I,
                              double *__restrict__ X2, double *__restrict__ Y2,
                              int32_t *__restrict__ I2) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    int32_t const nd = nodeOf[p];
    if (nd < 0 || p < aq[nd]) {
      X2[p] = X[p];
      Y2[p] = Y[p];
      I2[p] = I[p];
      continue;
    }
    int32_t const a = aq[nd];
    if (flag[p]) {   // member: stable, to the front
      int32_t const d = a + excl[p];
      X2[d] = X[p];
      Y2[d] = Y[p];
      I2[d] = I[p];
    }
    if (p >= a + m[nd]) {   // the non-member window, rotated
      int32_t const src = ptr[p];
      X2[p] = X[src];
      Y2[p] = Y[src];
      I2[p] = I[src];
    }
  }
}

__global__ void passAdvanceKernel(int nNodes, int32_t *__restrict__ aq, int32_t const *__restrict__ m,
                                  int32_t *__restrict__ off, int q) {
  int const nd = blockIdx.x * blockDim.x + threadIdx.x;
  if (nd < nNodes) {
    aq[nd] += m[nd];
    off[3 * nd + q] = aq[nd];
  }
}

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  void ensure(size_t k) {
    if (k <= n) return;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc(&p, std::max<size_t>(k, 1) * sizeof(T)) != cudaSuccess)
      throw std::runtime_error("quadtree build: out of device memory");
    n = k;
  }
};

void ckT(cudaError_t e, char const *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("quadtree build: ") + what + ": " + cudaGetErrorString(e));
}

int gridFor(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// a node of the breadth-first build, before depth-first numbering
struct BNode {
  QNode q;
  int kids[4] = {-1, -1, -1, -1};
};

}  // namespace

void buildQuadtreesGpu(double const *xy, int64_t const *setOff, int64_t numSets, int64_t leafSize,
                       void *stream, std::vector<Quadtree> &out) {
  cudaStream_t const st = static_cast<cudaStream_t>(stream);
  if (numSets < 1) throw std::runtime_error("quadtree build: no point sets");
  int64_t const n = setOff[numSets];
  if (n >= (int64_t)INT32_MAX) throw std::runtime_error("quadtree build: too many points");
  leafSize = leafSize < 1 ? 1 : leafSize;
  out.assign((size_t)numSets, Quadtree());
  DBuf<double> dxy, X, Y, X2, Y2, dsx, dsy, dbox;
  DBuf<int32_t> I, I2, nodeOf, flag, excl, ptrA, ptrB, di0, di1, daq, ds, dm, doff;
  DBuf<uint8_t> head;
  DBuf<int64_t> dset;
  DBuf<Seg> agg;
  size_t const nn = (size_t)std::max<int64_t>(n, 1);
  dxy.ensure(2 * nn);
  X.ensure(nn); Y.ensure(nn); X2.ensure(nn); Y2.ensure(nn);
  I.ensure(nn); I2.ensure(nn); nodeOf.ensure(nn); flag.ensure(nn); excl.ensure(nn);
  ptrA.ensure(nn); ptrB.ensure(nn); head.ensure(nn);
  int64_t const nTiles = (n + kScanTile - 1) / kScanTile;
  agg.ensure((size_t)std::max<int64_t>(nTiles, 1));
  dset.ensure((size_t)numSets + 1);
  dbox.ensure(4 * (size_t)numSets);
  ckT(cudaMemcpyAsync(dxy.p, xy, 2 * n * sizeof(double), cudaMemcpyHostToDevice, st), "upload");
  ckT(cudaMemcpyAsync(dset.p, setOff, (numSets + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st), "upload");
  if (n > 0) splitXyKernel<<<gridFor(n), 256, 0, st>>>(n, dxy.p, X.p, Y.p, I.p);
  bboxKernel<<<(unsigned)numSets, 256, 0, st>>>(dset.p, X.p, Y.p, dbox.p);
  std::vector<double> box(4 * (size_t)numSets);
  ckT(cudaMemcpyAsync(box.data(), dbox.p, box.size() * sizeof(double), cudaMemcpyDeviceToHost, st), "bbox");
  ckT(cudaStreamSynchronize(st), "bbox");

  // roots, then level by level
  std::vector<std::vector<BNode>> trees((size_t)numSets);
  struct Act { int tree, node; };
  std::vector<Act> act;
  for (int64_t t = 0; t < numSets; ++t) {
    QNode root = Quadtree::rootNode(box[4 * t], box[4 * t + 1], box[4 * t + 2], box[4 * t + 3]);
    root.i0 = setOff[t];
    root.i1 = setOff[t + 1];
    trees[(size_t)t].push_back(BNode{root, {-1, -1, -1, -1}});
    // the root is split whatever its size (Quadtree::build, as
    // quadtreeNodeInitRecursive from the root); its descendants only while
    // they hold more than leafSize points
    if (root.i1 - root.i0 > 0) act.push_back({(int)t, 0});
  }
  std::vector<int32_t> hi0, hi1, hoff;
  std::vector<double> hsx, hsy;
  while (!act.empty()) {
    int const na = (int)act.size();
    hi0.resize(na); hi1.resize(na); hsx.resize(na); hsy.resize(na); hoff.resize(3 * (size_t)na);
    int64_t maxLen = 1;
    for (int a = 0; a < na; ++a) {
      QNode const &q = trees[(size_t)act[a].tree][(size_t)act[a].node].q;
      hi0[a] = (int32_t)q.i0;
      hi1[a] = (int32_t)q.i1;
      hsx[a] = q.sx;
      hsy[a] = q.sy;
      maxLen = std::max<int64_t>(maxLen, q.i1 - q.i0);
    }
    di0.ensure(na); di1.ensure(na); daq.ensure(na); ds.ensure(na); dm.ensure(na);
    dsx.ensure(na); dsy.ensure(na); doff.ensure(3 * (size_t)na);
    ckT(cudaMemcpyAsync(di0.p, hi0.data(), na * 4, cudaMemcpyHostToDevice, st), "nodes");
    ckT(cudaMemcpyAsync(daq.p, hi0.data(), na * 4, cudaMemcpyHostToDevice, st), "nodes");
    ckT(cudaMemcpyAsync(di1.p, hi1.data(), na * 4, cudaMemcpyHostToDevice, st), "nodes");
    ckT(cudaMemcpyAsync(dsx.p, hsx.data(), na * 8, cudaMemcpyHostToDevice, st), "nodes");
    ckT(cudaMemcpyAsync(dsy.p, hsy.data(), na * 8, cudaMemcpyHostToDevice, st), "nodes");
    ckT(cudaMemsetAsync(nodeOf.p, 0xFF, n * 4, st), "nodeOf");
    nodeOfKernel<<<std::min(na, 152 * 16), 256, 0, st>>>(na, di0.p, di1.p, nodeOf.p);
    // doubling rounds: a chain is shorter than the longest range
    int rounds = 1;
    while ((int64_t(1) << rounds) < maxLen) ++rounds;
    for (int q = 0; q < 3; ++q) {
      passInitKernel<<<(na + 255) / 256, 256, 0, st>>>(na, di1.p, ds.p, dm.p);
      classifyKernel<<<gridFor(n), 256, 0, st>>>(n, q, nodeOf.p, daq.p, dsx.p, dsy.p, X.p, Y.p,
                                                 flag.p, head.p);
      segScanTileKernel<<<(unsigned)nTiles, kScanThreads, 0, st>>>(n, flag.p, head.p, excl.p, agg.p);
      segScanAggKernel<<<1, 1024, 0, st>>>(nTiles, agg.p);
      segScanFinishKernel<<<(unsigned)nTiles, kScanThreads, 0, st>>>(n, agg.p, flag.p, head.p, excl.p);
      passStatsKernel<<<gridFor(n), 256, 0, st>>>(n, nodeOf.p, daq.p, di1.p, flag.p, excl.p, ds.p, dm.p);
      ptrInitKernel<<<gridFor(n), 256, 0, st>>>(n, nodeOf.p, daq.p, ds.p, flag.p, excl.p, ptrA.p);
      for (int r = 0; r < rounds; ++r) {
        ptrJumpKernel<<<gridFor(n), 256, 0, st>>>(n, ptrA.p, ptrB.p);
        std::swap(ptrA.p, ptrB.p);
      }
      scatterKernel<<<gridFor(n), 256, 0, st>>>(n, nodeOf.p, daq.p, dm.p, flag.p, excl.p, ptrA.p,
                                                X.p, Y.p, I.p, X2.p, Y2.p, I2.p);
      std::swap(X.p, X2.p);
      std::swap(Y.p, Y2.p);
      std::swap(I.p, I2.p);
      passAdvanceKernel<<<(na + 255) / 256, 256, 0, st>>>(na, daq.p, dm.p, doff.p, q);
    }
    ckT(cudaGetLastError(), "sift launch");
    ckT(cudaMemcpyAsync(hoff.data(), doff.p, 3 * (size_t)na * 4, cudaMemcpyDeviceToHost, st), "offsets");
    ckT(cudaStreamSynchronize(st), "sift");
    // children in quadrant order (quadtree_node.c:196-282), as Quadtree::split
    std::vector<Act> next;
    for (int a = 0; a < na; ++a) {
      auto &tr = trees[(size_t)act[a].tree];
      int const pi = act[a].node;
      QNode const par = tr[(size_t)pi].q;
      int64_t const off[5] = {par.i0, hoff[3 * a], hoff[3 * a + 1], hoff[3 * a + 2], par.i1};
      for (int q = 0; q < 4; ++q) {
        if (off[q + 1] - off[q] == 0) continue;
        QNode ch = Quadtree::childNode(par, q);
        ch.i0 = off[q];
        ch.i1 = off[q + 1];
        int const ci = (int)tr.size();
        tr.push_back(BNode{ch, {-1, -1, -1, -1}});
        tr[(size_t)pi].kids[q] = ci;
        if (ch.i1 - ch.i0 > leafSize) {
          if (ch.depth > 200) throw std::runtime_error("quadtree deeper than 200 levels (duplicate points?)");
          next.push_back({act[a].tree, ci});
        }
      }
    }
    act.swap(next);
  }
  std::vector<int32_t> perm((size_t)n);
  if (n > 0) ckT(cudaMemcpyAsync(perm.data(), I.p, n * 4, cudaMemcpyDeviceToHost, st), "perm");
  ckT(cudaStreamSynchronize(st), "perm");

  // depth-first numbering (node index = creation order of the recursive build)
  for (int64_t t = 0; t < numSets; ++t) {
    auto const &tr = trees[(size_t)t];
    Quadtree &qt = out[(size_t)t];
    qt.leafSize = leafSize;
    qt.nodes.clear();
    qt.nodes.reserve(tr.size());
    std::vector<int> newIdx(tr.size(), -1);
    // a node's index is assigned when its parent creates it; its subtree is
    // numbered before its next sibling
    struct Fr { int b; int q; };
    newIdx[0] = 0;
    qt.nodes.push_back(tr[0].q);
    qt.nodes[0].i0 -= setOff[t];
    qt.nodes[0].i1 -= setOff[t];
    std::vector<Fr> stack{{0, 0}};
    while (!stack.empty()) {
      Fr &f = stack.back();
      if (f.q == 4) {
        stack.pop_back();
        continue;
      }
      int const q = f.q++;
      int const kb = tr[(size_t)f.b].kids[q];
      if (kb < 0) continue;
      int const ni = (int)qt.nodes.size();
      newIdx[(size_t)kb] = ni;
      QNode c = tr[(size_t)kb].q;
      c.i0 -= setOff[t];
      c.i1 -= setOff[t];
      c.parent = newIdx[(size_t)f.b];
      qt.nodes.push_back(c);
      qt.nodes[(size_t)newIdx[(size_t)f.b]].child[q] = ni;
      stack.push_back({kb, 0});
    }
    int64_t const a = setOff[t], b = setOff[t + 1];
    qt.perm.resize((size_t)(b - a));
    for (int64_t p = a; p < b; ++p) qt.perm[(size_t)(p - a)] = (int64_t)perm[(size_t)p] - a;
  }
}

}  // namespace bfg
