// C-ABI layer of libbfg.so (declarations and contracts in include/bfg.h).
#include "../../include/bfg.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "bfg_kernels.cuh"
#include "bfg_plan.hpp"
#include "hankel.cuh"

struct bfgContext_s {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::string lastError;
};

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    return e;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

struct BfgError {
  bfgStatus status;
  std::string msg;
};

void ck(cudaError_t e, char const *what) {
  if (e != cudaSuccess)
    throw BfgError{BFG_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

// CUDA events released on every exit path, a failed check included
struct Events {
  std::vector<cudaEvent_t> v;
  Events(size_t n, char const *what) : v(n, nullptr) {
    for (auto &e : v) {
      cudaError_t const r = cudaEventCreate(&e);
      if (r != cudaSuccess) {
        e = nullptr;
        release();
        ck(r, what);
      }
    }
  }
  ~Events() { release(); }
  Events(Events const &) = delete;
  Events &operator=(Events const &) = delete;
  cudaEvent_t operator[](size_t i) const { return v[i]; }
  void release() {
    for (auto &e : v)
      if (e) {
        cudaEventDestroy(e);
        e = nullptr;
      }
  }
};

template <typename T>
void upload(DevBuf &buf, std::vector<T> const &v, cudaStream_t s, char const *what) {
  size_t n = std::max<size_t>(1, v.size()) * sizeof(T);
  ck(buf.ensure(n), what);
  if (!v.empty())
    ck(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), what);
}

}  // namespace

struct bfgFac_s {
  bfgContext ctx = nullptr;
  bfgHelm2 helm{};
  bfgFacOptions opts{};
  bfg::Plan plan;
  bfg::ApplyProgram prog;
  bfgFacStats stats{};
  // device data
  DevBuf srcPts, tgtPts;            // x, y, nx, ny planes (tree order)
  bool srcHasNormals = false, tgtHasNormals = false;
  DevBuf arena64, arena32, arenaDf;
  bool arena32Ready = false, arenaDfReady = false;
  DevBuf srcPerm, tgtPerm;
  DevBuf items, contribs, rowSeg, segStart, segContrib0, segBase;
  DevBuf ws, xbuf;
  DevBuf hx128, hy128, hx64, hy64;  // staging of the host-operand apply
  // pipelined host-operand applies (bfgFacApplyHostAsync): two staging
  // slots; uploads and downloads on streams of their own, so that one
  // call's copies overlap another's compute on the context's stream
  struct HostSlot {
    DevBuf x128, y128, x64, y64;
    cudaEvent_t uploaded = nullptr, consumed = nullptr, computed = nullptr, downloaded = nullptr;
    bool started = false;
  } hslot[2];
  cudaStream_t upStream = nullptr, downStream = nullptr;
  int64_t asyncCalls = 0;
  ~bfgFac_s() {
    if (upStream) cudaStreamSynchronize(upStream);
    if (downStream) cudaStreamSynchronize(downStream);
    for (auto &h : hslot)
      for (cudaEvent_t e : {h.uploaded, h.consumed, h.computed, h.downloaded})
        if (e) cudaEventDestroy(e);
    if (upStream) cudaStreamDestroy(upStream);
    if (downStream) cudaStreamDestroy(downStream);
  }
  std::vector<int64_t> stageItem0;
  // split-BF16 tensor-core apply, per plane count (index terms - 2): the
  // chunk schedule of the 128-row program and the bf16 planes of the factors
  struct Tc {
    bool ready = false;
    int32_t ctas = 0;                 // resident CTAs on the device
    size_t stages = 0;
    DevBuf arena;
    bfg::ApplyProgram p128;           // the 128-row program the chunks cut
    // chunk dealings by number of chunk streams: R right-hand sides in
    // tiles of rt take ctas / ceil(R / rt) streams (every tile of every
    // stream resident)
    struct Sched {
      DevBuf chunks, ctaChunk0;
    };
    std::map<int32_t, Sched> sched;
    // RHS tile widths the autotuner chose, by R (else bfg::tcRhsTile(R))
    std::map<int64_t, int32_t> rhsTile;
  } tc[2];
  DevBuf tcStatus;                  // kStatusTcTimeout from the tensor-core kernel
  uint64_t tcWaitLimitNs = bfg::kTcWaitLimitNs;   // lowered only by the test hook
  // the inputs (original order), kept for bfgFacSave; k holds one
  // wavenumber per problem and the offsets are empty for a single problem
  std::vector<double> inSrcXy, inSrcN, inTgtXy, inTgtN, inK;
  std::vector<int64_t> inSrcOff, inTgtOff;
};

namespace {

bfgStatus fail(bfgContext ctx, bfgStatus st, std::string const &msg) {
  if (ctx) ctx->lastError = msg;
  return st;
}

// the 2 P quadtrees of P problems (source tree of problem p at 2p, target
// tree at 2p+1) built on the GPU in one pass over all of them
std::vector<bfg::Quadtree> gpuTrees(cudaStream_t s, double const *srcXy, int64_t const *srcOff,
                                    double const *tgtXy, int64_t const *tgtOff, int64_t P,
                                    int64_t leafSize) {
  std::vector<int64_t> off((size_t)(2 * P + 1), 0);
  for (int64_t p = 0; p < P; ++p) {
    off[(size_t)(2 * p + 1)] = off[(size_t)(2 * p)] + (srcOff[p + 1] - srcOff[p]);
    off[(size_t)(2 * p + 2)] = off[(size_t)(2 * p + 1)] + (tgtOff[p + 1] - tgtOff[p]);
  }
  std::vector<double> xy((size_t)(2 * off.back()));
  for (int64_t p = 0; p < P; ++p) {
    std::copy(srcXy + 2 * srcOff[p], srcXy + 2 * srcOff[p + 1], xy.begin() + 2 * off[(size_t)(2 * p)]);
    std::copy(tgtXy + 2 * tgtOff[p], tgtXy + 2 * tgtOff[p + 1], xy.begin() + 2 * off[(size_t)(2 * p + 1)]);
  }
  std::vector<bfg::Quadtree> trees;
  bfg::buildQuadtreesGpu(xy.data(), off.data(), 2 * P, leafSize, s, trees);
  return trees;
}

template <typename F>
bfgStatus guarded(bfgContext ctx, F &&f) {
  try {
    if (ctx) {
      int cur = -1;
      if (cudaGetDevice(&cur) == cudaSuccess && cur != ctx->device) cudaSetDevice(ctx->device);
    }
    return f();
  } catch (BfgError const &e) {
    return fail(ctx, e.status, e.msg);
  } catch (std::bad_alloc const &) {
    return fail(ctx, BFG_ERROR_MEMORY, "host allocation failed");
  } catch (std::exception const &e) {
    return fail(ctx, BFG_ERROR_RUNTIME, e.what());
  }
}

bfg::PointsDev pointsView(DevBuf const &b, int64_t n, bool normals) {
  bfg::PointsDev p;
  double const *base = b.as<double>();
  p.x = base;
  p.y = base + n;
  if (normals) {
    p.nx = base + 2 * n;
    p.ny = base + 3 * n;
  }
  return p;
}

void uploadTreePoints(DevBuf &buf, double const *xy, double const *nrm, int64_t n,
                      std::vector<int64_t> const &perm, cudaStream_t s) {
  std::vector<double> h((size_t)(nrm ? 4 : 2) * n);
  for (int64_t i = 0; i < n; ++i) {
    int64_t o = perm[(size_t)i];
    h[(size_t)i] = xy[2 * o];
    h[(size_t)(n + i)] = xy[2 * o + 1];
    if (nrm) {
      h[(size_t)(2 * n + i)] = nrm[2 * o];
      h[(size_t)(3 * n + i)] = nrm[2 * o + 1];
    }
  }
  upload(buf, h, s, "upload points");
}

bfg::KernelParams kernelParams(bfgHelm2 const &h, int32_t layerPot) {
  bfg::KernelParams kp{};
  kp.k = h.k;
  kp.layerPot = layerPot;
  kp.alphaRe = h.alphaRe;
  kp.alphaIm = h.alphaIm;
  kp.betaRe = h.betaRe;
  kp.betaIm = h.betaIm;
  return kp;
}

int32_t proxyLayerPot(int32_t lp) {
  // BF_PROXY_LAYER_POT (layer_pot.h:87-93)
  switch (lp) {
    case bfg::kLpSingle: return bfg::kLpSingle;
    case bfg::kLpPvDouble: return bfg::kLpPvDouble;
    case bfg::kLpPvNormalDerivSingle: return bfg::kLpSingle;
    case bfg::kLpCombinedField: return bfg::kLpCombinedField;
    default: return 0;
  }
}

bool validLayerPot(int32_t lp) {
  return lp == 1 || lp == 2 || lp == 3 || lp == 5;
}

bfg::FillDesc toDesc(bfg::Block const &b) {
  bfg::FillDesc d{};
  d.kind = b.kind;
  d.m = b.m;
  d.n = b.n;
  d.arenaOff = b.arenaOff;
  d.s0 = b.s0;
  d.t0 = b.t0;
  d.corig[0] = b.corig.cx; d.corig[1] = b.corig.cy; d.corig[2] = b.corig.r;
  d.ceq[0] = b.ceq.cx; d.ceq[1] = b.ceq.cy; d.ceq[2] = b.ceq.r;
  d.cchk[0] = b.cchk.cx; d.cchk[1] = b.cchk.cy; d.cchk[2] = b.cchk.r;
  d.k = b.k;
  d.j0 = 0;
  d.nTot = b.n;
  return d;
}

constexpr int64_t kSmemLimit = 220 * 1024;
// smallest relative pseudo-inverse cut the double-float Jacobi accepts: its
// columns carry rounding noise at ~1e-14 of the largest, and kept singular
// vectors closer to it than 1e4x do not settle within the sweep cap
constexpr double kDfJacobiMinCut = 1e-10;
constexpr int64_t kScratchBudgetEntries = (int64_t)1 << 27;   // 2 GiB of complex128
// ranks from which a block that misses shared memory gets a whole cluster
constexpr int32_t kClusterMinRank = 128;
// the randomized re-expansion path: blocks from this rank estimate whose
// initial sketch is at most kSketchMaxFraction of it; the sketch width is
// kSketchWidthScale k r1 r2 / R + kSketchWidthPad; scratch per batch
constexpr int32_t kSketchMinRank = 128;
// the same path at full width (l = p) for every other FIRST/MIDDLE block
// from this rank with the relative cut and FP64 sweeps: its Jacobi runs on
// the triangular factor of a QR of Z_equiv, which converges in fewer sweeps
// than the one-sided Jacobi on Z_equiv itself (factorization time at
// 65,536 / 262,144 points and of the 256-problem batch: 1.95 -> 1.12 s,
// 34.7 -> 24.2 s, 48.3 -> 26.1 s; the same operators to rounding).  The
// random Q stays at full width: with Q = I the QR of Z_equiv^H is not rank
// revealing and the sweeps were slower again (24.2 -> 31.0 s)
constexpr int32_t kQrMinRank = 32;
constexpr double kSketchMaxFraction = 0.8;
constexpr double kSketchWidthScale = 1.1;
constexpr int32_t kSketchWidthPad = 40;
constexpr int64_t kSketchBudgetEntries = (int64_t)1 << 30;   // 16 GiB of complex128
// LAST and DENSE blocks are filled in column pieces of at most this many
// columns and entries, so that one large block spreads over many CTAs
constexpr int32_t kFillPieceCols = 2048;
constexpr int64_t kFillPieceEntries = (int64_t)1 << 20;

// the sketch's capture threshold: its smallest singular value must lie
// below this fraction of the largest, three decades under the relative cut
// and never closer than 1e-13 to the kernels' rounding floor (~1e-14)
double sketchCapture(bfgFacOptions const &o) {
  return std::max(1e-13, std::min(1e-12, 1e-3 * o.pinvTol));
}

void factorize(bfgFac f) {
  cudaStream_t s = f->ctx->stream;
  bfg::Plan &plan = f->plan;
  int64_t const nSrc = (int64_t)plan.src.perm.size(), nTgt = (int64_t)plan.tgt.perm.size();
  (void)nTgt;
  bfg::PointsDev src = pointsView(f->srcPts, nSrc, f->srcHasNormals);
  bfg::PointsDev tgt = pointsView(f->tgtPts, (int64_t)plan.tgt.perm.size(), f->tgtHasNormals);

  ck(f->arena64.ensure(std::max<int64_t>(1, plan.arenaEntries) * sizeof(double2)), "arena");

  // FIRST/MIDDLE blocks by where their Jacobi working set lives: shared
  // memory (8 or 16 warps), global memory with one CTA, or global memory
  // with a thread-block cluster for the largest ranks (the critical path)
  // Blocks with the same Z_equiv (rank, equivalent circle, check circle,
  // wavenumber) share one SVD: a group's leader carries the largest n of its
  // members and is routed by it; every member gets its own Z_shift.
  struct GroupList {
    std::vector<bfg::FillDesc> lead;
    std::vector<std::vector<bfg::FillDesc>> mem;
  };
  std::vector<bfg::FillDesc> fill, full;
  GroupList reSmem8, reSmem16, reGlobal, reCluster;
  std::vector<bfg::SketchInput> sketch;
  int32_t maxProxyN = 1;
  int64_t maxRank = 0;
  bool const sketchCut = f->opts.pinvCut == 1 && f->opts.pinvTol >= kDfJacobiMinCut;
  auto route = [&](bfg::FillDesc const &d, std::vector<bfg::FillDesc> &&members) {
    GroupList *g;
    if (d.m <= 16 && bfg::reexpansionSmemBytes(d.m, d.n, 8) <= kSmemLimit)
      g = &reSmem8;
    else if (bfg::reexpansionSmemBytes(d.m, d.n, 16) <= kSmemLimit)
      g = &reSmem16;
    else if (d.m >= kClusterMinRank)
      g = &reCluster;
    else
      g = &reGlobal;
    g->lead.push_back(d);
    g->mem.push_back(std::move(members));
  };
  for (auto const &b : plan.blocks) {
    bfg::FillDesc d = toDesc(b);
    if (b.kind == bfg::kLast || b.kind == bfg::kDense) {
      if (b.kind == bfg::kLast) maxRank = std::max<int64_t>(maxRank, b.n);
      // column pieces (the proxy points of a LAST piece come from j0 / nTot)
      int64_t const w = std::max<int64_t>(
          1, std::min<int64_t>(kFillPieceCols, kFillPieceEntries / std::max(1, b.m)));
      for (int64_t j = 0; j < b.n; j += w) {
        bfg::FillDesc q = d;
        q.n = (int32_t)std::min<int64_t>(w, b.n - j);
        q.arenaOff = d.arenaOff + j * b.m;
        if (b.kind == bfg::kLast) {
          q.j0 = (int32_t)j;
          q.nTot = b.n;
          maxProxyN = std::max(maxProxyN, q.n);
        } else {
          q.s0 = d.s0 + j;
          q.j0 = 0;
          q.nTot = q.n;
        }
        fill.push_back(q);
      }
      continue;
    }
    maxRank = std::max<int64_t>(maxRank, b.m);
    bool const fullOk = bfg::reexpansionGeoBytes(b.m, b.n) <= kSmemLimit;
    if (f->opts.sketch && sketchCut && b.m >= kSketchMinRank) {
      int32_t const l = bfg::sketchWidth(d, kSketchWidthScale, kSketchWidthPad);
      if (l <= kSketchMaxFraction * b.m) {
        sketch.push_back(bfg::SketchInput{d, l, fullOk ? 1 : 0});
        continue;
      }
    }
    if (f->opts.sketch && sketchCut && f->opts.jacobiArith == 0 && b.m >= kQrMinRank) {
      sketch.push_back(bfg::SketchInput{d, b.m, 0});
      continue;
    }
    if (!fullOk) {
      if (!f->opts.sketch)
        throw BfgError{BFG_ERROR_NOT_IMPLEMENTED,
                       "block geometry exceeds shared memory (options.sketch = 0)"};
      // the randomized path with the capture test, or at full width
      int32_t const l = sketchCut ? bfg::sketchWidth(d, kSketchWidthScale, kSketchWidthPad) : b.m;
      sketch.push_back(bfg::SketchInput{d, l, 0});
      continue;
    }
    full.push_back(d);
  }
  std::stable_sort(fill.begin(), fill.end(), [](bfg::FillDesc const &a, bfg::FillDesc const &b) {
    return (int64_t)a.m * a.n > (int64_t)b.m * b.n;
  });

  DevBuf status, dFill, dSmem8, dSmem16, dBatch, dScratchOff, dFlags, scratch;
  ck(status.ensure(sizeof(int32_t)), "status");
  ck(cudaMemsetAsync(status.p, 0, sizeof(int32_t), s), "status");

  Events const ev(5, "event");
  cudaEvent_t const e0 = ev[0], e1 = ev[1], eFill = ev[2], eSmem = ev[3], eSketch = ev[4];
  ck(cudaEventRecord(e0, s), "event");

  bfg::KernelParams kpTrue = kernelParams(f->helm, f->helm.layerPot);
  bfg::KernelParams kpProxy = kernelParams(f->helm, proxyLayerPot(f->helm.layerPot));
  double2 *arena = f->arena64.as<double2>();
  int32_t *st = status.as<int32_t>();

  upload(dFill, fill, s, "descriptors");
  ck(bfg::launchFillBlocks(dFill.as<bfg::FillDesc>(), (int32_t)fill.size(), src, tgt, kpTrue,
                           arena, maxProxyN, st, s),
     "fill kernel");
  ck(cudaEventRecord(eFill, s), "event");

  // the randomized re-expansions; blocks it hands back join the full path
  {
    std::vector<bfg::FillDesc> back;
    bfg::SketchReport rep;
    ck(bfg::runSketchReexpansion(sketch, src, kpProxy, f->opts.pinvCut, f->opts.pinvTol,
                                 sketchCapture(f->opts), arena, kSketchBudgetEntries, s, &back,
                                 &rep),
       "randomized re-expansion");
    full.insert(full.end(), back.begin(), back.end());
    f->stats.numSketched = rep.blocks;
    f->stats.sketchGroups = rep.groups;
    f->stats.sketchRetries = rep.retries;
    f->stats.sketchFallbacks = rep.fallbacks;
    f->stats.sketchMaxWidth = rep.maxWidth;
    f->stats.sketchMs = rep.ms;
    f->stats.sketchMeanWidth = rep.blocks ? (double)rep.sumWidth / (double)rep.blocks : 0.0;
    for (int i = 0; i < 8; ++i) f->stats.sketchPhaseMs[i] = rep.phaseMs[i];
    if (rep.notConverged) f->stats.jacobiNotConverged = 1;
  }
  ck(cudaEventRecord(eSketch, s), "event");

  // the full path's groups, routed by their leaders
  {
    std::map<std::array<double, 8>, size_t> key;
    std::vector<std::vector<bfg::FillDesc>> groups;
    for (auto const &d : full) {
      std::array<double, 8> const k8 = {(double)d.m, d.ceq[0], d.ceq[1], d.ceq[2],
                                        d.cchk[0], d.cchk[1], d.cchk[2], d.k};
      auto it = key.find(k8);
      if (it == key.end()) {
        key.emplace(k8, groups.size());
        groups.push_back({d});
      } else {
        groups[it->second].push_back(d);
      }
    }
    for (auto &g : groups) {
      bfg::FillDesc lead = g[0];
      for (auto const &m : g) lead.n = std::max(lead.n, m.n);
      route(lead, std::move(g));
    }
    f->stats.reexpSvds = (int64_t)groups.size();
  }
  // largest work first, so that the longest CTAs start in the first wave
  auto cost = [](bfg::FillDesc const &lead, std::vector<bfg::FillDesc> const &mem) {
    double n = 0;
    for (auto const &m : mem) n += m.n;
    return (double)lead.m * lead.m * (3.0 * lead.m + n);
  };
  for (GroupList *g : {&reSmem8, &reSmem16, &reGlobal, &reCluster}) {
    std::vector<size_t> order(g->lead.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
      return cost(g->lead[a], g->mem[a]) > cost(g->lead[b], g->mem[b]);
    });
    GroupList sorted;
    for (size_t i : order) {
      sorted.lead.push_back(g->lead[i]);
      sorted.mem.push_back(std::move(g->mem[i]));
    }
    *g = std::move(sorted);
  }
  // a range of groups as the kernels take it: leaders, members back to back,
  // group starts
  auto flatten = [](GroupList const &g, size_t i0, size_t i1, std::vector<bfg::FillDesc> &lead,
                    std::vector<bfg::FillDesc> &mem, std::vector<int32_t> &start) {
    lead.assign(g.lead.begin() + (long)i0, g.lead.begin() + (long)i1);
    mem.clear();
    start.assign(1, 0);
    for (size_t i = i0; i < i1; ++i) {
      mem.insert(mem.end(), g.mem[i].begin(), g.mem[i].end());
      start.push_back((int32_t)mem.size());
    }
  };
  DevBuf dMem, dStart;
  std::vector<bfg::FillDesc> leadV, memV;
  std::vector<int32_t> startV;

  auto maxBytes = [](std::vector<bfg::FillDesc> const &v, int warps, bool geoOnly) {
    int64_t m = 0;
    for (auto const &d : v)
      m = std::max(m, geoOnly ? bfg::reexpansionGeoBytes(d.m, d.n)
                              : bfg::reexpansionSmemBytes(d.m, d.n, warps));
    return (int32_t)m;
  };
  DevBuf dMem16, dStart16;
  flatten(reSmem8, 0, reSmem8.lead.size(), leadV, memV, startV);
  upload(dSmem8, leadV, s, "descriptors");
  upload(dMem, memV, s, "descriptors");
  upload(dStart, startV, s, "descriptors");
  ck(bfg::launchReexpansion(dSmem8.as<bfg::FillDesc>(), (int32_t)leadV.size(), src, kpProxy,
                            f->opts.pinvCut, f->opts.pinvTol, arena, nullptr, nullptr, nullptr,
                            st, 0, maxBytes(leadV, 8, false), 256, f->opts.jacobiArith, s,
                            dMem.as<bfg::FillDesc>(), dStart.as<int32_t>()),
     "re-expansion kernel");
  flatten(reSmem16, 0, reSmem16.lead.size(), leadV, memV, startV);
  upload(dSmem16, leadV, s, "descriptors");
  upload(dMem16, memV, s, "descriptors");
  upload(dStart16, startV, s, "descriptors");
  ck(bfg::launchReexpansion(dSmem16.as<bfg::FillDesc>(), (int32_t)leadV.size(), src, kpProxy,
                            f->opts.pinvCut, f->opts.pinvTol, arena, nullptr, nullptr, nullptr,
                            st, 0, maxBytes(leadV, 16, false), 512, f->opts.jacobiArith, s,
                            dMem16.as<bfg::FillDesc>(), dStart16.as<int32_t>()),
     "re-expansion kernel");
  ck(cudaEventRecord(eSmem, s), "event");

  // global-memory working sets, in batches bounded by the scratch budget
  int32_t const clusterCtas = bfg::reexpansionClusterCtas();
  for (int mode = 1; mode <= 2; ++mode) {
    GroupList const &list = mode == 1 ? reGlobal : reCluster;
    int32_t const warps = mode == 1 ? 16 : 16 * clusterCtas;
    size_t i0 = 0;
    while (i0 < list.lead.size()) {
      std::vector<int64_t> offs;
      int64_t total = 0;
      size_t i1 = i0;
      while (i1 < list.lead.size()) {
        int64_t e = bfg::reexpansionScratchEntries(list.lead[i1].m, warps);
        if (i1 > i0 && total + e > kScratchBudgetEntries) break;
        offs.push_back(total);
        total += e;
        ++i1;
      }
      flatten(list, i0, i1, leadV, memV, startV);
      ck(scratch.ensure((size_t)total * sizeof(double2)), "re-expansion scratch");
      ck(dFlags.ensure(leadV.size() * clusterCtas * sizeof(int32_t)), "re-expansion flags");
      upload(dBatch, leadV, s, "descriptors");
      upload(dScratchOff, offs, s, "descriptors");
      upload(dMem, memV, s, "descriptors");
      upload(dStart, startV, s, "descriptors");
      ck(bfg::launchReexpansion(dBatch.as<bfg::FillDesc>(), (int32_t)leadV.size(), src, kpProxy,
                                f->opts.pinvCut, f->opts.pinvTol, arena, scratch.as<double2>(),
                                dScratchOff.as<int64_t>(), dFlags.as<int32_t>(), st, mode,
                                maxBytes(leadV, 0, true), 512, f->opts.jacobiArith, s,
                                dMem.as<bfg::FillDesc>(), dStart.as<int32_t>()),
         mode == 1 ? "re-expansion kernel (global)" : "re-expansion kernel (cluster)");
      // the batch's descriptors, offsets and scratch are reused by the next
      ck(cudaStreamSynchronize(s), "re-expansion");
      i0 = i1;
    }
  }
  ck(cudaEventRecord(e1, s), "event");
  ck(cudaStreamSynchronize(s), "factorization");
  float ms = 0, msFill = 0, msSmem = 0, msGlobal = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventElapsedTime(&msFill, e0, eFill);
  cudaEventElapsedTime(&msSmem, eSketch, eSmem);
  cudaEventElapsedTime(&msGlobal, eSmem, e1);
  f->stats.fillMs = msFill;
  f->stats.reexpSmemMs = msSmem;
  f->stats.reexpGlobalMs = msGlobal;
  int32_t hst = 0;
  ck(cudaMemcpy(&hst, status.p, sizeof hst, cudaMemcpyDeviceToHost), "status");
  if (hst & bfg::kStatusBadDescriptor) throw BfgError{BFG_ERROR_RUNTIME, "bad block descriptor"};

  f->stats.factorMs = ms;
  f->stats.maxRank = maxRank;
  if (hst & bfg::kStatusJacobiNotConverged) f->stats.jacobiNotConverged = 1;
}

void buildApply(bfgFac f) {
  cudaStream_t s = f->ctx->stream;
  bfg::makeApplyProgram(f->plan, f->prog);
  bfg::ApplyProgram const &p = f->prog;
  upload(f->items, p.items, s, "apply program");
  upload(f->contribs, p.contribs, s, "apply program");
  upload(f->rowSeg, p.rowSeg, s, "apply program");
  upload(f->segStart, p.segStart, s, "apply program");
  upload(f->segContrib0, p.segContrib0, s, "apply program");
  upload(f->segBase, p.segBase, s, "apply program");
  f->stageItem0 = p.stageItem0;
  ck(cudaStreamSynchronize(s), "apply program");
}

void fillStats(bfgFac f) {
  bfgFacStats &st = f->stats;
  st.numRows = (int64_t)f->plan.tgt.perm.size();
  st.numCols = (int64_t)f->plan.src.perm.size();
  st.numBlocks = (int64_t)f->plan.blocks.size();
  st.numFirst = st.numMiddle = st.numLast = st.numDense = 0;
  for (auto const &b : f->plan.blocks) {
    if (b.kind == bfg::kFirst) ++st.numFirst;
    else if (b.kind == bfg::kMiddle) ++st.numMiddle;
    else if (b.kind == bfg::kLast) ++st.numLast;
    else ++st.numDense;
  }
  st.numProducts = (int64_t)f->plan.products.size();
  st.arenaEntries = f->plan.arenaEntries;
  st.numStages = (int64_t)f->stageItem0.size() - 1;
  st.numItems = (int64_t)f->prog.items.size();
  st.flopsPerRhs = f->prog.flopsPerRhs;
}

template <typename T2>
void runApply(bfgFac f, T2 const *arena, T2 const *X, int64_t ldx, int64_t R, T2 *Y,
              int64_t ldy, uint32_t flags, std::vector<cudaEvent_t> *events) {
  cudaStream_t s = f->ctx->stream;
  bfg::ApplyProgram const &p = f->prog;
  ck(f->ws.ensure((size_t)std::max<int64_t>(1, p.wsRows) * R * sizeof(T2)), "workspace");
  T2 *W = f->ws.as<T2>();
  T2 const *Xt = X;
  int64_t ldxt = ldx;
  size_t ev = 0;
  auto mark = [&]() {
    if (events) ck(cudaEventRecord((*events)[ev++], s), "event");
  };
  mark();
  if (flags & BFG_APPLY_ORIGINAL_ORDER) {
    ck(f->xbuf.ensure((size_t)p.numCols * R * sizeof(T2)), "gather buffer");
    ck(bfg::launchGatherRows<T2>(X, ldx, f->srcPerm.as<int64_t>(), p.numCols, R,
                                 f->xbuf.as<T2>(), s),
       "gather");
    Xt = f->xbuf.as<T2>();
    ldxt = R;
    mark();
  }
  size_t const nStages = f->stageItem0.size() - 1;
  for (size_t st = 0; st < nStages; ++st) {
    int64_t a = f->stageItem0[st], b = f->stageItem0[st + 1];
    ck(bfg::launchApplyStage<T2>(f->items.as<bfg::ApplyItem>() + a, b - a,
                                 f->contribs.as<bfg::ApplyContrib>(), arena, Xt, ldxt, W, R, s),
       "apply stage");
    mark();
  }
  ck(bfg::launchApplyReduce<T2>(f->rowSeg.as<int32_t>(), f->segStart.as<int64_t>(),
                                f->segContrib0.as<int64_t>(), f->segBase.as<int64_t>(), W, R, Y,
                                ldy, p.numRows,
                                (flags & BFG_APPLY_ORIGINAL_ORDER) ? f->tgtPerm.as<int64_t>()
                                                                  : nullptr,
                                s),
     "apply reduce");
  mark();
}

int32_t tcTile(bfgFac_s::Tc const &tc, int64_t R);
bool isTcPrecision(bfgPrecision p);

// a tensor-core apply of more than one RHS tile copies its input tile-major
// first (the original-order gather does that on its way)
bool tcTiledCopy(bfgFac f, bfgPrecision prec, int64_t R, uint32_t flags) {
  return isTcPrecision(prec) && !(flags & BFG_APPLY_ORIGINAL_ORDER) &&
         R > tcTile(f->tc[prec == BFG_PRECISION_BF16X3 ? 1 : 0], R);
}

// launches of one device-operand apply: an input gather or copy, the
// stages, the final sum
size_t numApplyLaunches(bfgFac f, uint32_t flags, bfgPrecision prec, int64_t R) {
  bool const copy = (flags & BFG_APPLY_ORIGINAL_ORDER) || tcTiledCopy(f, prec, R, flags);
  return (f->stageItem0.size() - 1) + 1 + (copy ? 1 : 0);
}

void ensureArena32(bfgFac f) {
  if (f->arena32Ready) return;
  int64_t n = std::max<int64_t>(1, f->plan.arenaEntries);
  ck(f->arena32.ensure((size_t)n * sizeof(float2)), "FP32 arena");
  ck(bfg::launchArenaToF32(f->arena64.as<double2>(), f->arena32.as<float2>(), f->plan.arenaEntries,
                           f->ctx->stream),
     "FP32 arena");
  f->arena32Ready = true;
}

void ensureArenaDf(bfgFac f) {
  if (f->arenaDfReady) return;
  int64_t n = std::max<int64_t>(1, f->plan.arenaEntries);
  ck(f->arenaDf.ensure((size_t)n * sizeof(float4)), "double-float arena");
  ck(bfg::launchArenaToDf(f->arena64.as<double2>(), f->arenaDf.as<float4>(), f->plan.arenaEntries,
                          f->ctx->stream),
     "double-float arena");
  f->arenaDfReady = true;
}

// the double-float apply: input split (and gathered) into the X buffer,
// stages on double-float rows, final sum into complex128 Y.  Same launch
// count as runApply (the split stands in for its gather; without
// BFG_APPLY_ORIGINAL_ORDER it is timed with the first stage).
void runApplyDf(bfgFac f, double2 const *X, int64_t ldx, int64_t R, double2 *Y, int64_t ldy,
                uint32_t flags, std::vector<cudaEvent_t> *events) {
  cudaStream_t s = f->ctx->stream;
  bfg::ApplyProgram const &p = f->prog;
  ck(f->ws.ensure((size_t)std::max<int64_t>(1, p.wsRows) * R * sizeof(float4)), "workspace");
  ck(f->xbuf.ensure((size_t)std::max<int64_t>(1, p.numCols) * R * sizeof(float4)), "input buffer");
  float4 *W = f->ws.as<float4>(), *Xd = f->xbuf.as<float4>();
  size_t ev = 0;
  auto mark = [&]() {
    if (events) ck(cudaEventRecord((*events)[ev++], s), "event");
  };
  bool const orig = (flags & BFG_APPLY_ORIGINAL_ORDER) != 0;
  mark();
  ck(bfg::launchGatherToDf(X, ldx, orig ? f->srcPerm.as<int64_t>() : nullptr, p.numCols, R, Xd, s),
     "split X");
  if (orig) mark();
  size_t const nStages = f->stageItem0.size() - 1;
  for (size_t st = 0; st < nStages; ++st) {
    int64_t a = f->stageItem0[st], b = f->stageItem0[st + 1];
    ck(bfg::launchApplyStageDf(f->items.as<bfg::ApplyItem>() + a, b - a,
                               f->contribs.as<bfg::ApplyContrib>(), f->arenaDf.as<float4>(), Xd,
                               W, R, s),
       "apply stage");
    mark();
  }
  ck(bfg::launchApplyReduceDf(f->rowSeg.as<int32_t>(), f->segStart.as<int64_t>(),
                              f->segContrib0.as<int64_t>(), f->segBase.as<int64_t>(), W, R, Y,
                              ldy, p.numRows, orig ? f->tgtPerm.as<int64_t>() : nullptr, s),
     "apply reduce");
  mark();
}

void keepInputs(bfgFac f, double const *srcXy, double const *srcN, int64_t nSrc,
                double const *tgtXy, double const *tgtN, int64_t nTgt, double const *k,
                int64_t numProblems, int64_t const *srcOff, int64_t const *tgtOff) {
  f->inSrcXy.assign(srcXy, srcXy + 2 * nSrc);
  f->inTgtXy.assign(tgtXy, tgtXy + 2 * nTgt);
  if (srcN) f->inSrcN.assign(srcN, srcN + 2 * nSrc);
  if (tgtN) f->inTgtN.assign(tgtN, tgtN + 2 * nTgt);
  f->inK.assign(k, k + numProblems);
  if (srcOff) {
    f->inSrcOff.assign(srcOff, srcOff + numProblems + 1);
    f->inTgtOff.assign(tgtOff, tgtOff + numProblems + 1);
  }
}

bool isTcPrecision(bfgPrecision p) {
  return p == BFG_PRECISION_BF16X2 || p == BFG_PRECISION_BF16X3;
}

// Builds the tensor-core program, schedule and bf16 planes for `terms`
// planes (once per factorization and plane count).
void ensureTc(bfgFac f, int terms) {
  bfgFac_s::Tc &tc = f->tc[terms - 2];
  if (tc.ready) return;
  cudaStream_t s = f->ctx->stream;
  int32_t perSm = 0;
  ck(bfg::tcPrepare(terms, &perSm), "tensor-core apply");
  int sms = 0;
  ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, f->ctx->device), "device");
  if (perSm < 1) throw BfgError{BFG_ERROR_RUNTIME, "tensor-core apply: kernel does not fit an SM"};
  bfg::ApplyProgram &p128 = tc.p128;
  bfg::makeApplyProgram(f->plan, p128, bfg::kTcRows);
  if (p128.wsRows != f->prog.wsRows || p128.stageItem0.size() != f->stageItem0.size())
    throw BfgError{BFG_ERROR_RUNTIME, "tensor-core apply: program mismatch"};
  bfg::TcSchedule sc;
  bfg::makeTcSchedule(p128, terms, perSm * sms, sc);
  bfgFac_s::Tc::Sched &def = tc.sched[sc.ctas];
  upload(def.chunks, sc.chunks, s, "tensor-core schedule");
  upload(def.ctaChunk0, sc.ctaChunk0, s, "tensor-core schedule");
  DevBuf fills;
  upload(fills, sc.fills, s, "tensor-core schedule");
  ck(tc.arena.ensure((size_t)std::max<int64_t>(16, sc.arenaBytes)), "tensor-core factors");
  ck(bfg::launchTcFill(terms, fills.as<bfg::TcFill>(), (int64_t)sc.fills.size(),
                       f->arena64.as<double2>(), tc.arena.as<uint8_t>(), s),
     "tensor-core factors");
  if (!f->tcStatus.p) {
    ck(f->tcStatus.ensure(sizeof(int32_t)), "status");
    ck(cudaMemsetAsync(f->tcStatus.p, 0, sizeof(int32_t), s), "status");
  }
  ck(cudaStreamSynchronize(s), "tensor-core factors");
  tc.ctas = sc.ctas;
  tc.stages = p128.stageItem0.size() - 1;
  tc.ready = true;
}

// the tensor-core kernel's status word (synchronises); a bounded wait that
// ran out is reported as BFG_ERROR_TIMEOUT
void checkTcStatus(bfgFac f) {
  if (!f->tcStatus.p) return;
  int32_t st = 0;
  ck(cudaMemcpyAsync(&st, f->tcStatus.p, sizeof st, cudaMemcpyDeviceToHost, f->ctx->stream),
     "status");
  ck(cudaStreamSynchronize(f->ctx->stream), "status");
  if (st & bfg::kStatusTcTimeout) {
    cudaMemsetAsync(f->tcStatus.p, 0, sizeof(int32_t), f->ctx->stream);
    throw BfgError{BFG_ERROR_TIMEOUT, "tensor-core apply: a copy or MMA wait timed out"};
  }
}

// the RHS tile of an apply of R right-hand sides: the autotuner's choice
// for this R, else the default
int32_t tcTile(bfgFac_s::Tc const &tc, int64_t R) {
  auto const it = tc.rhsTile.find(R);
  return it != tc.rhsTile.end() ? it->second : bfg::tcRhsTile(R);
}

// chunk streams for R right-hand sides in tiles of rt: the resident CTAs
// shared out over the RHS tiles of every stream
int32_t tcStreams(bfgFac_s::Tc const &tc, int64_t R, int32_t rt) {
  int64_t const tiles = (R + rt - 1) / rt;
  return (int32_t)std::max<int64_t>(1, tc.ctas / std::max<int64_t>(1, tiles));
}

// the default dealing of the chunks to `streams` streams (built once)
bfgFac_s::Tc::Sched &tcSched(bfgFac f, int terms, int32_t streams) {
  bfgFac_s::Tc &tc = f->tc[terms - 2];
  auto it = tc.sched.find(streams);
  if (it != tc.sched.end()) return it->second;
  bfg::TcSchedule sc;
  bfg::makeTcSchedule(tc.p128, terms, streams, sc);
  bfgFac_s::Tc::Sched &d = tc.sched[streams];
  upload(d.chunks, sc.chunks, f->ctx->stream, "tensor-core schedule");
  upload(d.ctaChunk0, sc.ctaChunk0, f->ctx->stream, "tensor-core schedule");
  ck(cudaStreamSynchronize(f->ctx->stream), "tensor-core schedule");
  return d;
}

// xTiled > 0: X is already tile-major (tcInputTiling's layout: panel t of
// rt columns at X + t xTiled, leading dimension rt), as the host-operand
// applies convert it, so the first stage's full tiles arrive by bulk copies
// too; tree order only
void runApplyTc(bfgFac f, int terms, float2 const *X, int64_t ldx, int64_t R, float2 *Y,
                int64_t ldy, uint32_t flags, std::vector<cudaEvent_t> *events,
                int64_t xTiled = 0) {
  cudaStream_t s = f->ctx->stream;
  bfg::ApplyProgram const &p = f->prog;
  bfgFac_s::Tc &tc = f->tc[terms - 2];
  int32_t const rt = tcTile(tc, R);
  int32_t const streams = tcStreams(tc, R, rt);
  bfgFac_s::Tc::Sched &sched = tcSched(f, terms, streams);
  // With more than one RHS tile the workspace is tile-major (one panel of rt
  // columns per tile), so that every stage after the first brings a full
  // tile's input rows by one bulk copy; so is the gathered input of an
  // original-order apply.  One tile is row-major.
  int64_t const tiles = (R + rt - 1) / rt;
  bool const tiled = tiles > 1;
  int64_t const wsRows = std::max<int64_t>(1, p.wsRows);
  int64_t const ldw = tiled ? rt : R, wTs = tiled ? wsRows * rt : rt;
  ck(f->ws.ensure((size_t)wsRows * (tiled ? tiles * rt : R) * sizeof(float2)), "workspace");
  float2 *W = f->ws.as<float2>();
  float2 const *Xt = X;
  int64_t ldxt = ldx, xTs = rt;
  if (xTiled) {
    if (!tiled || (flags & BFG_APPLY_ORIGINAL_ORDER) || xTiled < p.numCols * rt)
      throw BfgError{BFG_ERROR_RUNTIME, "tensor-core apply: bad tile-major input"};
    ldxt = rt;
    xTs = xTiled;
  }
  size_t ev = 0;
  auto mark = [&]() {
    if (events) ck(cudaEventRecord((*events)[ev++], s), "event");
  };
  mark();
  if (tiled && !xTiled && !(flags & BFG_APPLY_ORIGINAL_ORDER)) {
    // the caller's row-major input copied tile-major, so that the first
    // stage too bulk-copies its input rows (one launch; the stage's
    // cp.async copies took 14 % more time than bulk copies)
    ck(f->xbuf.ensure((size_t)p.numCols * tiles * rt * sizeof(float2)), "input buffer");
    ck(bfg::launchGatherRows<float2>(X, ldx, nullptr, p.numCols, R, f->xbuf.as<float2>(), s, rt,
                                     p.numCols * rt),
       "tile-major input");
    Xt = f->xbuf.as<float2>();
    ldxt = rt;
    xTs = p.numCols * rt;
    mark();
  }
  if (flags & BFG_APPLY_ORIGINAL_ORDER) {
    ck(f->xbuf.ensure((size_t)p.numCols * (tiled ? tiles * rt : R) * sizeof(float2)),
       "gather buffer");
    ck(bfg::launchGatherRows<float2>(X, ldx, f->srcPerm.as<int64_t>(), p.numCols, R,
                                     f->xbuf.as<float2>(), s, tiled ? rt : 0,
                                     tiled ? p.numCols * rt : 0),
       "gather");
    Xt = f->xbuf.as<float2>();
    ldxt = tiled ? rt : R;
    xTs = tiled ? p.numCols * rt : rt;
    mark();
  }
  for (size_t st = 0; st < tc.stages; ++st) {
    ck(bfg::launchApplyTc(terms, rt, sched.chunks.as<bfg::TcChunk>(),
                          sched.ctaChunk0.as<int64_t>() + st * (size_t)(streams + 1), streams,
                          tc.arena.as<uint8_t>(), Xt, ldxt, xTs, W, ldw, wTs, R,
                          f->tcStatus.as<int32_t>(), s, f->tcWaitLimitNs),
       "tensor-core apply stage");
    mark();
  }
  ck(bfg::launchApplyReduce<float2>(f->rowSeg.as<int32_t>(), f->segStart.as<int64_t>(),
                                    f->segContrib0.as<int64_t>(), f->segBase.as<int64_t>(), W, R,
                                    Y, ldy, p.numRows,
                                    (flags & BFG_APPLY_ORIGINAL_ORDER) ? f->tgtPerm.as<int64_t>()
                                                                      : nullptr,
                                    s, tiled ? rt : 0, tiled ? wTs : 0),
     "apply reduce");
  mark();
}

// one-time preparation of a precision's copy of the factors
void preparePrecision(bfgFac f, bfgPrecision prec) {
  if (prec == BFG_PRECISION_FP32) ensureArena32(f);
  if (prec == BFG_PRECISION_DF64) ensureArenaDf(f);
  if (prec == BFG_PRECISION_BF16X2) ensureTc(f, 2);
  if (prec == BFG_PRECISION_BF16X3) ensureTc(f, 3);
}

bfgStatus applyDispatch(bfgFac f, bfgPrecision prec, void const *X, int64_t ldx, int64_t R,
                        void *Y, int64_t ldy, uint32_t flags, std::vector<cudaEvent_t> *ev) {
  if (!X || !Y || R < 1 || ldx < R || ldy < R)
    return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "apply: bad operand pointers or shapes");
  if (flags & ~BFG_APPLY_ORIGINAL_ORDER)
    return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "apply: unknown flags");
  if (prec == BFG_PRECISION_FP64) {
    runApply<double2>(f, f->arena64.as<double2>(), static_cast<double2 const *>(X), ldx, R,
                      static_cast<double2 *>(Y), ldy, flags, ev);
  } else if (prec == BFG_PRECISION_FP32) {
    ensureArena32(f);
    runApply<float2>(f, f->arena32.as<float2>(), static_cast<float2 const *>(X), ldx, R,
                     static_cast<float2 *>(Y), ldy, flags, ev);
  } else if (prec == BFG_PRECISION_DF64) {
    ensureArenaDf(f);
    runApplyDf(f, static_cast<double2 const *>(X), ldx, R, static_cast<double2 *>(Y), ldy, flags,
               ev);
  } else if (isTcPrecision(prec)) {
    int const terms = prec == BFG_PRECISION_BF16X3 ? 3 : 2;
    ensureTc(f, terms);
    runApplyTc(f, terms, static_cast<float2 const *>(X), ldx, R, static_cast<float2 *>(Y), ldy,
               flags, ev);
  } else {
    return fail(f->ctx, BFG_ERROR_NOT_IMPLEMENTED, "apply: unknown precision");
  }
  return BFG_OK;
}

// The host-operand applies convert their complex128 input to complex64 for
// the FP32 and tensor-core precisions.  A tensor-core apply of more than one
// RHS tile in tree order takes that input tile-major (panel t of rt columns
// at t x numCols x rt, leading dimension rt), so the conversion writes that
// layout and the first stage bulk-copies full tiles too.  Returns the panel
// stride, 0 for a row-major input; *rt the tile.
int64_t tcInputTiling(bfgFac f, bfgPrecision prec, int64_t R, uint32_t flags, int32_t *rt) {
  *rt = 0;
  if (!isTcPrecision(prec) || (flags & BFG_APPLY_ORIGINAL_ORDER)) return 0;
  *rt = tcTile(f->tc[prec == BFG_PRECISION_BF16X3 ? 1 : 0], R);
  return R > *rt ? f->prog.numCols * *rt : 0;
}

// the tensor-core apply of a tile-major input (tcInputTiling)
bfgStatus applyTcTiledInput(bfgFac f, bfgPrecision prec, float2 const *X, int64_t xTiled,
                            int64_t R, float2 *Y, int64_t ldy, uint32_t flags) {
  int const terms = prec == BFG_PRECISION_BF16X3 ? 3 : 2;
  ensureTc(f, terms);
  runApplyTc(f, terms, X, tcTile(f->tc[terms - 2], R), R, Y, ldy, flags, nullptr, xTiled);
  return BFG_OK;
}

}  // namespace

// Support of bfgFacApplyNoAlloc (bfg_noalloc.cu): the FP64 apply with a
// workspace the caller provides, so that nothing is allocated.
namespace bfg {

int64_t noAllocWorkspaceEntries(bfgFac f, int64_t R, uint32_t flags) {
  int64_t e = std::max<int64_t>(1, f->prog.wsRows) * R;
  if (flags & BFG_APPLY_ORIGINAL_ORDER) e += f->prog.numCols * R;
  return e;
}

int noAllocDevice(bfgFac f) { return f->ctx->device; }

bfgStatus noAllocFail(bfgFac f, bfgStatus st, char const *msg) { return fail(f->ctx, st, msg); }

bfgStatus noAllocApplyFp64(bfgFac f, double2 const *X, int64_t ldx, int64_t R, double2 *Y,
                           int64_t ldy, uint32_t flags, double2 *scratch) {
  return guarded(f->ctx, [&]() -> bfgStatus {
    cudaStream_t s = f->ctx->stream;
    bfg::ApplyProgram const &p = f->prog;
    double2 *W = scratch;
    double2 const *Xt = X;
    int64_t ldxt = ldx;
    if (flags & BFG_APPLY_ORIGINAL_ORDER) {
      double2 *xg = scratch + std::max<int64_t>(1, p.wsRows) * R;
      ck(bfg::launchGatherRows<double2>(X, ldx, f->srcPerm.as<int64_t>(), p.numCols, R, xg, s),
         "gather");
      Xt = xg;
      ldxt = R;
    }
    size_t const nStages = f->stageItem0.size() - 1;
    for (size_t st = 0; st < nStages; ++st) {
      int64_t a = f->stageItem0[st], b = f->stageItem0[st + 1];
      ck(bfg::launchApplyStage<double2>(f->items.as<bfg::ApplyItem>() + a, b - a,
                                        f->contribs.as<bfg::ApplyContrib>(),
                                        f->arena64.as<double2>(), Xt, ldxt, W, R, s),
         "apply stage");
    }
    ck(bfg::launchApplyReduce<double2>(
           f->rowSeg.as<int32_t>(), f->segStart.as<int64_t>(), f->segContrib0.as<int64_t>(),
           f->segBase.as<int64_t>(), W, R, Y, ldy, p.numRows,
           (flags & BFG_APPLY_ORIGINAL_ORDER) ? f->tgtPerm.as<int64_t>() : nullptr, s),
       "apply reduce");
    return BFG_OK;
  });
}

}  // namespace bfg

namespace {

// On-disk factorization: this header, then the wavenumbers (numProblems), the
// problem offsets (batched only, numProblems + 1 each), source xy, source
// normals (if any), target xy, target normals (if any), and the FP64 factor
// arena (arenaEntries complex128 values in plan order).  All little-endian,
// written as laid out in memory (the same layout on x86-64 and aarch64).
constexpr char kFacMagic[8] = {'B', 'F', 'G', 'F', 'A', 'C', '\0', '\1'};
constexpr uint32_t kFacVersion = 2;   // 2: bfgFacOptions with jacobiArith

struct FacFileHeader {
  char magic[8];
  uint32_t version, reserved;
  bfgHelm2 helm;
  bfgFacOptions opts;
  int64_t numProblems;
  int32_t batched, srcHasNormals, tgtHasNormals, reserved2;
  int64_t nSrc, nTgt, arenaEntries;
};
static_assert(sizeof(FacFileHeader) == 152, "file header layout");

constexpr int64_t kFileChunkEntries = int64_t(1) << 24;   // 256 MB of complex128

void writeAll(FILE *fp, void const *p, size_t n) {
  if (n && std::fwrite(p, 1, n, fp) != n) throw BfgError{BFG_ERROR_RUNTIME, "save: write failed"};
}
void readAll(FILE *fp, void *p, size_t n) {
  if (n && std::fread(p, 1, n, fp) != n)
    throw BfgError{BFG_ERROR_RUNTIME, "load: file truncated"};
}

}  // namespace

extern "C" {

bfgStatus bfgContextCreate(int32_t device, bfgContext *out) {
  if (!out) return BFG_ERROR_INVALID_ARGUMENTS;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return BFG_ERROR_CUDA;
  if (device < 0 || device >= count) return BFG_ERROR_INVALID_ARGUMENTS;
  auto *ctx = new (std::nothrow) bfgContext_s;
  if (!ctx) return BFG_ERROR_MEMORY;
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return BFG_ERROR_CUDA;
  }
  ctx->stream = ctx->own;
  *out = ctx;
  return BFG_OK;
}

bfgStatus bfgContextDestroy(bfgContext ctx) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  if (ctx->own) {
    cudaStreamSynchronize(ctx->own);
    cudaStreamDestroy(ctx->own);
  }
  delete ctx;
  return BFG_OK;
}

bfgStatus bfgContextSetStream(bfgContext ctx, void *stream) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return BFG_OK;
}

bfgStatus bfgContextGetStream(bfgContext ctx, void **stream) {
  if (!ctx || !stream) return BFG_ERROR_INVALID_ARGUMENTS;
  *stream = ctx->stream;
  return BFG_OK;
}

bfgStatus bfgContextSynchronize(bfgContext ctx) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fail(ctx, BFG_ERROR_CUDA, cudaGetErrorString(e));
  return BFG_OK;
}

char const *bfgGetErrorString(bfgContext ctx) {
  return ctx ? ctx->lastError.c_str() : "no context";
}

void bfgFacOptionsDefault(bfgFacOptions *o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->leafSize = 1;
  o->rankEps = 1e-15;
  o->pinvCut = 0;
  o->pinvTol = 0.0;
  o->sketch = 1;
}

bfgStatus bfgFacHelm2MakeMultilevel(bfgContext ctx, bfgHelm2 const *helm, double const *srcXy,
                                    double const *srcNormals, int64_t numSrc,
                                    double const *tgtXy, double const *tgtNormals,
                                    int64_t numTgt, bfgFacOptions const *opts, bfgFac *out) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(ctx, [&]() -> bfgStatus {
    if (!helm || !srcXy || !tgtXy || !out || numSrc < 1 || numTgt < 1)
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "make: null argument or empty point set");
    *out = nullptr;
    if (!(helm->k > 0) || !validLayerPot(helm->layerPot))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "make: k must be > 0 and the layer potential known");
    bool const needSrcN = helm->layerPot == bfg::kLpPvDouble ||
                          helm->layerPot == bfg::kLpCombinedField;
    bool const needTgtN = helm->layerPot == bfg::kLpPvNormalDerivSingle;
    if ((needSrcN && !srcNormals) || (needTgtN && !tgtNormals))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "make: this layer potential needs normals");
    bfgFacOptions o;
    bfgFacOptionsDefault(&o);
    if (opts) o = *opts;
    if (o.leafSize < 1 || !(o.rankEps > 0 && o.rankEps < 1) || (o.pinvCut != 0 && o.pinvCut != 1) || (o.jacobiArith != 0 && o.jacobiArith != 1) ||
        (o.sketch != 0 && o.sketch != 1) ||
        (o.jacobiArith == 1 && !(o.pinvCut == 1 && o.pinvTol >= kDfJacobiMinCut)) ||
        (o.pinvCut == 1 && !(o.pinvTol > 0 && o.pinvTol < 1)))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "make: bad options");
    for (int64_t i = 0; i < 2 * numSrc; ++i)
      if (!std::isfinite(srcXy[i])) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "make: non-finite source point");
    for (int64_t i = 0; i < 2 * numTgt; ++i)
      if (!std::isfinite(tgtXy[i])) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "make: non-finite target point");

    auto *f = new bfgFac_s;
    f->ctx = ctx;
    f->helm = *helm;
    f->opts = o;
    keepInputs(f, srcXy, srcNormals, numSrc, tgtXy, tgtNormals, numTgt, &helm->k, 1, nullptr,
               nullptr);
    try {
      bfg::PlanParams pp;
      pp.k = helm->k;
      pp.leafSize = o.leafSize;
      pp.rankEps = o.rankEps;
      if (o.treeOnGpu) {
        int64_t const so[2] = {0, numSrc}, to[2] = {0, numTgt};
        auto trees = gpuTrees(ctx->stream, srcXy, so, tgtXy, to, 1, o.leafSize);
        bfg::makePlan(f->plan, pp, srcXy, numSrc, tgtXy, numTgt, &trees[0], &trees[1]);
      } else {
        bfg::makePlan(f->plan, pp, srcXy, numSrc, tgtXy, numTgt);
      }
      cudaStream_t s = ctx->stream;
      f->srcHasNormals = srcNormals != nullptr;
      f->tgtHasNormals = tgtNormals != nullptr;
      uploadTreePoints(f->srcPts, srcXy, srcNormals, numSrc, f->plan.src.perm, s);
      uploadTreePoints(f->tgtPts, tgtXy, tgtNormals, numTgt, f->plan.tgt.perm, s);
      upload(f->srcPerm, f->plan.src.perm, s, "perm");
      upload(f->tgtPerm, f->plan.tgt.perm, s, "perm");
      factorize(f);
      buildApply(f);
      fillStats(f);
    } catch (std::runtime_error const &e) {
      delete f;
      return fail(ctx, BFG_ERROR_RUNTIME, std::string("make: ") + e.what());
    } catch (...) {
      delete f;
      throw;
    }
    *out = f;
    return BFG_OK;
  });
}

bfgStatus bfgFacHelm2MakeBatched(bfgContext ctx, bfgHelm2 const *helm, double const *k,
                                 int64_t numProblems, double const *srcXy,
                                 double const *srcNormals, int64_t const *srcOffsets,
                                 double const *tgtXy, double const *tgtNormals,
                                 int64_t const *tgtOffsets, bfgFacOptions const *opts,
                                 bfgFac *out) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(ctx, [&]() -> bfgStatus {
    if (!helm || !k || !srcXy || !tgtXy || !srcOffsets || !tgtOffsets || !out || numProblems < 1)
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: null argument");
    *out = nullptr;
    if (!validLayerPot(helm->layerPot))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: unknown layer potential");
    if (srcOffsets[0] != 0 || tgtOffsets[0] != 0)
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: offsets must start at 0");
    for (int64_t p = 0; p < numProblems; ++p) {
      if (!(k[p] > 0) || srcOffsets[p + 1] <= srcOffsets[p] || tgtOffsets[p + 1] <= tgtOffsets[p])
        return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS,
                    "batched make: every problem needs k > 0 and points");
    }
    bool const needSrcN = helm->layerPot == bfg::kLpPvDouble ||
                          helm->layerPot == bfg::kLpCombinedField;
    bool const needTgtN = helm->layerPot == bfg::kLpPvNormalDerivSingle;
    if ((needSrcN && !srcNormals) || (needTgtN && !tgtNormals))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: normals needed");
    int64_t const nSrc = srcOffsets[numProblems], nTgt = tgtOffsets[numProblems];
    for (int64_t i = 0; i < 2 * nSrc; ++i)
      if (!std::isfinite(srcXy[i])) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: non-finite point");
    for (int64_t i = 0; i < 2 * nTgt; ++i)
      if (!std::isfinite(tgtXy[i])) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: non-finite point");
    bfgFacOptions o;
    bfgFacOptionsDefault(&o);
    if (opts) o = *opts;
    if (o.leafSize < 1 || !(o.rankEps > 0 && o.rankEps < 1) || (o.pinvCut != 0 && o.pinvCut != 1) || (o.jacobiArith != 0 && o.jacobiArith != 1) ||
        (o.sketch != 0 && o.sketch != 1) ||
        (o.jacobiArith == 1 && !(o.pinvCut == 1 && o.pinvTol >= kDfJacobiMinCut)) ||
        (o.pinvCut == 1 && !(o.pinvTol > 0 && o.pinvTol < 1)))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "batched make: bad options");
    auto *f = new bfgFac_s;
    f->ctx = ctx;
    f->helm = *helm;
    f->helm.k = k[0];
    f->opts = o;
    keepInputs(f, srcXy, srcNormals, nSrc, tgtXy, tgtNormals, nTgt, k, numProblems, srcOffsets,
               tgtOffsets);
    try {
      bfg::PlanParams pp;
      pp.leafSize = o.leafSize;
      pp.rankEps = o.rankEps;
      if (o.treeOnGpu) {
        auto trees = gpuTrees(ctx->stream, srcXy, srcOffsets, tgtXy, tgtOffsets, numProblems,
                              o.leafSize);
        bfg::makePlanBatched(f->plan, pp, k, srcXy, srcOffsets, tgtXy, tgtOffsets, numProblems,
                             &trees);
      } else {
        bfg::makePlanBatched(f->plan, pp, k, srcXy, srcOffsets, tgtXy, tgtOffsets, numProblems);
      }
      cudaStream_t s = ctx->stream;
      f->srcHasNormals = srcNormals != nullptr;
      f->tgtHasNormals = tgtNormals != nullptr;
      uploadTreePoints(f->srcPts, srcXy, srcNormals, nSrc, f->plan.src.perm, s);
      uploadTreePoints(f->tgtPts, tgtXy, tgtNormals, nTgt, f->plan.tgt.perm, s);
      upload(f->srcPerm, f->plan.src.perm, s, "perm");
      upload(f->tgtPerm, f->plan.tgt.perm, s, "perm");
      factorize(f);
      buildApply(f);
      fillStats(f);
    } catch (std::runtime_error const &e) {
      delete f;
      return fail(ctx, BFG_ERROR_RUNTIME, std::string("batched make: ") + e.what());
    } catch (...) {
      delete f;
      throw;
    }
    *out = f;
    return BFG_OK;
  });
}

bfgStatus bfgFacSave(bfgFac f, char const *path) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    if (!path) return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "save: null path");
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(f->ctx, BFG_ERROR_RUNTIME, std::string("save: cannot open ") + path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard(fp, std::fclose);
    FacFileHeader h{};
    std::memcpy(h.magic, kFacMagic, sizeof h.magic);
    h.version = kFacVersion;
    h.helm = f->helm;
    h.opts = f->opts;
    h.numProblems = (int64_t)f->inK.size();
    h.batched = f->inSrcOff.empty() ? 0 : 1;
    h.srcHasNormals = f->inSrcN.empty() ? 0 : 1;
    h.tgtHasNormals = f->inTgtN.empty() ? 0 : 1;
    h.nSrc = (int64_t)f->inSrcXy.size() / 2;
    h.nTgt = (int64_t)f->inTgtXy.size() / 2;
    h.arenaEntries = f->plan.arenaEntries;
    writeAll(fp, &h, sizeof h);
    writeAll(fp, f->inK.data(), f->inK.size() * sizeof(double));
    if (h.batched) {
      writeAll(fp, f->inSrcOff.data(), f->inSrcOff.size() * sizeof(int64_t));
      writeAll(fp, f->inTgtOff.data(), f->inTgtOff.size() * sizeof(int64_t));
    }
    writeAll(fp, f->inSrcXy.data(), f->inSrcXy.size() * sizeof(double));
    writeAll(fp, f->inSrcN.data(), f->inSrcN.size() * sizeof(double));
    writeAll(fp, f->inTgtXy.data(), f->inTgtXy.size() * sizeof(double));
    writeAll(fp, f->inTgtN.data(), f->inTgtN.size() * sizeof(double));
    ck(cudaStreamSynchronize(f->ctx->stream), "save");
    std::vector<double2> buf((size_t)std::min(h.arenaEntries, kFileChunkEntries));
    for (int64_t off = 0; off < h.arenaEntries; off += kFileChunkEntries) {
      int64_t const n = std::min(kFileChunkEntries, h.arenaEntries - off);
      ck(cudaMemcpy(buf.data(), f->arena64.as<double2>() + off, (size_t)n * sizeof(double2),
                    cudaMemcpyDeviceToHost),
         "save");
      writeAll(fp, buf.data(), (size_t)n * sizeof(double2));
    }
    if (std::fclose(guard.release()) != 0)
      return fail(f->ctx, BFG_ERROR_RUNTIME, "save: write failed");
    return BFG_OK;
  });
}

bfgStatus bfgFacLoad(bfgContext ctx, char const *path, bfgFac *out) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(ctx, [&]() -> bfgStatus {
    if (!path || !out) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "load: null argument");
    *out = nullptr;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(ctx, BFG_ERROR_RUNTIME, std::string("load: cannot open ") + path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard(fp, std::fclose);
    FacFileHeader h{};
    readAll(fp, &h, sizeof h);
    if (std::memcmp(h.magic, kFacMagic, sizeof h.magic) != 0 || h.version != kFacVersion)
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "load: not a factorization file of this version");
    int64_t const kMaxPoints = int64_t(1) << 34;
    if (h.numProblems < 1 || h.nSrc < 1 || h.nTgt < 1 || h.nSrc > kMaxPoints ||
        h.nTgt > kMaxPoints || h.arenaEntries < 0 || (h.batched != 0 && h.batched != 1) ||
        (!h.batched && h.numProblems != 1) || h.numProblems > h.nSrc ||
        !validLayerPot(h.helm.layerPot))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "load: inconsistent header");
    auto *f = new bfgFac_s;
    f->ctx = ctx;
    f->helm = h.helm;
    f->opts = h.opts;
    try {
      f->inK.resize((size_t)h.numProblems);
      readAll(fp, f->inK.data(), f->inK.size() * sizeof(double));
      if (h.batched) {
        f->inSrcOff.resize((size_t)h.numProblems + 1);
        f->inTgtOff.resize((size_t)h.numProblems + 1);
        readAll(fp, f->inSrcOff.data(), f->inSrcOff.size() * sizeof(int64_t));
        readAll(fp, f->inTgtOff.data(), f->inTgtOff.size() * sizeof(int64_t));
        for (int64_t q = 0; q < h.numProblems; ++q)
          if (f->inSrcOff[(size_t)q + 1] <= f->inSrcOff[(size_t)q] ||
              f->inTgtOff[(size_t)q + 1] <= f->inTgtOff[(size_t)q])
            throw BfgError{BFG_ERROR_INVALID_ARGUMENTS, "load: bad problem offsets"};
        if (f->inSrcOff[0] != 0 || f->inTgtOff[0] != 0 ||
            f->inSrcOff[(size_t)h.numProblems] != h.nSrc ||
            f->inTgtOff[(size_t)h.numProblems] != h.nTgt)
          throw BfgError{BFG_ERROR_INVALID_ARGUMENTS, "load: bad problem offsets"};
      }
      for (double kk : f->inK)
        if (!(kk > 0)) throw BfgError{BFG_ERROR_INVALID_ARGUMENTS, "load: bad wavenumber"};
      f->inSrcXy.resize((size_t)(2 * h.nSrc));
      readAll(fp, f->inSrcXy.data(), f->inSrcXy.size() * sizeof(double));
      if (h.srcHasNormals) {
        f->inSrcN.resize((size_t)(2 * h.nSrc));
        readAll(fp, f->inSrcN.data(), f->inSrcN.size() * sizeof(double));
      }
      f->inTgtXy.resize((size_t)(2 * h.nTgt));
      readAll(fp, f->inTgtXy.data(), f->inTgtXy.size() * sizeof(double));
      if (h.tgtHasNormals) {
        f->inTgtN.resize((size_t)(2 * h.nTgt));
        readAll(fp, f->inTgtN.data(), f->inTgtN.size() * sizeof(double));
      }
      // the plan is a deterministic function of the inputs: rebuild it and
      // check it against the stored factors
      bfg::PlanParams pp;
      pp.leafSize = h.opts.leafSize;
      pp.rankEps = h.opts.rankEps;
      int64_t const so1[2] = {0, h.nSrc}, to1[2] = {0, h.nTgt};
      int64_t const *so = h.batched ? f->inSrcOff.data() : so1;
      int64_t const *to = h.batched ? f->inTgtOff.data() : to1;
      int64_t const np = h.batched ? h.numProblems : 1;
      std::vector<bfg::Quadtree> trees;
      if (h.opts.treeOnGpu)
        trees = gpuTrees(ctx->stream, f->inSrcXy.data(), so, f->inTgtXy.data(), to, np,
                         h.opts.leafSize);
      if (h.batched) {
        bfg::makePlanBatched(f->plan, pp, f->inK.data(), f->inSrcXy.data(), f->inSrcOff.data(),
                             f->inTgtXy.data(), f->inTgtOff.data(), h.numProblems,
                             trees.empty() ? nullptr : &trees);
      } else {
        pp.k = f->inK[0];
        bfg::makePlan(f->plan, pp, f->inSrcXy.data(), h.nSrc, f->inTgtXy.data(), h.nTgt,
                      trees.empty() ? nullptr : &trees[0], trees.empty() ? nullptr : &trees[1]);
      }
      if (f->plan.arenaEntries != h.arenaEntries)
        throw BfgError{BFG_ERROR_INVALID_ARGUMENTS,
                       "load: the stored factors do not match the plan of the stored inputs"};
      cudaStream_t s = ctx->stream;
      f->srcHasNormals = h.srcHasNormals != 0;
      f->tgtHasNormals = h.tgtHasNormals != 0;
      uploadTreePoints(f->srcPts, f->inSrcXy.data(), h.srcHasNormals ? f->inSrcN.data() : nullptr,
                       h.nSrc, f->plan.src.perm, s);
      uploadTreePoints(f->tgtPts, f->inTgtXy.data(), h.tgtHasNormals ? f->inTgtN.data() : nullptr,
                       h.nTgt, f->plan.tgt.perm, s);
      upload(f->srcPerm, f->plan.src.perm, s, "perm");
      upload(f->tgtPerm, f->plan.tgt.perm, s, "perm");
      ck(cudaStreamSynchronize(s), "load");
      ck(f->arena64.ensure((size_t)std::max<int64_t>(1, h.arenaEntries) * sizeof(double2)),
         "arena");
      std::vector<double2> buf((size_t)std::min(h.arenaEntries, kFileChunkEntries));
      for (int64_t off = 0; off < h.arenaEntries; off += kFileChunkEntries) {
        int64_t const n = std::min(kFileChunkEntries, h.arenaEntries - off);
        readAll(fp, buf.data(), (size_t)n * sizeof(double2));
        ck(cudaMemcpy(f->arena64.as<double2>() + off, buf.data(), (size_t)n * sizeof(double2),
                      cudaMemcpyHostToDevice),
           "load");
      }
      int64_t maxRank = 0;
      for (auto const &b : f->plan.blocks) {
        if (b.kind == bfg::kLast) maxRank = std::max<int64_t>(maxRank, b.n);
        if (b.kind == bfg::kFirst || b.kind == bfg::kMiddle) maxRank = std::max<int64_t>(maxRank, b.m);
      }
      f->stats.maxRank = maxRank;
      buildApply(f);
      fillStats(f);
    } catch (std::runtime_error const &e) {
      delete f;
      return fail(ctx, BFG_ERROR_RUNTIME, std::string("load: ") + e.what());
    } catch (...) {
      delete f;
      throw;
    }
    *out = f;
    return BFG_OK;
  });
}

bfgStatus bfgFacDestroy(bfgFac f) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  cudaStreamSynchronize(f->ctx->stream);
  delete f;
  return BFG_OK;
}

bfgStatus bfgFacGetShape(bfgFac f, int64_t *rows, int64_t *cols) {
  if (!f || !rows || !cols) return BFG_ERROR_INVALID_ARGUMENTS;
  *rows = (int64_t)f->plan.tgt.perm.size();
  *cols = (int64_t)f->plan.src.perm.size();
  return BFG_OK;
}

bfgStatus bfgFacGetPerms(bfgFac f, int64_t *srcPerm, int64_t *tgtPerm) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  if (srcPerm) std::copy(f->plan.src.perm.begin(), f->plan.src.perm.end(), srcPerm);
  if (tgtPerm) std::copy(f->plan.tgt.perm.begin(), f->plan.tgt.perm.end(), tgtPerm);
  return BFG_OK;
}

bfgStatus bfgFacNumBytes(bfgFac f, int64_t *bytes) {
  if (!f || !bytes) return BFG_ERROR_INVALID_ARGUMENTS;
  *bytes = f->plan.arenaEntries * 16;
  return BFG_OK;
}

bfgStatus bfgFacGetStats(bfgFac f, bfgFacStats *st) {
  if (!f || !st) return BFG_ERROR_INVALID_ARGUMENTS;
  *st = f->stats;
  st->applyBufferBytes = (int64_t)(f->ws.bytes + f->xbuf.bytes);
  return BFG_OK;
}

bfgStatus bfgFacDescribe(bfgFac f, char *buf, int64_t cap, int64_t *len) {
  if (!f || !len) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    std::string t = f->plan.text();
    *len = (int64_t)t.size();
    if (buf && cap > 0) {
      int64_t n = std::min<int64_t>(cap - 1, (int64_t)t.size());
      std::memcpy(buf, t.data(), (size_t)n);
      buf[n] = 0;
      if (cap <= (int64_t)t.size()) return fail(f->ctx, BFG_ERROR_OUT_OF_RANGE, "describe: buffer too small");
    }
    return BFG_OK;
  });
}

bfgStatus bfgFacCopyBlocks(bfgFac f, double *entries, int64_t capEntries, int64_t *table,
                           int64_t capBlocks) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    if (entries) {
      if (capEntries < f->plan.arenaEntries)
        return fail(f->ctx, BFG_ERROR_OUT_OF_RANGE, "copy blocks: entry buffer too small");
      ck(cudaStreamSynchronize(f->ctx->stream), "sync");
      ck(cudaMemcpy(entries, f->arena64.p, (size_t)f->plan.arenaEntries * 16, cudaMemcpyDeviceToHost),
         "copy blocks");
    }
    if (table) {
      if (capBlocks < (int64_t)f->plan.blocks.size())
        return fail(f->ctx, BFG_ERROR_OUT_OF_RANGE, "copy blocks: table too small");
      for (size_t i = 0; i < f->plan.blockOrder.size(); ++i) {
        auto const &b = f->plan.blocks[f->plan.blockOrder[i]];
        table[4 * i] = b.kind;
        table[4 * i + 1] = b.m;
        table[4 * i + 2] = b.n;
        table[4 * i + 3] = b.arenaOff;
      }
    }
    return BFG_OK;
  });
}

bfgStatus bfgFacSynchronize(bfgFac f) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    ck(cudaStreamSynchronize(f->ctx->stream), "synchronize");
    checkTcStatus(f);
    return BFG_OK;
  });
}

bfgStatus bfgFacApply(bfgFac f, bfgPrecision prec, void const *X, int64_t ldx, int64_t R,
                      void *Y, int64_t ldy, uint32_t flags) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() { return applyDispatch(f, prec, X, ldx, R, Y, ldy, flags, nullptr); });
}

bfgStatus bfgFacApplyTimed(bfgFac f, bfgPrecision prec, void const *X, int64_t ldx, int64_t R,
                           void *Y, int64_t ldy, uint32_t flags, float *ms, int32_t cap,
                           int32_t *numLaunches) {
  if (!f || !numLaunches) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    size_t const n = numApplyLaunches(f, flags, prec, R);
    *numLaunches = (int32_t)n;
    if (!ms || cap < (int32_t)n) return fail(f->ctx, BFG_ERROR_OUT_OF_RANGE, "timed apply: buffer too small");
    preparePrecision(f, prec);
    Events ev(n + 1, "event");
    bfgStatus st = applyDispatch(f, prec, X, ldx, R, Y, ldy, flags, &ev.v);
    if (st == BFG_OK) {
      ck(cudaEventSynchronize(ev[n]), "event");
      for (size_t i = 0; i < n; ++i) cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
    }
    if (st == BFG_OK && isTcPrecision(prec)) checkTcStatus(f);
    return st;
  });
}

bfgStatus bfgFacGetApplyLaunches(bfgFac f, bfgPrecision prec, int64_t R, uint32_t flags,
                                 int64_t *info, int32_t cap, int32_t *numLaunches) {
  if (!f || !numLaunches || R < 1) return BFG_ERROR_INVALID_ARGUMENTS;
  if (prec < BFG_PRECISION_FP64 || prec > BFG_PRECISION_DF64)
    return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "launch info: unknown precision");
  size_t const n = numApplyLaunches(f, flags, prec, R);
  *numLaunches = (int32_t)n;
  if (!info || cap < (int32_t)n) return fail(f->ctx, BFG_ERROR_OUT_OF_RANGE, "launch info: buffer too small");
  bfg::ApplyProgram const &p = f->prog;
  size_t k = 0;
  if ((flags & BFG_APPLY_ORIGINAL_ORDER) || tcTiledCopy(f, prec, R, flags)) {
    info[3 * k] = 0;
    info[3 * k + 1] = p.numCols;
    info[3 * k + 2] = p.numCols;
    ++k;
  }
  for (size_t s = 0; s + 1 < f->stageItem0.size(); ++s, ++k) {
    info[3 * k] = p.stageEntries[s];
    info[3 * k + 1] = p.stageRowsIn[s];
    info[3 * k + 2] = p.stageRowsOut[s];
  }
  info[3 * k] = 0;
  info[3 * k + 1] = p.sumRows;
  info[3 * k + 2] = p.numRows;
  return BFG_OK;
}

bfgStatus bfgFacGetLaunchInfo(bfgFac f, uint32_t flags, int64_t *info, int32_t cap,
                              int32_t *numLaunches) {
  return bfgFacGetApplyLaunches(f, BFG_PRECISION_FP64, 1, flags, info, cap, numLaunches);
}

bfgStatus bfgFacApplyHost(bfgFac f, bfgPrecision prec, double const *X, int64_t ldx, int64_t R,
                          double *Y, int64_t ldy, uint32_t flags) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    if (!X || !Y || R < 1 || ldx < R || ldy < R)
      return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "apply: bad operand pointers or shapes");
    cudaStream_t s = f->ctx->stream;
    int64_t const nr = f->prog.numRows, nc = f->prog.numCols;
    // complex128 staging on the device (the host operands are complex128
    // whatever the arithmetic); the buffers persist across calls
    ck(f->hx128.ensure((size_t)nc * R * 16), "apply buffers");
    ck(f->hy128.ensure((size_t)nr * R * 16), "apply buffers");
    // one contiguous copy when the rows are back to back (a 2D copy of
    // 256-byte rows moves them one by one)
    if (ldx == R)
      ck(cudaMemcpyAsync(f->hx128.p, X, (size_t)nc * R * 16, cudaMemcpyHostToDevice, s), "copy X");
    else
      ck(cudaMemcpy2DAsync(f->hx128.p, (size_t)R * 16, X, (size_t)ldx * 16, (size_t)R * 16,
                           (size_t)nc, cudaMemcpyHostToDevice, s),
         "copy X");
    if (prec == BFG_PRECISION_FP64 || prec == BFG_PRECISION_DF64) {
      bfgStatus st = applyDispatch(f, prec, f->hx128.p, R, R, f->hy128.p, R, flags, nullptr);
      if (st != BFG_OK) return st;
    } else if (prec == BFG_PRECISION_FP32 || isTcPrecision(prec)) {
      int32_t rt = 0;
      int64_t const xTiled = tcInputTiling(f, prec, R, flags, &rt);
      ck(f->hx64.ensure((size_t)nc * (xTiled ? (R + rt - 1) / rt * rt : R) * 8), "apply buffers");
      ck(f->hy64.ensure((size_t)nr * R * 8), "apply buffers");
      ck(bfg::launchC128ToC64(f->hx128.as<double2>(), R, nc, R, f->hx64.as<float2>(), R, s,
                              xTiled ? rt : 0, xTiled),
         "convert X");
      bfgStatus st =
          xTiled ? applyTcTiledInput(f, prec, f->hx64.as<float2>(), xTiled, R, f->hy64.as<float2>(),
                                     R, flags)
                 : applyDispatch(f, prec, f->hx64.p, R, R, f->hy64.p, R, flags, nullptr);
      if (st != BFG_OK) return st;
      ck(bfg::launchC64ToC128(f->hy64.as<float2>(), R, nr, R, f->hy128.as<double2>(), R, s),
         "convert Y");
    } else {
      return fail(f->ctx, BFG_ERROR_NOT_IMPLEMENTED, "apply: unknown precision");
    }
    if (ldy == R)
      ck(cudaMemcpyAsync(Y, f->hy128.p, (size_t)nr * R * 16, cudaMemcpyDeviceToHost, s), "copy Y");
    else
      ck(cudaMemcpy2DAsync(Y, (size_t)ldy * 16, f->hy128.p, (size_t)R * 16, (size_t)R * 16,
                           (size_t)nr, cudaMemcpyDeviceToHost, s),
         "copy Y");
    ck(cudaStreamSynchronize(s), "apply");
    if (isTcPrecision(prec)) checkTcStatus(f);
    return BFG_OK;
  });
}

bfgStatus bfgFacSetTcWaitLimit(bfgFac f, uint64_t waitLimitNs) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  f->tcWaitLimitNs = waitLimitNs;
  return BFG_OK;
}

bfgStatus bfgFacAutotune(bfgFac f, bfgPrecision prec, int64_t R, double *stageMs,
                         int32_t capacity, int32_t *numStages) {
  if (!f || R < 1 || (capacity > 0 && !stageMs)) return BFG_ERROR_INVALID_ARGUMENTS;
  if (!isTcPrecision(prec))
    return fail(f->ctx, BFG_ERROR_NOT_IMPLEMENTED,
                "autotune: the tuned schedule is the tensor-core apply's (BF16X2, BF16X3)");
  return guarded(f->ctx, [&]() -> bfgStatus {
    int const terms = prec == BFG_PRECISION_BF16X3 ? 3 : 2;
    ensureTc(f, terms);
    bfgFac_s::Tc &tc = f->tc[terms - 2];
    cudaStream_t s = f->ctx->stream;
    bfg::ApplyProgram const &p128 = tc.p128;
    size_t const nStages = tc.stages;
    std::vector<bfg::TcCostModel> const models = bfg::tcCandidateModels();   // default first
    size_t const K = models.size();
    // both RHS tile widths, the default first; per width its own stream count
    int32_t const widths[2] = {bfg::tcRhsTile(R), bfg::tcRhsTile(R) == 16 ? 32 : 16};
    struct Width {
      int32_t rt = 0, ctas = 0;
      std::vector<bfg::TcSchedule> cands;
      std::vector<std::vector<float>> best;   // [model][stage] ms
    } wd[2];
    for (int w = 0; w < 2; ++w) {
      wd[w].rt = widths[w];
      wd[w].ctas = tcStreams(tc, R, widths[w]);
      wd[w].cands.resize(K);
      for (size_t k = 0; k < K; ++k) {
        bfg::makeTcSchedule(p128, terms, wd[w].ctas, wd[w].cands[k], models[k]);
        if (wd[w].cands[k].arenaBytes != wd[0].cands[0].arenaBytes)
          throw BfgError{BFG_ERROR_RUNTIME, "autotune: schedules disagree on the tiles"};
      }
      wd[w].best.assign(K, std::vector<float>(nStages, 1e30f));
    }
    // scratch operands: the times do not depend on the values; input and
    // workspace laid out as the apply lays them out (tile-major with more
    // than one tile)
    bfg::ApplyProgram const &p = f->prog;
    int64_t const wsRows = std::max<int64_t>(1, p.wsRows);
    int64_t const cols32 = (R + 31) / 32 * 32;   // room for either tiling
    DevBuf xs;
    ck(xs.ensure((size_t)std::max<int64_t>(1, p.numCols) * cols32 * sizeof(float2)), "autotune");
    ck(cudaMemsetAsync(xs.p, 0, (size_t)p.numCols * cols32 * sizeof(float2), s), "autotune");
    ck(f->ws.ensure((size_t)wsRows * cols32 * sizeof(float2)), "workspace");
    Events const ev(nStages + 1, "autotune");
    int const reps = 5;
    DevBuf dch, dc0;
    for (Width &w : wd)
      for (size_t k = 0; k < K; ++k) {
        upload(dch, w.cands[k].chunks, s, "autotune");
        upload(dc0, w.cands[k].ctaChunk0, s, "autotune");
        for (int rep = 0; rep < reps + 1; ++rep) {
          ck(cudaEventRecord(ev[0], s), "autotune");
          for (size_t st = 0; st < nStages; ++st) {
            bool const tiled = R > w.rt;
            ck(bfg::launchApplyTc(terms, w.rt, dch.as<bfg::TcChunk>(),
                                  dc0.as<int64_t>() + st * (size_t)(w.ctas + 1), w.ctas,
                                  tc.arena.as<uint8_t>(), xs.as<float2>(), tiled ? w.rt : R,
                                  tiled ? p.numCols * w.rt : w.rt, f->ws.as<float2>(),
                                  tiled ? w.rt : R, tiled ? wsRows * w.rt : w.rt, R,
                                  f->tcStatus.as<int32_t>(), s),
               "autotune");
            ck(cudaEventRecord(ev[st + 1], s), "autotune");
          }
          ck(cudaStreamSynchronize(s), "autotune");
          if (rep == 0) continue;   // warm-up
          for (size_t st = 0; st < nStages; ++st) {
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, ev[st], ev[st + 1]), "autotune");
            w.best[k][st] = std::min(w.best[k][st], ms);
          }
        }
      }
    checkTcStatus(f);
    // per width and stage the fastest model; the width with the smaller sum
    // of those (the default on a tie)
    std::vector<size_t> pick[2];
    double total[2] = {0, 0};
    for (int w = 0; w < 2; ++w)
      for (size_t st = 0; st < nStages; ++st) {
        size_t kb = 0;
        for (size_t k = 1; k < K; ++k)
          if (wd[w].best[k][st] < wd[w].best[kb][st]) kb = k;
        pick[w].push_back(kb);
        total[w] += wd[w].best[kb][st];
      }
    int const wb = total[1] < total[0] ? 1 : 0;
    Width const &win = wd[wb];
    // the chosen width's per-stage schedules, spliced into one
    std::vector<bfg::TcChunk> chunks;
    std::vector<int64_t> c0;
    for (size_t st = 0; st < nStages; ++st) {
      bfg::TcSchedule const &c = win.cands[pick[wb][st]];
      int64_t const a = c.ctaChunk0[st * (size_t)(win.ctas + 1)];
      int64_t const b = c.ctaChunk0[st * (size_t)(win.ctas + 1) + win.ctas];
      int64_t const base = (int64_t)chunks.size();
      for (int32_t q = 0; q <= win.ctas; ++q)
        c0.push_back(c.ctaChunk0[st * (size_t)(win.ctas + 1) + q] - a + base);
      chunks.insert(chunks.end(), c.chunks.begin() + a, c.chunks.begin() + b);
      if ((int64_t)(2 * st + 1) < capacity) {
        stageMs[2 * st] = wd[0].best[0][st];
        stageMs[2 * st + 1] = win.best[pick[wb][st]][st];
      }
    }
    if (numStages) *numStages = (int32_t)nStages;
    bfgFac_s::Tc::Sched &tuned = tc.sched[win.ctas];
    upload(tuned.chunks, chunks, s, "tensor-core schedule");
    upload(tuned.ctaChunk0, c0, s, "tensor-core schedule");
    ck(cudaStreamSynchronize(s), "tensor-core schedule");
    tc.rhsTile[R] = win.rt;
    return BFG_OK;
  });
}

bfgStatus bfgFacGetRhsTile(bfgFac f, bfgPrecision prec, int64_t R, int32_t *rhsTile) {
  if (!f || R < 1 || !rhsTile) return BFG_ERROR_INVALID_ARGUMENTS;
  if (!isTcPrecision(prec))
    return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "RHS tile: a tensor-core precision only");
  *rhsTile = tcTile(f->tc[prec == BFG_PRECISION_BF16X3 ? 1 : 0], R);
  return BFG_OK;
}

bfgStatus bfgFacPrepare(bfgFac f, bfgPrecision prec) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  if (prec < BFG_PRECISION_FP64 || prec > BFG_PRECISION_DF64)
    return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "prepare: unknown precision");
  return guarded(f->ctx, [&]() -> bfgStatus {
    preparePrecision(f, prec);
    ck(cudaStreamSynchronize(f->ctx->stream), "prepare");
    return BFG_OK;
  });
}

bfgStatus bfgFacApplyHostAsync(bfgFac f, bfgPrecision prec, double const *X, int64_t ldx,
                               int64_t R, double *Y, int64_t ldy, uint32_t flags) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    if (!X || !Y || R < 1 || ldx < R || ldy < R)
      return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "apply: bad operand pointers or shapes");
    bool const c128 = prec == BFG_PRECISION_FP64 || prec == BFG_PRECISION_DF64;
    if (!c128 && prec != BFG_PRECISION_FP32 && !isTcPrecision(prec))
      return fail(f->ctx, BFG_ERROR_NOT_IMPLEMENTED, "apply: unknown precision");
    preparePrecision(f, prec);
    if (!f->upStream) {
      ck(cudaStreamCreateWithFlags(&f->upStream, cudaStreamNonBlocking), "copy streams");
      ck(cudaStreamCreateWithFlags(&f->downStream, cudaStreamNonBlocking), "copy streams");
      for (auto &h : f->hslot)
        for (cudaEvent_t *e : {&h.uploaded, &h.consumed, &h.computed, &h.downloaded})
          ck(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "copy events");
    }
    cudaStream_t const cs = f->ctx->stream, up = f->upStream, down = f->downStream;
    int64_t const nr = f->prog.numRows, nc = f->prog.numCols;
    auto &h = f->hslot[f->asyncCalls & 1];
    int32_t rt = 0;
    int64_t const xTiled = tcInputTiling(f, prec, R, flags, &rt);
    ck(h.x128.ensure((size_t)nc * R * 16), "apply buffers");
    ck(h.y128.ensure((size_t)nr * R * 16), "apply buffers");
    if (!c128) {
      ck(h.x64.ensure((size_t)nc * (xTiled ? (R + rt - 1) / rt * rt : R) * 8), "apply buffers");
      ck(h.y64.ensure((size_t)nr * R * 8), "apply buffers");
    }
    // upload, once the compute of this slot's previous call has read it
    if (h.started) ck(cudaStreamWaitEvent(up, h.consumed, 0), "order");
    if (ldx == R)
      ck(cudaMemcpyAsync(h.x128.p, X, (size_t)nc * R * 16, cudaMemcpyHostToDevice, up), "copy X");
    else
      ck(cudaMemcpy2DAsync(h.x128.p, (size_t)R * 16, X, (size_t)ldx * 16, (size_t)R * 16,
                           (size_t)nc, cudaMemcpyHostToDevice, up),
         "copy X");
    ck(cudaEventRecord(h.uploaded, up), "order");
    // compute, once the upload landed and the slot's previous download left
    ck(cudaStreamWaitEvent(cs, h.uploaded, 0), "order");
    if (h.started) ck(cudaStreamWaitEvent(cs, h.downloaded, 0), "order");
    if (c128) {
      bfgStatus st = applyDispatch(f, prec, h.x128.p, R, R, h.y128.p, R, flags, nullptr);
      if (st != BFG_OK) return st;
      ck(cudaEventRecord(h.consumed, cs), "order");
    } else {
      ck(bfg::launchC128ToC64(h.x128.as<double2>(), R, nc, R, h.x64.as<float2>(), R, cs,
                              xTiled ? rt : 0, xTiled),
         "convert X");
      ck(cudaEventRecord(h.consumed, cs), "order");
      bfgStatus st =
          xTiled ? applyTcTiledInput(f, prec, h.x64.as<float2>(), xTiled, R, h.y64.as<float2>(), R,
                                     flags)
                 : applyDispatch(f, prec, h.x64.p, R, R, h.y64.p, R, flags, nullptr);
      if (st != BFG_OK) return st;
      ck(bfg::launchC64ToC128(h.y64.as<float2>(), R, nr, R, h.y128.as<double2>(), R, cs),
         "convert Y");
    }
    ck(cudaEventRecord(h.computed, cs), "order");
    // download
    ck(cudaStreamWaitEvent(down, h.computed, 0), "order");
    if (ldy == R)
      ck(cudaMemcpyAsync(Y, h.y128.p, (size_t)nr * R * 16, cudaMemcpyDeviceToHost, down), "copy Y");
    else
      ck(cudaMemcpy2DAsync(Y, (size_t)ldy * 16, h.y128.p, (size_t)R * 16, (size_t)R * 16,
                           (size_t)nr, cudaMemcpyDeviceToHost, down),
         "copy Y");
    ck(cudaEventRecord(h.downloaded, down), "order");
    h.started = true;
    ++f->asyncCalls;
    return BFG_OK;
  });
}

bfgStatus bfgFacApplyHostWait(bfgFac f) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    if (f->upStream) {
      ck(cudaStreamSynchronize(f->upStream), "apply");
      ck(cudaStreamSynchronize(f->downStream), "apply");
    }
    ck(cudaStreamSynchronize(f->ctx->stream), "apply");
    checkTcStatus(f);
    return BFG_OK;
  });
}

bfgStatus bfgFacDenseRows(bfgFac f, int64_t const *rows, int64_t nSel, void const *X, int64_t ldx,
                          int64_t R, void *out, int64_t ldo) {
  if (!f) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(f->ctx, [&]() -> bfgStatus {
    if (!rows || !X || !out || nSel < 0 || R < 1 || ldx < R || ldo < R)
      return fail(f->ctx, BFG_ERROR_INVALID_ARGUMENTS, "dense rows: bad arguments");
    int64_t const nr = f->prog.numRows, nc = f->prog.numCols;
    std::vector<int64_t> r(rows, rows + nSel);
    for (int64_t v : r)
      if (v < 0 || v >= nr) return fail(f->ctx, BFG_ERROR_OUT_OF_RANGE, "dense rows: row out of range");
    DevBuf dr;
    upload(dr, r, f->ctx->stream, "rows");
    bfg::KernelParams kp = kernelParams(f->helm, f->helm.layerPot);
    ck(bfg::launchDenseRows(pointsView(f->srcPts, nc, f->srcHasNormals), nc,
                            pointsView(f->tgtPts, nr, f->tgtHasNormals), dr.as<int64_t>(), nSel,
                            kp, static_cast<double2 const *>(X), ldx, R,
                            static_cast<double2 *>(out), ldo, f->ctx->stream),
       "dense rows");
    ck(cudaStreamSynchronize(f->ctx->stream), "dense rows");
    return BFG_OK;
  });
}

bfgStatus bfgHelm2KernelMatrix(bfgContext ctx, bfgHelm2 const *helm, double const *srcXy,
                               double const *srcNormals, int64_t n, double const *tgtXy,
                               double const *tgtNormals, int64_t m, double *out) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(ctx, [&]() -> bfgStatus {
    if (!helm || !srcXy || !tgtXy || !out || n < 0 || m < 0 || !validLayerPot(helm->layerPot))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "kernel matrix: bad arguments");
    bool const needSrcN = helm->layerPot == bfg::kLpPvDouble ||
                          helm->layerPot == bfg::kLpCombinedField;
    bool const needTgtN = helm->layerPot == bfg::kLpPvNormalDerivSingle;
    if ((needSrcN && !srcNormals) || (needTgtN && !tgtNormals))
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "kernel matrix: normals needed");
    cudaStream_t s = ctx->stream;
    std::vector<int64_t> idS(n), idT(m);
    for (int64_t i = 0; i < n; ++i) idS[i] = i;
    for (int64_t i = 0; i < m; ++i) idT[i] = i;
    DevBuf ds, dt, dout;
    uploadTreePoints(ds, srcXy, srcNormals, n, idS, s);
    uploadTreePoints(dt, tgtXy, tgtNormals, m, idT, s);
    ck(dout.ensure((size_t)std::max<int64_t>(1, m * n) * 16), "kernel matrix");
    ck(bfg::launchKernelMatrix(pointsView(ds, n, srcNormals != nullptr), n,
                               pointsView(dt, m, tgtNormals != nullptr), m,
                               kernelParams(*helm, helm->layerPot), dout.as<double2>(), s),
       "kernel matrix");
    ck(cudaMemcpyAsync(out, dout.p, (size_t)m * n * 16, cudaMemcpyDeviceToHost, s), "kernel matrix");
    ck(cudaStreamSynchronize(s), "kernel matrix");
    return BFG_OK;
  });
}

bfgStatus bfgBessel01(bfgContext ctx, double const *x, int64_t n, double *out) {
  if (!ctx) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(ctx, [&]() -> bfgStatus {
    if (!x || !out || n < 0) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "bessel: bad arguments");
    for (int64_t i = 0; i < n; ++i)
      if (!(x[i] > 0) || !std::isfinite(x[i]))
        return fail(ctx, BFG_ERROR_OUT_OF_RANGE, "bessel: arguments must be finite and > 0");
    cudaStream_t s = ctx->stream;
    DevBuf dx, dout;
    ck(dx.ensure((size_t)std::max<int64_t>(1, n) * 8), "bessel");
    ck(dout.ensure((size_t)std::max<int64_t>(1, n) * 32), "bessel");
    ck(cudaMemcpyAsync(dx.p, x, (size_t)n * 8, cudaMemcpyHostToDevice, s), "bessel");
    ck(bfg::launchBessel01(dx.as<double>(), n, dout.as<double>(), s), "bessel");
    ck(cudaMemcpyAsync(out, dout.p, (size_t)n * 32, cudaMemcpyDeviceToHost, s), "bessel");
    ck(cudaStreamSynchronize(s), "bessel");
    return BFG_OK;
  });
}

bfgStatus bfgMeasureFp64Rate(bfgContext ctx, double *tflops) {
  if (!ctx || !tflops) return BFG_ERROR_INVALID_ARGUMENTS;
  return guarded(ctx, [&]() -> bfgStatus {
    cudaStream_t s = ctx->stream;
    int sms = 0;
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "device");
    int32_t const blocks = 8 * sms;
    DevBuf out;
    ck(out.ensure((size_t)blocks * sizeof(double)), "fp64 rate");
    Events const ev(2, "fp64 rate");
    ck(bfg::launchFp64Rate(blocks, 1024, out.as<double>(), s), "fp64 rate");   // warm-up
    int32_t const iters = 4096;
    ck(cudaEventRecord(ev[0], s), "fp64 rate");
    ck(bfg::launchFp64Rate(blocks, iters, out.as<double>(), s), "fp64 rate");
    ck(cudaEventRecord(ev[1], s), "fp64 rate");
    ck(cudaEventSynchronize(ev[1]), "fp64 rate");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, ev[0], ev[1]), "fp64 rate");
    double const flops = 2.0 * 8.0 * iters * 256.0 * blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return BFG_OK;
  });
}

bfgStatus bfgPlanHelm2(double k, double const *srcXy, int64_t numSrc, double const *tgtXy,
                       int64_t numTgt, bfgFacOptions const *opts, int64_t *srcPerm,
                       int64_t *tgtPerm, char *buf, int64_t cap, int64_t *len) {
  if (!srcXy || !tgtXy || numSrc < 1 || numTgt < 1 || !(k > 0)) return BFG_ERROR_INVALID_ARGUMENTS;
  try {
    bfgFacOptions o;
    bfgFacOptionsDefault(&o);
    if (opts) o = *opts;
    if (o.leafSize < 1 || !(o.rankEps > 0 && o.rankEps < 1)) return BFG_ERROR_INVALID_ARGUMENTS;
    bfg::PlanParams pp;
    pp.k = k;
    pp.leafSize = o.leafSize;
    pp.rankEps = o.rankEps;
    bfg::Plan plan;
    bfg::makePlan(plan, pp, srcXy, numSrc, tgtXy, numTgt);
    if (srcPerm) std::copy(plan.src.perm.begin(), plan.src.perm.end(), srcPerm);
    if (tgtPerm) std::copy(plan.tgt.perm.begin(), plan.tgt.perm.end(), tgtPerm);
    std::string t = plan.text();
    if (len) *len = (int64_t)t.size();
    if (buf && cap > 0) {
      int64_t n = std::min<int64_t>(cap - 1, (int64_t)t.size());
      std::memcpy(buf, t.data(), (size_t)n);
      buf[n] = 0;
      if (cap <= (int64_t)t.size()) return BFG_ERROR_OUT_OF_RANGE;
    }
    return BFG_OK;
  } catch (std::bad_alloc const &) {
    return BFG_ERROR_MEMORY;
  } catch (std::exception const &) {
    return BFG_ERROR_RUNTIME;
  }
}

bfgStatus bfgQuadtreeBuild(bfgContext ctx, double const *xy, int64_t const *setOffsets,
                           int64_t numSets, int64_t leafSize, int32_t onGpu, int64_t *perm,
                           bfgQuadtreeNode *nodes, int64_t nodeCapacity, int64_t *nodeOffsets) {
  if (!xy || !setOffsets || numSets < 1 || leafSize < 1 || !perm || !nodeOffsets ||
      (onGpu && !ctx) || (nodes && nodeCapacity < 0) || setOffsets[0] != 0)
    return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "quadtree: bad arguments");
  for (int64_t t = 0; t < numSets; ++t)
    if (setOffsets[t + 1] < setOffsets[t])
      return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "quadtree: decreasing set offsets");
  int64_t const n = setOffsets[numSets];
  for (int64_t i = 0; i < 2 * n; ++i)
    if (!std::isfinite(xy[i])) return fail(ctx, BFG_ERROR_INVALID_ARGUMENTS, "quadtree: non-finite point");
  return guarded(ctx, [&]() -> bfgStatus {
    std::vector<bfg::Quadtree> trees;
    if (onGpu) {
      bfg::buildQuadtreesGpu(xy, setOffsets, numSets, leafSize, ctx->stream, trees);
    } else {
      trees.resize((size_t)numSets);
      for (int64_t t = 0; t < numSets; ++t)
        trees[(size_t)t].build(xy + 2 * setOffsets[t], setOffsets[t + 1] - setOffsets[t], leafSize);
    }
    nodeOffsets[0] = 0;
    for (int64_t t = 0; t < numSets; ++t) {
      nodeOffsets[t + 1] = nodeOffsets[t] + (int64_t)trees[(size_t)t].nodes.size();
      std::copy(trees[(size_t)t].perm.begin(), trees[(size_t)t].perm.end(), perm + setOffsets[t]);
    }
    if (!nodes) return BFG_OK;
    if (nodeOffsets[numSets] > nodeCapacity)
      return fail(ctx, BFG_ERROR_OUT_OF_RANGE, "quadtree: node capacity too small");
    for (int64_t t = 0; t < numSets; ++t)
      for (size_t i = 0; i < trees[(size_t)t].nodes.size(); ++i) {
        bfg::QNode const &q = trees[(size_t)t].nodes[i];
        bfgQuadtreeNode &o = nodes[nodeOffsets[t] + (int64_t)i];
        o.xmin = q.xmin;
        o.ymin = q.ymin;
        o.xmax = q.xmax;
        o.ymax = q.ymax;
        o.splitX = q.sx;
        o.splitY = q.sy;
        o.i0 = q.i0;
        o.i1 = q.i1;
        o.parent = q.parent;
        o.depth = q.depth;
        for (int c = 0; c < 4; ++c) o.child[c] = q.child[c];
      }
    return BFG_OK;
  });
}

bfgStatus bfgBessel01Host(double const *x, int64_t n, double *out) {
  if (!x || !out || n < 0) return BFG_ERROR_INVALID_ARGUMENTS;
  for (int64_t i = 0; i < n; ++i) {
    if (!(x[i] > 0) || !std::isfinite(x[i])) return BFG_ERROR_OUT_OF_RANGE;
    bfg::Bessel01 b = bfg::bessel01<true>(x[i]);
    out[4 * i] = b.j0;
    out[4 * i + 1] = b.y0;
    out[4 * i + 2] = b.j1;
    out[4 * i + 3] = b.y1;
  }
  return BFG_OK;
}

// rand.c:19-76 with explicit state
void bfgRngSeed(bfgRng *rng, uint64_t seed) {
  uint64_t x = seed;
  for (int i = 0; i < 4; ++i) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    rng->s[i] = z ^ (z >> 31);
  }
}

static uint64_t rngNext(bfgRng *rng) {
  uint64_t *s = rng->s;
  uint64_t const result = s[0] + s[3];
  uint64_t const t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = (s[3] << 45) | (s[3] >> 19);
  return result;
}

double bfgRngUniform1(bfgRng *rng) { return (double)(rngNext(rng) >> 11) * 0x1.0p-53; }

void bfgRngUniform(bfgRng *rng, int64_t n, double *out) {
  for (int64_t i = 0; i < n; ++i) out[i] = bfgRngUniform1(rng);
}

void bfgRngComplexRandn(bfgRng *rng, int64_t n, double *x) {
  // bfRealRandn on 2n reals (rand.c:50-76)
  int64_t const m = 2 * n;
  bfgRngUniform(rng, 2 * (m / 2), x);
  double const twoPi = 6.283185307179586;
  for (int64_t i = 0; i < m / 2; ++i) {
    double mag = std::sqrt(-2 * std::log(x[2 * i]));
    double theta = twoPi * x[2 * i + 1];
    x[2 * i] = mag * std::cos(theta);
    x[2 * i + 1] = mag * std::sin(theta);
  }
}

}  // extern "C"
