// Host-only self-check of the apply's work decomposition (bfgPlanCheckApply).
//
// The device apply does not walk the factorization's block structure: it
// runs a staged program (makeApplyProgram: items of up to 32 rows, each
// summing the blocks of one block row, workspace regions per product, the
// last factors of up to kFinGroup products sharing one region, and a final
// segmented sum), and the tensor-core kernel runs that program's 128-row
// variant cut into chunks dealt to persistent CTAs (makeTcSchedule).  This
// file evaluates A X three ways in FP64 on the host -- directly from the
// plan's structure (fac_helm2.c:943-1002 with mat_block_dense.c:512-572,
// mat_product.c, mat_block_diag.c, mat_block_coo.c Mul), by executing the
// staged program, and by executing every chunk schedule the autotuner can
// choose -- over seeded block values, and reports how far the last two are
// from the first.  No operator values are returned: this checks schedules,
// it is not an apply.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <unordered_map>
#include <vector>

#include "bfg.h"
#include "bfg_plan.hpp"

namespace {

using cd = std::complex<double>;

struct CheckError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// splitmix64: seeded values, reproducible on every platform
struct Mix {
  uint64_t s;
  double next() {   // uniform in [-1, 1)
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
};

// every stored block column-major m x n at its arena offset, entries
// uniform in the unit square scaled by 1/sqrt(n) so products stay O(1)
std::vector<cd> seededArena(bfg::Plan const &plan, uint64_t seed) {
  std::vector<cd> a((size_t)plan.arenaEntries);
  Mix g{seed};
  for (int32_t bi : plan.blockOrder) {
    bfg::Block const &b = plan.blocks[(size_t)bi];
    double const sc = 1.0 / std::sqrt((double)std::max(1, b.n));
    for (int64_t e = 0; e < (int64_t)b.m * b.n; ++e) {
      double const re = g.next(), im = g.next();
      a[(size_t)(b.arenaOff + e)] = cd(re * sc, im * sc);
    }
  }
  return a;
}

// Y[t0 + r] += B v[c0 + c] for an m x n block; rows of R entries
void blockMul(std::vector<cd> const &A, bfg::Block const &b, cd const *v, cd *y, int R) {
  for (int32_t c = 0; c < b.n; ++c) {
    cd const *vc = v + (size_t)c * R;
    cd const *col = A.data() + b.arenaOff + (int64_t)c * b.m;
    for (int32_t r = 0; r < b.m; ++r) {
      cd const a = col[r];
      cd *yr = y + (size_t)r * R;
      for (int q = 0; q < R; ++q) yr[q] += a * vc[q];
    }
  }
}

// A X from the plan's structure, recursively (tree order in and out)
void directNode(bfg::Plan const &plan, std::vector<cd> const &A, int32_t id, cd const *X,
                cd *Y, int R) {
  bfg::PNode const &nd = plan.pnodes[(size_t)id];
  if (nd.type == 0) {
    for (int32_t i = 0; i < nd.nr; ++i)
      for (int32_t j = 0; j < nd.nc; ++j)
        directNode(plan, A, nd.children[(size_t)i * nd.nc + j], X, Y, R);
    return;
  }
  if (nd.type == 2) {
    bfg::Block const &b = plan.blocks[(size_t)nd.block];
    if (b.t1 - b.t0 != b.m || b.s1 - b.s0 != b.n) throw CheckError("dense block ranges");
    blockMul(A, b, X + (size_t)b.s0 * R, Y + (size_t)b.t0 * R, R);
    return;
  }
  bfg::Product const &pr = plan.products[(size_t)nd.product];
  size_t const nf = pr.factors.size();
  std::vector<cd> v(X + (size_t)pr.s0 * R, X + (size_t)pr.s1 * R);
  int64_t rowsIn = pr.s1 - pr.s0;
  for (size_t a = nf; a-- > 0;) {   // stored [last, ..., first]: first applied first
    bfg::Factor const &f = plan.factors[(size_t)pr.factors[a]];
    if (f.colOff.back() != rowsIn) throw CheckError("factor columns do not chain");
    std::vector<cd> w((size_t)f.rowOff.back() * R, cd(0, 0));
    for (int32_t bi : f.blocks) {
      bfg::Block const &b = plan.blocks[(size_t)bi];
      if (f.rowOff[(size_t)b.ri + 1] - f.rowOff[(size_t)b.ri] != b.m ||
          f.colOff[(size_t)b.ci + 1] - f.colOff[(size_t)b.ci] != b.n)
        throw CheckError("block does not fit its factor's partition");
      blockMul(A, b, v.data() + (size_t)f.colOff[(size_t)b.ci] * R,
               w.data() + (size_t)f.rowOff[(size_t)b.ri] * R, R);
    }
    v.swap(w);
    rowsIn = f.rowOff.back();
  }
  if (rowsIn != pr.t1 - pr.t0) throw CheckError("product rows");
  for (int64_t i = 0; i < rowsIn * R; ++i) Y[(size_t)(pr.t0 * R + i)] += v[(size_t)i];
}

// The final sum of the device apply: target row i adds the workspace rows
// of every region of its segment.
void finalSum(bfg::ApplyProgram const &prog, std::vector<cd> const &ws, int R, cd *Y) {
  for (int64_t i = 0; i < prog.numRows; ++i) {
    int32_t const s = prog.rowSeg[(size_t)i];
    for (int64_t c = prog.segContrib0[(size_t)s]; c < prog.segContrib0[(size_t)s + 1]; ++c) {
      int64_t const row = prog.segBase[(size_t)c] + (i - prog.segStart[(size_t)s]);
      for (int q = 0; q < R; ++q) Y[(size_t)(i * R + q)] += ws[(size_t)(row * R + q)];
    }
  }
}

// Writes of one stage, committed after the whole stage has run: the device
// runs a stage's items concurrently, so a read of a row the same stage
// writes would be a race; here it reads the pre-stage value (NaN if no
// earlier stage wrote it) and the comparison catches it.
struct StageWrites {
  std::vector<std::pair<int64_t, std::vector<cd>>> rows;   // (first row, rows x R)
  void commit(std::vector<cd> &ws, int R, std::vector<int32_t> &stamp, int32_t stage) {
    for (auto &w : rows) {
      int64_t const n = (int64_t)w.second.size() / R;
      for (int64_t r = 0; r < n; ++r) {
        if (stamp[(size_t)(w.first + r)] == stage)
          throw CheckError("a workspace row is written twice in one stage");
        stamp[(size_t)(w.first + r)] = stage;
      }
      std::copy(w.second.begin(), w.second.end(), ws.begin() + w.first * R);
    }
    rows.clear();
  }
};

void runProgram(bfg::ApplyProgram const &prog, std::vector<cd> const &A, cd const *X, int R,
                cd *Y) {
  std::vector<cd> ws((size_t)(prog.wsRows * R),
                     cd(std::numeric_limits<double>::quiet_NaN(), 0.0));
  std::vector<int32_t> stamp((size_t)prog.wsRows, -1);
  StageWrites sw;
  for (size_t s = 0; s + 1 < prog.stageItem0.size(); ++s) {
    for (int64_t it = prog.stageItem0[s]; it < prog.stageItem0[s + 1]; ++it) {
      bfg::ApplyItem const &item = prog.items[(size_t)it];
      std::vector<cd> acc((size_t)item.rows * R, cd(0, 0));
      for (int32_t c = 0; c < item.nContrib; ++c) {
        bfg::ApplyContrib const &cb = prog.contribs[(size_t)(item.contrib0 + c)];
        cd const *in = cb.inIsX ? X : ws.data();
        for (int32_t j = 0; j < cb.n; ++j)
          for (int32_t r = 0; r < item.rows; ++r) {
            cd const a = A[(size_t)(cb.aOff + r + (int64_t)j * cb.lda)];
            for (int q = 0; q < R; ++q)
              acc[(size_t)(r * R + q)] += a * in[(size_t)((cb.inRow + j) * R + q)];
          }
      }
      sw.rows.push_back({item.outRow, std::move(acc)});
    }
    sw.commit(ws, R, stamp, (int32_t)s);
  }
  finalSum(prog, ws, R, Y);
}

// The tensor-core schedule: per stage, each CTA runs its chunks in order; a
// chunk flagged first starts an item's accumulator, one flagged last writes
// it.  The final sum is the staged program's (the device shares it).
void runTcSchedule(bfg::ApplyProgram const &prog, bfg::TcSchedule const &sc,
                   std::vector<cd> const &A, cd const *X, int R, cd *Y) {
  std::unordered_map<int64_t, size_t> fillOf;
  for (size_t i = 0; i < sc.fills.size(); ++i) fillOf[sc.fills[i].tileOff] = i;
  size_t const nStages = prog.stageItem0.size() - 1;
  if (sc.ctaChunk0.size() != nStages * (size_t)(sc.ctas + 1))
    throw CheckError("chunk schedule has the wrong number of stages");
  std::vector<cd> ws((size_t)(prog.wsRows * R),
                     cd(std::numeric_limits<double>::quiet_NaN(), 0.0));
  std::vector<int32_t> stamp((size_t)prog.wsRows, -1);
  StageWrites sw;
  for (size_t s = 0; s < nStages; ++s) {
    for (int32_t c = 0; c < sc.ctas; ++c) {
      int64_t const k0 = sc.ctaChunk0[s * (size_t)(sc.ctas + 1) + (size_t)c];
      int64_t const k1 = sc.ctaChunk0[s * (size_t)(sc.ctas + 1) + (size_t)c + 1];
      std::vector<cd> acc;
      bool open = false;
      for (int64_t k = k0; k < k1; ++k) {
        bfg::TcChunk const &ch = sc.chunks[(size_t)k];
        if (ch.flags & bfg::kTcFirst) {
          if (open) throw CheckError("a chunk item starts before the previous one ended");
          acc.assign((size_t)ch.rows * R, cd(0, 0));
          open = true;
        }
        if (!open) throw CheckError("a chunk outside any item");
        auto const hit = fillOf.find(ch.tileOff);
        if (hit == fillOf.end()) throw CheckError("a chunk without its tile");
        bfg::TcFill const &f = sc.fills[hit->second];
        if (f.nc != ch.nc || f.rows != ch.rows || ch.rows > bfg::kTcRows)
          throw CheckError("a chunk and its tile disagree");
        cd const *in = ch.inIsX ? X : ws.data();
        for (int32_t j = 0; j < ch.nc; ++j)
          for (int32_t r = 0; r < ch.rows; ++r) {
            cd const a = A[(size_t)(f.srcOff + r + (int64_t)j * f.lda)];
            for (int q = 0; q < R; ++q)
              acc[(size_t)(r * R + q)] += a * in[(size_t)((ch.inRow + j) * R + q)];
          }
        if (ch.flags & bfg::kTcLast) {
          sw.rows.push_back({ch.outRow, std::move(acc)});
          acc.clear();
          open = false;
        }
      }
      if (open) throw CheckError("a CTA's last item has no last chunk");
    }
    sw.commit(ws, R, stamp, (int32_t)s);
  }
  finalSum(prog, ws, R, Y);
}

double relDiff(std::vector<cd> const &y, std::vector<cd> const &ref) {
  double num = 0, den = 0;
  for (size_t i = 0; i < y.size(); ++i) {
    num += std::norm(y[i] - ref[i]);
    den += std::norm(ref[i]);
  }
  if (!std::isfinite(num)) return std::numeric_limits<double>::infinity();
  return den > 0 ? std::sqrt(num / den) : std::sqrt(num);
}

}  // namespace

extern "C" bfgStatus bfgPlanCheckApply(double const *k, int64_t numProblems, double const *srcXy,
                                       int64_t const *srcOffsets, double const *tgtXy,
                                       int64_t const *tgtOffsets, bfgFacOptions const *opts,
                                       int32_t numRhs, int32_t ctas, uint64_t seed,
                                       double *relErr) {
  if (!k || numProblems < 1 || !srcXy || !tgtXy || !srcOffsets || !tgtOffsets || !relErr ||
      numRhs < 1 || numRhs > 64 || ctas < 1 || srcOffsets[0] != 0 || tgtOffsets[0] != 0)
    return BFG_ERROR_INVALID_ARGUMENTS;
  for (int64_t p = 0; p < numProblems; ++p)
    if (!(k[p] > 0) || srcOffsets[p + 1] <= srcOffsets[p] || tgtOffsets[p + 1] <= tgtOffsets[p])
      return BFG_ERROR_INVALID_ARGUMENTS;
  int64_t const nSrc = srcOffsets[numProblems], nTgt = tgtOffsets[numProblems];
  for (int64_t i = 0; i < 2 * nSrc; ++i)
    if (!std::isfinite(srcXy[i])) return BFG_ERROR_INVALID_ARGUMENTS;
  for (int64_t i = 0; i < 2 * nTgt; ++i)
    if (!std::isfinite(tgtXy[i])) return BFG_ERROR_INVALID_ARGUMENTS;
  try {
    bfgFacOptions o;
    bfgFacOptionsDefault(&o);
    if (opts) o = *opts;
    if (o.leafSize < 1 || !(o.rankEps > 0 && o.rankEps < 1)) return BFG_ERROR_INVALID_ARGUMENTS;
    bfg::PlanParams pp;
    pp.k = k[0];
    pp.leafSize = o.leafSize;
    pp.rankEps = o.rankEps;
    bfg::Plan plan;
    // the planner each factorization call uses
    if (numProblems == 1)
      bfg::makePlan(plan, pp, srcXy, nSrc, tgtXy, nTgt);
    else
      bfg::makePlanBatched(plan, pp, k, srcXy, srcOffsets, tgtXy, tgtOffsets, numProblems);

    int const R = numRhs;
    std::vector<cd> const A = seededArena(plan, seed);
    std::vector<cd> X((size_t)(nSrc * R));
    Mix g{seed ^ 0x5851f42d4c957f2dull};
    for (auto &x : X) {
      double const re = g.next();
      x = cd(re, g.next());
    }
    std::vector<cd> yRef((size_t)(nTgt * R), cd(0, 0));
    for (auto const &root : plan.roots) directNode(plan, A, root.pnode, X.data(), yRef.data(), R);

    bfg::ApplyProgram prog;
    bfg::makeApplyProgram(plan, prog);
    std::vector<cd> y((size_t)(nTgt * R), cd(0, 0));
    runProgram(prog, A, X.data(), R, y.data());
    relErr[0] = relDiff(y, yRef);

    bfg::ApplyProgram p128;
    bfg::makeApplyProgram(plan, p128, bfg::kTcRows);
    if (p128.wsRows != prog.wsRows || p128.stageItem0.size() != prog.stageItem0.size())
      throw CheckError("the 32- and 128-row programs differ in layout");
    double worst = 0;
    for (bfg::TcCostModel const &m : bfg::tcCandidateModels()) {
      bfg::TcSchedule sc;
      bfg::makeTcSchedule(p128, 3, ctas, sc, m);
      std::fill(y.begin(), y.end(), cd(0, 0));
      runTcSchedule(prog, sc, A, X.data(), R, y.data());
      worst = std::max(worst, relDiff(y, yRef));
    }
    relErr[1] = worst;
    return BFG_OK;
  } catch (CheckError const &) {
    return BFG_ERROR_RUNTIME;
  } catch (std::bad_alloc const &) {
    return BFG_ERROR_MEMORY;
  } catch (std::exception const &) {
    return BFG_ERROR_RUNTIME;
  }
}
