// Quadtree, planner and descriptor flattening.  The planner follows the
// reference's control flow node pair by node pair so that block shapes,
// ranks and orderings are identical (checked against the reference's own
// output by the parity tests):
//   facHelm2MakeMultilevel_rec / _dense / _separated / _diag
//                                         fac_helm2.c:741-941
//   bfFacHelm2Prepare                     fac_helm2.c:551-651
//   bfFacHelm2Make                        fac_helm2.c:653-704
//   makeFirstFactor / makeFactor / makeLastFactor
//                                         fac_helm2.c:42-509
//   bfHelm2RankEstForTwoCircles           helm2.c:14-36
//   bfQuadtreeNodesAreSeparated           quadtree_node.c:393-401
// Floating-point expressions that decide integers (ranks, separation) are
// written in the same operation order as the reference.
#include "bfg_plan.hpp"

#include <algorithm>
#include <atomic>
#include <thread>
#include <cmath>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <tuple>

namespace bfg {

namespace {
constexpr double kEpsMach = 2.220446049250313e-16;        // def.h:29
constexpr int64_t kMaxDenseMatrixSize = 128 * 128;         // fac_helm2.c:20
}  // namespace

// ---------------------------------------------------------------------------
// Quadtree
// ---------------------------------------------------------------------------
void Quadtree::build(double const *xy, int64_t n, int64_t leafSize_) {
  leafSize = leafSize_ < 1 ? 1 : leafSize_;
  nodes.clear();
  perm.resize(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = i;
  std::vector<double> px(n), py(n);
  for (int64_t i = 0; i < n; ++i) {
    px[i] = xy[2 * i];
    py[i] = xy[2 * i + 1];
  }
  // bfPoints2GetBoundingBox (points.c:415-430)
  double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  for (int64_t i = 0; i < n; ++i) {
    xmin = std::fmin(xmin, px[i]);
    xmax = std::fmax(xmax, px[i]);
    ymin = std::fmin(ymin, py[i]);
    ymax = std::fmax(ymax, py[i]);
  }
  QNode root = rootNode(xmin, xmax, ymin, ymax);
  root.i0 = 0;
  root.i1 = n;
  nodes.push_back(root);
  if (n > 0) split(0, px.data(), py.data());
}

QNode Quadtree::rootNode(double xmin, double xmax, double ymin, double ymax) {
  // bfBbox2RescaleToSquare (bbox.c:18-30)
  double w = xmax - xmin, h = ymax - ymin;
  // the reference's formula divides by a zero side for one point or for
  // collinear points (its boxes become NaN there); the limit of the formula
  // is used instead, and a unit square around a single point
  if (w == 0 && h == 0) {
    xmin -= 0.5;
    xmax += 0.5;
    ymin -= 0.5;
    ymax += 0.5;
  } else if (w > h) {
    double c = (ymin + ymax) / 2;
    if (h > 0) {
      ymin = w * (ymin - c) / h + c;
      ymax = w * (ymax - c) / h + c;
    } else {
      ymin = c - w / 2;
      ymax = c + w / 2;
    }
  } else {
    double c = (xmin + xmax) / 2;
    if (w > 0) {
      xmin = h * (xmin - c) / w + c;
      xmax = h * (xmax - c) / w + c;
    } else {
      xmin = c - h / 2;
      xmax = c + h / 2;
    }
  }
  QNode root;
  root.xmin = xmin; root.ymin = ymin; root.xmax = xmax; root.ymax = ymax;
  root.sx = (xmin + xmax) / 2;
  root.sy = (ymin + ymax) / 2;
  return root;
}

QNode Quadtree::childNode(QNode const &par, int q) {
  double const xmin = par.xmin, ymin = par.ymin, xmax = par.xmax, ymax = par.ymax;
  double const sx = par.sx, sy = par.sy;
  double const box[4][4] = {{xmin, ymin, sx, sy}, {xmin, sy, sx, ymax},
                            {sx, ymin, xmax, sy}, {sx, sy, xmax, ymax}};
  QNode ch;
  ch.xmin = box[q][0]; ch.ymin = box[q][1]; ch.xmax = box[q][2]; ch.ymax = box[q][3];
  ch.sx = (ch.xmin + ch.xmax) / 2;
  ch.sy = (ch.ymin + ch.ymax) / 2;
  ch.depth = par.depth + 1;
  return ch;
}

void Quadtree::split(int node, double const *px, double const *py) {
  int64_t const i0 = nodes[node].i0, i1 = nodes[node].i1;
  double const sx = nodes[node].sx, sy = nodes[node].sy;
  int64_t *p = perm.data();
  auto in = [&](int q, int64_t idx) {
    double x = px[p[idx]], y = py[p[idx]];
    switch (q) {
      case 0: return x <= sx && y <= sy;
      case 1: return x <= sx && y > sy;
      default: return x > sx && y <= sy;
    }
  };
  int64_t off[5];
  off[0] = i0;
  off[4] = i1;
  for (int q = 0; q < 3; ++q) {
    // the sift of quadtree_node.c:148-194
    int64_t i = off[q];
    while (i < i1 && in(q, i)) ++i;
    int64_t j = i == i1 ? i : i + 1;
    while (j < i1) {
      if (in(q, j) && !in(q, i)) {
        std::swap(p[i], p[j]);
        ++i;
      }
      ++j;
    }
    off[q + 1] = i;
  }
  int const depth = nodes[node].depth;
  for (int q = 0; q < 4; ++q) {
    int64_t cnt = off[q + 1] - off[q];
    if (cnt == 0) continue;
    QNode ch = childNode(nodes[node], q);
    ch.parent = node;
    ch.i0 = off[q];
    ch.i1 = off[q + 1];
    int idx = (int)nodes.size();
    nodes.push_back(ch);
    nodes[node].child[q] = idx;
    if (cnt > leafSize) {
      if (depth + 1 > 200) throw std::runtime_error("quadtree deeper than 200 levels (duplicate points?)");
      split(idx, px, py);
    }
  }
}

Circle Quadtree::circle(int node) const {
  QNode const &nd = nodes[node];
  Circle c;
  c.r = std::hypot(nd.xmax - nd.xmin, nd.ymax - nd.ymin) / 2;
  c.cx = (nd.xmin + nd.xmax) / 2;
  c.cy = (nd.ymin + nd.ymax) / 2;
  return c;
}

std::vector<int> Quadtree::children(int node) const {
  std::vector<int> out;
  for (int q = 0; q < 4; ++q)
    if (nodes[node].child[q] >= 0) out.push_back(nodes[node].child[q]);
  return out;
}

std::vector<std::vector<int>> Quadtree::levelsBelow(int node) const {
  std::vector<int> order{node};
  for (size_t i = 0; i < order.size(); ++i)
    for (int q = 0; q < 4; ++q)
      if (nodes[order[i]].child[q] >= 0) order.push_back(nodes[order[i]].child[q]);
  std::vector<std::vector<int>> levels;
  for (int nd : order) {
    if (levels.empty() || nodes[levels.back()[0]].depth != nodes[nd].depth)
      levels.emplace_back();
    levels.back().push_back(nd);
  }
  return levels;
}

// ---------------------------------------------------------------------------
// Planner
// ---------------------------------------------------------------------------
namespace {

int64_t rankEst(double k, Circle const &c1, Circle const &c2, double C, double eps) {
  double r1 = c1.r, r2 = c2.r;
  double R = std::hypot(c2.cx - c1.cx, c2.cy - c1.cy);
  double d = R - r1 - r2;
  if (!(r1 > 0 && r2 > 0 && R > 0 && d > 0))
    throw std::runtime_error("rank estimate requested for overlapping circles");
  double p = k * r1 * r2 / d - C * std::log10(eps);
  if (!(p > 0)) throw std::runtime_error("non-positive rank estimate");
  return (int64_t)std::ceil(p);
}

class Planner {
 public:
  Planner(Plan &plan, PlanParams const &prm) : P(plan), prm(prm) {}

  // bfFacHelm2MakeMultilevel (fac_helm2.c:943-1002) starts from the nodes at
  // depth 2; a leaf shallower than that (tiny point sets) would leave its
  // points out of every block, so it joins the list in tree order (for trees
  // whose depth-1 nodes are all split this is the reference's list)
  int32_t run() { return rec(frontier(P.src), frontier(P.tgt)); }

  static std::vector<int> frontier(Quadtree const &t) {
    std::vector<int> out;
    auto walk = [&](auto &&self, int nd) -> void {
      std::vector<int> kids = t.children(nd);
      if (t.nodes[nd].depth == 2 || kids.empty()) {
        out.push_back(nd);
        return;
      }
      for (int ch : kids) self(self, ch);
    };
    for (int ch : t.children(0)) walk(walk, ch);
    return out;
  }

 private:
  Plan &P;
  PlanParams prm;

  int64_t rank(Circle const &a, Circle const &b) { return rankEst(prm.k, a, b, 1.0, prm.rankEps); }
  QNode const &sn(int i) const { return P.src.nodes[i]; }
  QNode const &tn(int i) const { return P.tgt.nodes[i]; }

  bool separated(int s, int t) const {
    Circle c1 = P.src.circle(s), c2 = P.tgt.circle(t);
    double R = std::hypot(c2.cx - c1.cx, c2.cy - c1.cy);
    return R > c1.r + c2.r + 1e1 * kEpsMach;
  }

  int32_t newPNode(PNode &&nd) {
    P.pnodes.push_back(std::move(nd));
    return (int32_t)P.pnodes.size() - 1;
  }

  int32_t dense(int s, int t) {
    Block b{};
    b.kind = kDense;
    b.m = (int32_t)tn(t).numPoints();
    b.n = (int32_t)sn(s).numPoints();
    b.s0 = sn(s).i0; b.s1 = sn(s).i1;
    b.t0 = tn(t).i0; b.t1 = tn(t).i1;
    P.blocks.push_back(b);
    PNode nd;
    nd.type = 2;
    nd.block = (int32_t)P.blocks.size() - 1;
    return newPNode(std::move(nd));
  }

  // facHelm2MakeMultilevel_rec (fac_helm2.c:860-941)
  int32_t rec(std::vector<int> const &srcNodes, std::vector<int> const &tgtNodes) {
    PNode nd;
    nd.type = 0;
    nd.nr = (int32_t)tgtNodes.size();
    nd.nc = (int32_t)srcNodes.size();
    nd.rowOff.push_back(0);
    nd.colOff.push_back(0);
    std::vector<int32_t> children;
    for (size_t i = 0; i < tgtNodes.size(); ++i) {
      int t = tgtNodes[i];
      int64_t m = tn(t).numPoints();
      for (size_t j = 0; j < srcNodes.size(); ++j) {
        int s = srcNodes[j];
        int64_t n = sn(s).numPoints();
        bool sep = separated(s, t);
        // A leaf on either side can only be handled densely; the reference
        // has a leaf size of one, where this case cannot reach the other
        // branches without aborting (Prepare asserts an internal target).
        bool leafy = sn(s).leaf() || tn(t).leaf();
        int32_t child;
        if (m * n < kMaxDenseMatrixSize || leafy)
          child = dense(s, t);
        else if (sep)
          child = separatedPair(s, t);
        else
          child = rec(P.src.children(s), P.tgt.children(t));
        children.push_back(child);
        if (i == 0) nd.colOff.push_back(nd.colOff.back() + n);
      }
      nd.rowOff.push_back(nd.rowOff.back() + m);
    }
    nd.children = std::move(children);
    return newPNode(std::move(nd));
  }

  bool allRanksOk(int t, std::vector<int> const &srcLevel) {
    Circle tc = P.tgt.circle(t);
    for (int s : srcLevel)
      if (rank(tc, P.src.circle(s)) > sn(s).numPoints()) return false;
    return true;
  }

  bool internal(Quadtree const &tr, std::vector<int> const &lv) const {
    for (int nd : lv)
      if (tr.nodes[nd].leaf()) return false;
    return true;
  }

  // bfFacHelm2Prepare + bfFacHelm2Make (fac_helm2.c:551-704)
  int32_t separatedPair(int s, int t) {
    int64_t const numSrc = sn(s).numPoints();
    auto srcLevels = P.src.levelsBelow(s);
    auto tgtLevels = P.tgt.levelsBelow(t);
    int64_t maxAllow = tn(t).depth;
    if (!internal(P.tgt, tgtLevels[0])) throw std::runtime_error("target node is a leaf");
    size_t ti = 1;
    while (ti < tgtLevels.size() && internal(P.tgt, tgtLevels[ti])) {
      ++maxAllow;
      ++ti;
    }
    int64_t si = (int64_t)srcLevels.size() - 1;
    int64_t srcDepth = sn(srcLevels[si][0]).depth;
    int64_t const tgtDepth = tn(t).depth;
    int guard = 0;
    auto step = [&]() {
      if (si > 0) --si;
      --srcDepth;
      if (++guard > 100000) throw std::runtime_error("level search did not terminate");
    };
    auto npts = [&](std::vector<int> const &lv) {
      int64_t c = 0;
      for (int nd : lv) c += sn(nd).numPoints();
      return c;
    };
    while (srcDepth > maxAllow) step();
    while (npts(srcLevels[si]) != numSrc) step();
    while (!internal(P.src, srcLevels[si])) step();
    while (srcDepth > tgtDepth && !allRanksOk(t, srcLevels[si])) step();
    int64_t nf = allRanksOk(t, srcLevels[si]) ? srcDepth - tgtDepth + 2 : 0;
    if (nf == 0) return dense(s, t);

    std::vector<int32_t> fac;
    size_t tli = 0;
    fac.push_back(firstFactor(srcLevels[si], tgtLevels[tli]));
    for (int64_t i = 1; i < nf - 1; ++i) {
      if (si > 0) --si;
      fac.push_back(middleFactor(fac.back(), srcLevels[si], tgtLevels[tli]));
      if (tli + 1 < tgtLevels.size()) ++tli;
    }
    fac.push_back(lastFactor(fac.back(), srcLevels[si], tgtLevels[tli]));
    Product pr;
    pr.factors.assign(fac.rbegin(), fac.rend());
    pr.t0 = tn(t).i0; pr.t1 = tn(t).i1;
    pr.s0 = sn(s).i0; pr.s1 = sn(s).i1;
    P.products.push_back(std::move(pr));
    PNode nd;
    nd.type = 1;
    nd.product = (int32_t)P.products.size() - 1;
    return newPNode(std::move(nd));
  }

  int32_t pushFactor(Factor &&f) {
    P.factors.push_back(std::move(f));
    return (int32_t)P.factors.size() - 1;
  }

  // makeFirstFactor (fac_helm2.c:42-160)
  int32_t firstFactor(std::vector<int> const &srcLevel, std::vector<int> const &tgtLevel) {
    if (tgtLevel.size() != 1) throw std::runtime_error("first factor needs one target node");
    Circle tc = P.tgt.circle(tgtLevel[0]);
    Factor f;
    f.kind = 0;
    f.nbr = f.nbc = (int32_t)srcLevel.size();
    f.rowOff.push_back(0);
    f.colOff.push_back(0);
    for (size_t i = 0; i < srcLevel.size(); ++i) {
      int s = srcLevel[i];
      Circle sc = P.src.circle(s);
      int64_t p = rank(sc, tc);
      Block b{};
      b.kind = kFirst;
      b.m = (int32_t)p;
      b.n = (int32_t)sn(s).numPoints();
      b.ri = b.ci = (int32_t)i;
      b.s0 = sn(s).i0; b.s1 = sn(s).i1;
      b.ceq = sc;
      b.cchk = tc;
      P.blocks.push_back(b);
      f.blocks.push_back((int32_t)P.blocks.size() - 1);
      f.rowOff.push_back(f.rowOff.back() + p);
      f.colOff.push_back(f.colOff.back() + b.n);
    }
    return pushFactor(std::move(f));
  }

  int64_t blockRows(int32_t fi, int64_t i) const {
    return P.factors[fi].rowOff[i + 1] - P.factors[fi].rowOff[i];
  }

  // makeFactor (fac_helm2.c:222-401), including the block-row rank = max
  // over the row (305-307)
  int32_t middleFactor(int32_t prev, std::vector<int> const &srcLevel,
                       std::vector<int> const &tgtLevel) {
    int64_t nTgtNodes = (int64_t)tgtLevel.size(), nTgtChildren = 0;
    int64_t nSrcNodes = (int64_t)srcLevel.size(), nSrcChildren = 0;
    for (int t : tgtLevel) nTgtChildren += (int64_t)P.tgt.children(t).size();
    for (int s : srcLevel) nSrcChildren += (int64_t)P.src.children(s).size();
    int64_t nbr = nTgtChildren * nSrcNodes, nbc = nSrcChildren * nTgtNodes;
    if (nbc != P.factors[prev].nbr) throw std::runtime_error("factor shapes are incompatible");
    Factor f;
    f.kind = 1;
    f.nbr = (int32_t)nbr;
    f.nbc = (int32_t)nbc;
    f.colOff.push_back(0);
    for (int64_t j = 0; j < nbc; ++j) f.colOff.push_back(f.colOff.back() + blockRows(prev, j));
    std::vector<int64_t> rows(nbr, -1);
    struct Entry { int64_t i, j; Circle schc, scirc, tchc; };
    std::vector<Entry> entries;
    int64_t iOffset = 0;
    for (int64_t tiIdx = 0; tiIdx < nTgtNodes; ++tiIdx) {
      int t = tgtLevel[tiIdx];
      Circle tcirc = P.tgt.circle(t);
      for (int tch : P.tgt.children(t)) {
        Circle tchc = P.tgt.circle(tch);
        int64_t j = tiIdx * nSrcChildren;
        for (int64_t siIdx = 0; siIdx < nSrcNodes; ++siIdx) {
          int s = srcLevel[siIdx];
          Circle scirc = P.src.circle(s);
          for (int sch : P.src.children(s)) {
            Circle schc = P.src.circle(sch);
            int64_t i = iOffset + siIdx;
            int64_t rankOr = rank(schc, tcirc);
            int64_t rankEq = rank(scirc, tchc);
            int64_t r = rankOr > rankEq ? rankOr : rankEq;
            if (rows[i] < 0 || r > rows[i]) rows[i] = r;
            entries.push_back({i, j, schc, scirc, tchc});
            ++j;
          }
        }
        iOffset += nSrcNodes;
      }
    }
    f.rowOff.push_back(0);
    for (int64_t i = 0; i < nbr; ++i) f.rowOff.push_back(f.rowOff.back() + rows[i]);
    for (auto const &e : entries) {
      Block b{};
      b.kind = kMiddle;
      b.ri = (int32_t)e.i;
      b.ci = (int32_t)e.j;
      b.m = (int32_t)(f.rowOff[e.i + 1] - f.rowOff[e.i]);
      b.n = (int32_t)(f.colOff[e.j + 1] - f.colOff[e.j]);
      b.corig = e.schc;
      b.ceq = e.scirc;
      b.cchk = e.tchc;
      P.blocks.push_back(b);
      f.blocks.push_back((int32_t)P.blocks.size() - 1);
    }
    return pushFactor(std::move(f));
  }

  // makeLastFactor (fac_helm2.c:403-509)
  int32_t lastFactor(int32_t prev, std::vector<int> const &srcLevel,
                     std::vector<int> const &tgtLevel) {
    if (srcLevel.size() != 1) throw std::runtime_error("last factor needs one source node");
    Circle sc = P.src.circle(srcLevel[0]);
    Factor f;
    f.kind = 0;
    f.nbr = f.nbc = (int32_t)tgtLevel.size();
    f.rowOff.push_back(0);
    f.colOff.push_back(0);
    for (size_t i = 0; i < tgtLevel.size(); ++i) {
      int t = tgtLevel[i];
      Block b{};
      b.kind = kLast;
      b.m = (int32_t)tn(t).numPoints();
      b.n = (int32_t)blockRows(prev, (int64_t)i);
      b.ri = b.ci = (int32_t)i;
      b.t0 = tn(t).i0; b.t1 = tn(t).i1;
      b.ceq = sc;
      P.blocks.push_back(b);
      f.blocks.push_back((int32_t)P.blocks.size() - 1);
      f.rowOff.push_back(f.rowOff.back() + b.m);
      f.colOff.push_back(f.colOff.back() + b.n);
    }
    return pushFactor(std::move(f));
  }
};

void appendOffsets(std::string &out, char const *tag, std::vector<int64_t> const &v) {
  out += tag;
  char buf[32];
  for (int64_t x : v) {
    std::snprintf(buf, sizeof buf, " %lld", (long long)x);
    out += buf;
  }
  out += '\n';
}

}  // namespace

void makePlan(Plan &plan, PlanParams const &params, double const *srcXy,
              int64_t nSrc, double const *tgtXy, int64_t nTgt, Quadtree const *srcTree,
              Quadtree const *tgtTree) {
  if (nSrc < 1 || nTgt < 1) throw std::runtime_error("empty point set");
  if (!(params.k > 0)) throw std::runtime_error("wavenumber must be positive");
  if (!(params.rankEps > 0 && params.rankEps < 1)) throw std::runtime_error("rank eps must be in (0,1)");
  plan = Plan();
  if (srcTree) {
    if ((int64_t)srcTree->perm.size() != nSrc || srcTree->leafSize != std::max<int64_t>(1, params.leafSize))
      throw std::runtime_error("source tree does not match the points");
    plan.src = *srcTree;
  } else {
    plan.src.build(srcXy, nSrc, params.leafSize);
  }
  if (tgtTree) {
    if ((int64_t)tgtTree->perm.size() != nTgt || tgtTree->leafSize != std::max<int64_t>(1, params.leafSize))
      throw std::runtime_error("target tree does not match the points");
    plan.tgt = *tgtTree;
  } else {
    plan.tgt.build(tgtXy, nTgt, params.leafSize);
  }
  Planner pl(plan, params);
  plan.root = pl.run();
  // plan order: block-dense children row-major, product factors in stored
  // order, blocks in factor order
  plan.blockOrder.clear();
  std::vector<int32_t> st{plan.root};
  while (!st.empty()) {
    int32_t idx = st.back();
    st.pop_back();
    PNode const &nd = plan.pnodes[idx];
    if (nd.type == 0) {
      for (auto it = nd.children.rbegin(); it != nd.children.rend(); ++it) st.push_back(*it);
    } else if (nd.type == 1) {
      for (int32_t fi : plan.products[nd.product].factors)
        for (int32_t bi : plan.factors[fi].blocks) plan.blockOrder.push_back(bi);
    } else {
      plan.blockOrder.push_back(nd.block);
    }
  }
  if (plan.blockOrder.size() != plan.blocks.size())
    throw std::runtime_error("plan traversal lost blocks");
  for (auto &b : plan.blocks) b.k = params.k;
  plan.roots.assign(1, Plan::Root{plan.root, 0, 0});
  int64_t off = 0;
  for (int32_t bi : plan.blockOrder) {
    plan.blocks[bi].arenaOff = off;
    off += (int64_t)plan.blocks[bi].m * plan.blocks[bi].n;
  }
  plan.arenaEntries = off;
}

void makePlanBatched(Plan &plan, PlanParams const &params, double const *k,
                     double const *srcXy, int64_t const *srcOff, double const *tgtXy,
                     int64_t const *tgtOff, int64_t numProblems,
                     std::vector<Quadtree> const *trees) {
  if (trees && (int64_t)trees->size() != 2 * numProblems)
    throw std::runtime_error("one source and one target tree per problem");
  if (numProblems < 1) throw std::runtime_error("no problems");
  std::vector<Plan> subs((size_t)numProblems);
  std::vector<std::string> errs((size_t)numProblems);
  unsigned nthreads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
  std::atomic<int64_t> next{0};
  auto worker = [&]() {
    for (int64_t p; (p = next++) < numProblems;) {
      try {
        PlanParams pp = params;
        pp.k = k[p];
        makePlan(subs[(size_t)p], pp, srcXy + 2 * srcOff[p], srcOff[p + 1] - srcOff[p],
                 tgtXy + 2 * tgtOff[p], tgtOff[p + 1] - tgtOff[p],
                 trees ? &(*trees)[(size_t)(2 * p)] : nullptr,
                 trees ? &(*trees)[(size_t)(2 * p + 1)] : nullptr);
      } catch (std::exception const &e) {
        errs[(size_t)p] = e.what();
      }
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nthreads; ++t) pool.emplace_back(worker);
  for (auto &t : pool) t.join();
  for (int64_t p = 0; p < numProblems; ++p)
    if (!errs[(size_t)p].empty())
      throw std::runtime_error("problem " + std::to_string(p) + ": " + errs[(size_t)p]);

  plan = Plan();
  for (int64_t p = 0; p < numProblems; ++p) {
    Plan const &q = subs[(size_t)p];
    int32_t const bBase = (int32_t)plan.blocks.size(), fBase = (int32_t)plan.factors.size();
    int32_t const prBase = (int32_t)plan.products.size(), nBase = (int32_t)plan.pnodes.size();
    int64_t const sB = srcOff[p], tB = tgtOff[p];
    for (Block b : q.blocks) {
      b.s0 += sB; b.s1 += sB; b.t0 += tB; b.t1 += tB;
      plan.blocks.push_back(b);
    }
    for (Factor f : q.factors) {
      for (auto &bi : f.blocks) bi += bBase;
      plan.factors.push_back(std::move(f));
    }
    for (Product pr : q.products) {
      for (auto &fi : pr.factors) fi += fBase;
      pr.t0 += tB; pr.t1 += tB; pr.s0 += sB; pr.s1 += sB;
      plan.products.push_back(std::move(pr));
    }
    for (PNode nd : q.pnodes) {
      for (auto &c : nd.children) c += nBase;
      if (nd.product >= 0) nd.product += prBase;
      if (nd.block >= 0) nd.block += bBase;
      plan.pnodes.push_back(std::move(nd));
    }
    for (int32_t bi : q.blockOrder) plan.blockOrder.push_back(bi + bBase);
    plan.roots.push_back(Plan::Root{q.root + nBase, tB, sB});
    for (int64_t v : q.src.perm) plan.src.perm.push_back(v + sB);
    for (int64_t v : q.tgt.perm) plan.tgt.perm.push_back(v + tB);
  }
  plan.root = plan.roots[0].pnode;
  int64_t off = 0;
  for (int32_t bi : plan.blockOrder) {
    plan.blocks[bi].arenaOff = off;
    off += (int64_t)plan.blocks[bi].m * plan.blocks[bi].n;
  }
  plan.arenaEntries = off;
}

std::string Plan::text() const {
  std::string out;
  char buf[128];
  // iterative pre-order walk that emits children in order; a batch of
  // problems prints each one after a "PROBLEM p" line
  struct Frame { int32_t kind; int32_t idx; };
  std::vector<Frame> st;
  for (size_t r = roots.size(); r-- > 0;) {
    st.push_back({0, roots[r].pnode});
    if (roots.size() > 1) st.push_back({2, (int32_t)r});
  }
  while (!st.empty()) {
    Frame fr = st.back();
    st.pop_back();
    if (fr.kind == 2) {
      std::snprintf(buf, sizeof buf, "PROBLEM %d\n", fr.idx);
      out += buf;
    } else if (fr.kind == 0) {
      PNode const &nd = pnodes[fr.idx];
      if (nd.type == 0) {
        std::snprintf(buf, sizeof buf, "BD %d %d\n", nd.nr, nd.nc);
        out += buf;
        appendOffsets(out, "RO", nd.rowOff);
        appendOffsets(out, "CO", nd.colOff);
        for (auto it = nd.children.rbegin(); it != nd.children.rend(); ++it) st.push_back({0, *it});
      } else if (nd.type == 1) {
        Product const &pr = products[nd.product];
        std::snprintf(buf, sizeof buf, "PR %zu\n", pr.factors.size());
        out += buf;
        for (auto it = pr.factors.rbegin(); it != pr.factors.rend(); ++it) st.push_back({1, *it});
      } else {
        Block const &b = blocks[nd.block];
        std::snprintf(buf, sizeof buf, "DC %d %d\n", b.m, b.n);
        out += buf;
      }
    } else {
      Factor const &f = factors[fr.idx];
      if (f.kind == 0)
        std::snprintf(buf, sizeof buf, "DG %zu\n", f.blocks.size());
      else
        std::snprintf(buf, sizeof buf, "CB %d %d %zu\n", f.nbr, f.nbc, f.blocks.size());
      out += buf;
      appendOffsets(out, "RO", f.rowOff);
      appendOffsets(out, "CO", f.colOff);
      for (int32_t bi : f.blocks) {
        Block const &b = blocks[bi];
        if (f.kind == 0)
          std::snprintf(buf, sizeof buf, "B %d %d\n", b.m, b.n);
        else
          std::snprintf(buf, sizeof buf, "B %d %d %d %d\n", b.ri, b.ci, b.m, b.n);
        out += buf;
      }
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Apply program
// ---------------------------------------------------------------------------
void makeApplyProgram(Plan const &plan, ApplyProgram &prog, int itemRows) {
  prog = ApplyProgram();
  prog.numRows = (int64_t)plan.tgt.perm.size();
  prog.numCols = (int64_t)plan.src.perm.size();

  // stage -> list of (items) built per stage; we first collect per stage
  std::vector<std::vector<ApplyItem>> stItems;
  std::vector<std::vector<std::vector<ApplyContrib>>> stContribs;
  auto stageFor = [&](size_t s) {
    while (stItems.size() <= s) {
      stItems.emplace_back();
      stContribs.emplace_back();
      prog.stageEntries.push_back(0);
      prog.stageRowsIn.push_back(0);
      prog.stageRowsOut.push_back(0);
    }
  };
  struct Region { int64_t t0, t1, base; };
  std::vector<Region> regions;
  int64_t ws = 0;
  double flops = 0;

  // merge (optional): output row -> item of this stage already writing it;
  // a block row whose items exist adds its blocks to them
  auto addBlockRows = [&](size_t stage, int64_t outBase, int64_t rows,
                          std::vector<std::pair<Block const *, int64_t>> const &blks,
                          int inIsX, std::map<int64_t, size_t> *merge) {
    // blks: (block, first input row); all share the block row
    for (int64_t r0 = 0; r0 < rows; r0 += itemRows) {
      std::vector<ApplyContrib> cs;
      for (auto const &bp : blks) {
        ApplyContrib c{};
        c.aOff = bp.first->arenaOff + r0;
        c.lda = bp.first->m;
        c.n = bp.first->n;
        c.inRow = bp.second;
        c.inIsX = inIsX;
        cs.push_back(c);
      }
      stageFor(stage);
      int64_t const outRow = outBase + r0;
      if (merge) {
        auto hit = merge->find(outRow);
        if (hit != merge->end()) {
          auto &dst = stContribs[stage][hit->second];
          dst.insert(dst.end(), cs.begin(), cs.end());
          stItems[stage][hit->second].nContrib = (int32_t)dst.size();
          continue;
        }
        (*merge)[outRow] = stItems[stage].size();
      }
      ApplyItem it{};
      it.outRow = outRow;
      it.rows = (int32_t)std::min<int64_t>(itemRows, rows - r0);
      it.nContrib = (int32_t)cs.size();
      stItems[stage].push_back(it);
      stContribs[stage].push_back(std::move(cs));
    }
  };
  // Products with the same target rows, factor count and last-factor row
  // partition (the butterflies of one target box against the source boxes
  // of the frontier) write their last factor into one region, up to
  // kFinGroup of them: each item of it accumulates the final blocks of all,
  // so the stage writes each target row once per group instead of once per
  // product and the final sum has that many fewer terms.  (Larger groups
  // make items so long that the tensor-core CTAs balance poorly.)
  struct FinGroup {
    int64_t fin;
    int members;
    std::map<int64_t, size_t> items;
  };
  std::map<std::tuple<int64_t, int64_t, size_t, std::vector<int64_t>>, FinGroup> finGroups;

  // walk the HODBF in plan order, assigning workspace regions
  std::vector<std::pair<int32_t, std::pair<int64_t, int64_t>>> st;
  for (size_t r = plan.roots.size(); r-- > 0;)
    st.push_back({plan.roots[r].pnode, {plan.roots[r].rowBase, plan.roots[r].colBase}});
  // (pnode, (rowBase, colBase)) -- rowBase/colBase are absolute tree offsets
  std::vector<std::pair<int32_t, std::pair<int64_t, int64_t>>> order;
  while (!st.empty()) {
    auto cur = st.back();
    st.pop_back();
    PNode const &nd = plan.pnodes[cur.first];
    if (nd.type == 0) {
      for (int i = nd.nr - 1; i >= 0; --i)
        for (int j = nd.nc - 1; j >= 0; --j)
          st.push_back({nd.children[(size_t)i * nd.nc + j],
                        {cur.second.first + nd.rowOff[i], cur.second.second + nd.colOff[j]}});
    } else {
      order.push_back(cur);
    }
  }
  for (auto const &ent : order) {
    PNode const &nd = plan.pnodes[ent.first];
    if (nd.type == 2) {
      Block const &b = plan.blocks[nd.block];
      int64_t base = ws;
      ws += b.m;
      addBlockRows(0, base, b.m, {{&b, b.s0}}, 1, nullptr);
      regions.push_back({b.t0, b.t1, base});
      flops += 8.0 * b.m * b.n;
      prog.stageEntries[0] += (int64_t)b.m * b.n;
      prog.stageRowsIn[0] += b.n;
      prog.stageRowsOut[0] += b.m;
      continue;
    }
    Product const &pr = plan.products[nd.product];
    size_t nf = pr.factors.size();
    // application order: stored index nf-1 first
    int64_t maxMid = 0;
    for (size_t a = 0; a + 1 < nf; ++a) {
      Factor const &f = plan.factors[pr.factors[nf - 1 - a]];
      maxMid = std::max(maxMid, f.rowOff.back());
    }
    int64_t base = ws;
    ws += 2 * maxMid;
    Factor const &lastF = plan.factors[pr.factors[0]];
    auto key = std::make_tuple(pr.t0, pr.t1, nf, lastF.rowOff);
    auto grp = finGroups.find(key);
    bool const joined = grp != finGroups.end() && grp->second.members < kFinGroup;
    if (joined) {
      ++grp->second.members;
    } else {
      grp = finGroups.insert_or_assign(key, FinGroup{ws, 1, {}}).first;
      ws += pr.t1 - pr.t0;
      regions.push_back({pr.t0, pr.t1, grp->second.fin});
    }
    int64_t const fin = grp->second.fin;
    for (size_t a = 0; a < nf; ++a) {
      Factor const &f = plan.factors[pr.factors[nf - 1 - a]];
      bool first = a == 0, last = a + 1 == nf;
      int64_t outBase = last ? fin : base + (int64_t)(a % 2) * maxMid;
      int64_t inBase = first ? pr.s0 : base + (int64_t)((a + 1) % 2) * maxMid;
      // group blocks by block row, keeping stored order within a row
      std::vector<std::vector<std::pair<Block const *, int64_t>>> byRow(f.nbr);
      for (int32_t bi : f.blocks) {
        Block const &b = plan.blocks[bi];
        byRow[b.ri].push_back({&b, inBase + f.colOff[b.ci]});
        flops += 8.0 * b.m * b.n;
      }
      for (int32_t i = 0; i < f.nbr; ++i) {
        if (byRow[i].empty()) continue;
        addBlockRows(a, outBase + f.rowOff[i], f.rowOff[i + 1] - f.rowOff[i], byRow[i],
                     first ? 1 : 0, last ? &grp->second.items : nullptr);
      }
      stageFor(a);
      for (int32_t bi : f.blocks)
        prog.stageEntries[a] += (int64_t)plan.blocks[bi].m * plan.blocks[bi].n;
      prog.stageRowsIn[a] += f.colOff.back();
      if (!(last && joined)) prog.stageRowsOut[a] += f.rowOff.back();
    }
  }
  prog.wsRows = ws;
  prog.flopsPerRhs = flops;

  // flatten stages, each in decreasing order of work (rows x columns): the
  // GPU starts CTAs in launch order, so the longest items start first and the
  // short ones fill in behind them.  Items write disjoint rows, so the order
  // changes no result.
  prog.stageItem0.push_back(0);
  for (size_t s = 0; s < stItems.size(); ++s) {
    std::vector<int64_t> work(stItems[s].size());
    for (size_t k = 0; k < stItems[s].size(); ++k) {
      int64_t cols = 0;
      for (auto const &c : stContribs[s][k]) cols += c.n;
      work[k] = cols * stItems[s][k].rows;
    }
    std::vector<size_t> idx(stItems[s].size());
    for (size_t k = 0; k < idx.size(); ++k) idx[k] = k;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](size_t a, size_t b) { return work[a] > work[b]; });
    for (size_t k : idx) {
      ApplyItem it = stItems[s][k];
      it.contrib0 = (int64_t)prog.contribs.size();
      for (auto const &c : stContribs[s][k]) prog.contribs.push_back(c);
      prog.items.push_back(it);
    }
    prog.stageItem0.push_back((int64_t)prog.items.size());
  }

  // final reduction segments: the common refinement of all region ranges
  std::vector<int64_t> bounds{0, prog.numRows};
  for (auto const &r : regions) {
    bounds.push_back(r.t0);
    bounds.push_back(r.t1);
  }
  std::sort(bounds.begin(), bounds.end());
  bounds.erase(std::unique(bounds.begin(), bounds.end()), bounds.end());
  size_t nseg = bounds.size() - 1;
  std::vector<std::vector<int64_t>> segC(nseg);
  for (auto const &r : regions) {
    prog.sumRows += r.t1 - r.t0;
    size_t a = (size_t)(std::lower_bound(bounds.begin(), bounds.end(), r.t0) - bounds.begin());
    size_t b = (size_t)(std::lower_bound(bounds.begin(), bounds.end(), r.t1) - bounds.begin());
    for (size_t s = a; s < b; ++s) segC[s].push_back(r.base + (bounds[s] - r.t0));
  }
  prog.rowSeg.assign((size_t)prog.numRows, 0);
  prog.segContrib0.push_back(0);
  for (size_t s = 0; s < nseg; ++s) {
    prog.segStart.push_back(bounds[s]);
    for (int64_t i = bounds[s]; i < bounds[s + 1]; ++i) prog.rowSeg[(size_t)i] = (int32_t)s;
    for (int64_t c : segC[s]) prog.segBase.push_back(c);
    prog.segContrib0.push_back((int64_t)prog.segBase.size());
  }
}

std::vector<TcCostModel> tcCandidateModels() {
  return {{60, 1, 29}, {40, 1, 29}, {90, 1, 29}, {60, 3, 29}, {60, 0, 29}, {60, 1, 60}, {0, 0, 100}};
}

void makeTcSchedule(ApplyProgram const &prog, int terms, int ctas, TcSchedule &sc,
                    TcCostModel const &model) {
  sc = TcSchedule();
  sc.ctas = ctas;
  size_t const nStages = prog.stageItem0.empty() ? 0 : prog.stageItem0.size() - 1;
  int64_t arena = 0;
  for (size_t s = 0; s < nStages; ++s) {
    int64_t const a = prog.stageItem0[s], b = prog.stageItem0[s + 1];
    // chunks of every item of the stage, in item order
    std::vector<std::vector<TcChunk>> itemChunks((size_t)(b - a));
    std::vector<int64_t> cost((size_t)(b - a), 0);
    for (int64_t i = a; i < b; ++i) {
      ApplyItem const &it = prog.items[(size_t)i];
      int32_t const mg = (it.rows + 7) / 8;
      auto &ch = itemChunks[(size_t)(i - a)];
      for (int32_t c = 0; c < it.nContrib; ++c) {
        ApplyContrib const &cb = prog.contribs[(size_t)(it.contrib0 + c)];
        int32_t const width = 4 * tcMaxKGroups(mg);
        for (int32_t cj = 0; cj < cb.n; cj += width) {
          TcChunk k{};
          k.nc = std::min(width, cb.n - cj);
          k.kg = (k.nc + 3) / 4;
          k.mg = mg;
          k.rows = it.rows;
          k.inRow = cb.inRow + cj;
          k.inIsX = cb.inIsX;
          k.outRow = it.outRow;
          k.tileOff = arena;
          TcFill f{};
          f.srcOff = cb.aOff + (int64_t)cj * cb.lda;
          f.tileOff = arena;
          f.lda = cb.lda;
          f.rows = it.rows;
          f.nc = k.nc;
          f.kg = k.kg;
          f.mg = mg;
          sc.fills.push_back(f);
          arena += (int64_t)terms * k.kg * mg * 128;
          ch.push_back(k);
          // time of a chunk on the tensor-core kernel, in units of ~10 ns: a
          // fixed hand-off (~0.6 us) plus TERMS MMAs per k-step, or its tile
          // bytes at the CTA's share of HBM bandwidth if that is longer
          // (per-CTA durations measured on the GB300 follow the chunk count,
          // not the bytes)
          int64_t const ksteps = (k.kg + 1) / 2;
          cost[(size_t)(i - a)] += std::max<int64_t>(
              model.perChunk + model.perKstep * terms * ksteps,
              (int64_t)k.kg * mg * terms * model.bytesPct / 100);
        }
      }
      // every block has at least one column, so every item has a chunk
      if (ch.empty()) throw std::runtime_error("apply item without columns");
      ch.front().flags |= kTcFirst;
      ch.back().flags |= kTcLast;
    }
    // longest item first to the least-loaded CTA
    std::vector<size_t> order((size_t)(b - a));
    for (size_t k = 0; k < order.size(); ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t x, size_t y) { return cost[x] > cost[y]; });
    std::vector<std::vector<size_t>> perCta((size_t)ctas);
    std::vector<int64_t> load((size_t)ctas, 0);
    for (size_t k : order) {
      size_t best = 0;
      for (size_t c = 1; c < (size_t)ctas; ++c)
        if (load[c] < load[best]) best = c;
      perCta[best].push_back(k);
      load[best] += cost[k];
    }
    for (int c = 0; c < ctas; ++c) {
      sc.ctaChunk0.push_back((int64_t)sc.chunks.size());
      int64_t n0 = (int64_t)sc.chunks.size();
      for (size_t k : perCta[(size_t)c])
        for (TcChunk const &ch : itemChunks[k]) sc.chunks.push_back(ch);
      sc.maxChunksPerCta =
          std::max<int32_t>(sc.maxChunksPerCta, (int32_t)((int64_t)sc.chunks.size() - n0));
    }
    sc.ctaChunk0.push_back((int64_t)sc.chunks.size());
  }
  sc.arenaBytes = arena;
}

}  // namespace bfg
