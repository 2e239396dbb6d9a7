"""Test infrastructure -- the CPU oracle for the butterfly Helmholtz hot path.

This module restates, on the CPU and in FP64, the reference library's
algorithm for the multilevel butterfly factorization of the 2-D Helmholtz
kernel and its application to vectors.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import
it, and only as the correctness reference (or the timed CPU baseline) --
never as the product path.

Parity pin: the restatement is checked against the reference library itself
(``oracle/build_ref.sh`` compiles the reference's own sources into
``oracle/_ref``; ``tests/golden/make_golden.py`` ran its driver and committed
the outputs as fixtures under ``tests/golden``).  Integer structure
(permutations, ranks, block shapes) must match exactly; numbers match to
rounding.

Arithmetic that must agree bit-for-bit with the reference (bounding circles,
rank estimates, separation tests) goes through glibc's ``hypot``/``log10``/
``ceil`` in the same operation order as the C code.  Kernel entries use
glibc's ``j0/y0/j1/y1`` through ``oracle/c/oracle_kernels.c`` (the
reference's live Bessel path, bessel.c:284-308).  The least-squares
re-expansion uses LAPACK ``zgesvd`` (scipy.linalg, ``lapack_driver="gesvd"``)
like ``bfMatDenseComplexSvd`` (mat_dense_complex.c:1521-1569).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")

EPS_MACH = 2.220446049250313e-16          # def.h:29
MAX_DENSE_MATRIX_SIZE = 128 * 128         # fac_helm2.c:20
TWO_PI = 6.283185307179586                # const.h (BF_TWO_PI)

# layer potentials (layer_pot.h:52-65) and the proxy map (layer_pot.h:87-93)
LP_SINGLE, LP_PV_DOUBLE, LP_PV_NORMAL_DERIV_SINGLE, LP_COMBINED_FIELD = 1, 2, 3, 5
PROXY_LAYER_POT = {LP_SINGLE: LP_SINGLE, LP_PV_DOUBLE: LP_PV_DOUBLE,
                   LP_PV_NORMAL_DERIV_SINGLE: LP_SINGLE,
                   LP_COMBINED_FIELD: LP_COMBINED_FIELD}
USES_SRC_NORMALS = {LP_PV_DOUBLE, LP_COMBINED_FIELD}
USES_TGT_NORMALS = {LP_PV_NORMAL_DERIV_SINGLE}

_libm = ctypes.CDLL("libm.so.6")
for _name in ("hypot", "log10", "ceil"):
    getattr(_libm, _name).restype = ctypes.c_double
_libm.hypot.argtypes = [ctypes.c_double, ctypes.c_double]
_libm.log10.argtypes = [ctypes.c_double]
_libm.ceil.argtypes = [ctypes.c_double]


def c_hypot(a: float, b: float) -> float:
    return _libm.hypot(a, b)


# ---------------------------------------------------------------------------
# native helpers (glibc Bessel kernels + apply port)
# ---------------------------------------------------------------------------
_lib = None


def build_native(force: bool = False) -> str:
    """Compile oracle/c/oracle_kernels.c into oracle/_build (gcc, OpenMP)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    out = os.path.join(BUILD_DIR, "liboracle.so")
    src = os.path.join(HERE, "c", "oracle_kernels.c")
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", src,
                               "-o", out + ".tmp", "-lm"])
        os.replace(out + ".tmp", out)
    return out


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_native())
        _lib.oracle_kernel_matrix.restype = ctypes.c_int
        _lib.oracle_apply_port.restype = ctypes.c_int
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------------------
# RNG: splitmix64 seeding xoshiro256+ (rand.c:19-76, xoshiro256plus.c,
# splitmix64.c -- public-domain generators restated)
# ---------------------------------------------------------------------------
_M64 = (1 << 64) - 1


class RefRng:
    def __init__(self, seed: int = 0):
        self.seed(seed)

    def seed(self, seed: int) -> None:
        x = seed & _M64
        s = []
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & _M64
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
            s.append(z ^ (z >> 31))
        self.s = s

    def next_u64(self) -> int:
        s0, s1, s2, s3 = self.s
        result = (s0 + s3) & _M64
        t = (s1 << 17) & _M64
        s2 ^= s0
        s3 ^= s1
        s1 ^= s2
        s0 ^= s3
        s2 ^= t
        s3 = ((s3 << 45) | (s3 >> 19)) & _M64
        self.s = [s0, s1, s2, s3]
        return result

    def uniform1(self) -> float:
        return (self.next_u64() >> 11) * 2.0 ** -53

    def uniform(self, n: int) -> np.ndarray:
        return np.array([self.uniform1() for _ in range(n)], dtype=np.float64)

    def randn(self, n: int) -> np.ndarray:
        """Box-Muller pairs as in bfRealRandn (rand.c:50-70)."""
        x = self.uniform(2 * (n // 2))
        out = np.empty(n)
        u0, u1 = x[0::2], x[1::2]
        mag = np.array([math.sqrt(-2 * math.log(v)) for v in u0])
        theta = TWO_PI * u1
        out[0:2 * (n // 2):2] = mag * np.cos(theta)
        out[1:2 * (n // 2):2] = mag * np.sin(theta)
        if n % 2 == 1:
            u = self.uniform(2)
            out[n - 1] = math.sqrt(-2 * math.log(u[0])) * math.cos(TWO_PI * u[1])
        return out

    def complex_randn(self, n: int) -> np.ndarray:
        return self.randn(2 * n).view(np.complex128)


# ---------------------------------------------------------------------------
# geometry generators for the workloads
# ---------------------------------------------------------------------------
def uniform_square_points(n: int, seed: int) -> np.ndarray:
    """n points iid uniform in [-1,1]^2: x then y from successive draws."""
    rng = RefRng(seed)
    u = rng.uniform(2 * n)
    return (2 * u - 1).reshape(n, 2)


def curve_points(kind: str, n: int, a: float = 3.0, b: float = 2.0,
                 amp: float = 0.5, lobes: int = 5) -> np.ndarray:
    """Equispaced in the curve parameter theta_i = (2 pi / n) i, as
    bfCircle2SamplePoints does (circle.c:12-34)."""
    scale = TWO_PI / n
    theta = scale * np.arange(n, dtype=np.float64)
    if kind == "circle":
        return np.stack([a * np.cos(theta), a * np.sin(theta)], axis=1)
    if kind == "ellipse":
        return np.stack([a * np.cos(theta), b * np.sin(theta)], axis=1)
    if kind == "star":
        r = a + amp * np.cos(lobes * theta)
        return np.stack([r * np.cos(theta), r * np.sin(theta)], axis=1)
    raise ValueError(kind)


# ---------------------------------------------------------------------------
# quadtree (quadtree.c:80-98, quadtree_node.c:123-330, tree_node.c:140-186)
# ---------------------------------------------------------------------------
class QNode:
    __slots__ = ("bbox", "split", "offset", "child", "depth", "parent",
                 "index", "i0", "i1")

    def __init__(self, bbox, depth, parent, index):
        self.bbox = bbox            # (xmin, ymin, xmax, ymax)
        self.split = ((bbox[0] + bbox[2]) / 2, (bbox[1] + bbox[3]) / 2)
        self.offset = None
        self.child = [None, None, None, None]
        self.depth = depth
        self.parent = parent
        self.index = index
        self.i0 = self.i1 = 0

    @property
    def is_leaf(self) -> bool:
        return all(c is None for c in self.child)

    @property
    def num_points(self) -> int:
        return self.i1 - self.i0

    def children(self):
        return [c for c in self.child if c is not None]

    def circle(self):
        """bfQuadtreeNodeGetBoundingCircle (quadtree_node.c:321-330)."""
        xmin, ymin, xmax, ymax = self.bbox
        r = c_hypot(xmax - xmin, ymax - ymin) / 2
        return ((xmin + xmax) / 2, (ymin + ymax) / 2, r)


class Quadtree:
    """Quadtree over ``points`` (N,2).  ``leaf_size`` generalises the
    reference's fixed LEAF_SIZE_THRESHOLD = 1 (quadtree_node.c:17): a node
    with more than ``leaf_size`` points is split."""

    def __init__(self, points: np.ndarray, leaf_size: int = 1):
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        n = len(points)
        self.perm = list(range(n))
        px = self.points[:, 0].tolist()
        py = self.points[:, 1].tolist()
        # bounding box (points.c:415-430), rescaled to a square (bbox.c:18-30)
        xmin, xmax = min(px), max(px)
        ymin, ymax = min(py), max(py)
        w, h = xmax - xmin, ymax - ymin
        # bfBbox2RescaleToSquare (bbox.c:18-30) divides by a zero side for one
        # point or collinear points; there the limit of its formula (or, for a
        # single point, a unit square) is used instead
        if w == 0 and h == 0:
            xmin, xmax, ymin, ymax = xmin - 0.5, xmax + 0.5, ymin - 0.5, ymax + 0.5
        elif w > h:
            c = (ymin + ymax) / 2
            if h > 0:
                ymin, ymax = w * (ymin - c) / h + c, w * (ymax - c) / h + c
            else:
                ymin, ymax = c - w / 2, c + w / 2
        else:
            c = (xmin + xmax) / 2
            if w > 0:
                xmin, xmax = h * (xmin - c) / w + c, h * (xmax - c) / w + c
            else:
                xmin, xmax = c - h / 2, c + h / 2
        self.root = QNode((xmin, ymin, xmax, ymax), 0, None, None)
        self.leaf_size = leaf_size
        self._build(self.root, px, py, 0, n)

    def _build(self, node, px, py, i0, i1):
        perm = self.perm
        sx, sy = node.split
        node.i0, node.i1 = i0, i1
        off = [i0, 0, 0, 0, i1]
        preds = (lambda x, y: x <= sx and y <= sy,
                 lambda x, y: x <= sx and y > sy,
                 lambda x, y: x > sx and y <= sy)
        for q, pred in enumerate(preds):
            # the sift of quadtree_node.c:148-194
            i = off[q]
            while i < i1 and pred(px[perm[i]], py[perm[i]]):
                i += 1
            j = i if i == i1 else i + 1
            while j < i1:
                if pred(px[perm[j]], py[perm[j]]) and not pred(px[perm[i]], py[perm[i]]):
                    perm[i], perm[j] = perm[j], perm[i]
                    i += 1
                j += 1
            off[q + 1] = i
        node.offset = off
        xmin, ymin, xmax, ymax = node.bbox
        boxes = ((xmin, ymin, sx, sy), (xmin, sy, sx, ymax),
                 (sx, ymin, xmax, sy), (sx, sy, xmax, ymax))
        for q in range(4):
            cnt = off[q + 1] - off[q]
            if cnt == 0:
                continue
            ch = QNode(boxes[q], node.depth + 1, node, q)
            ch.i0, ch.i1 = off[q], off[q + 1]
            if cnt > self.leaf_size:
                self._build(ch, px, py, off[q], off[q + 1])
            node.child[q] = ch

    def levels_below(self, node):
        """LR level order grouped by depth (tree_level_iter.c:12-88)."""
        nodes = [node]
        i = 0
        while i < len(nodes):
            nodes.extend(nodes[i].children())
            i += 1
        levels, cur = [], []
        for nd in nodes:
            if cur and nd.depth != cur[0].depth:
                levels.append(cur)
                cur = []
            cur.append(nd)
        levels.append(cur)
        return levels

    def tree_points(self) -> np.ndarray:
        return self.points[np.asarray(self.perm, dtype=np.int64)]

    def max_depth(self) -> int:
        return max(lv[0].depth for lv in self.levels_below(self.root))


def rank_est(k: float, c1, c2, C: float = 1.0, eps: float = 1e-15) -> int:
    """bfHelm2RankEstForTwoCircles (helm2.c:14-36), same operation order."""
    r1, r2 = c1[2], c2[2]
    R = c_hypot(c2[0] - c1[0], c2[1] - c1[1])
    d = R - r1 - r2
    if not (r1 > 0 and r2 > 0 and R > 0 and d > 0):
        raise ValueError("rank estimate on overlapping circles")
    p = k * r1 * r2 / d - C * _libm.log10(eps)
    return int(_libm.ceil(p))


def nodes_separated(src: QNode, tgt: QNode) -> bool:
    """bfQuadtreeNodesAreSeparated (quadtree_node.c:393-401)."""
    c1, c2 = src.circle(), tgt.circle()
    R = c_hypot(c2[0] - c1[0], c2[1] - c1[1])
    return R > c1[2] + c2[2] + 1e1 * EPS_MACH


# ---------------------------------------------------------------------------
# planner (fac_helm2.c:42-1002): the block structure of the factorization
# ---------------------------------------------------------------------------
@dataclass
class Block:
    """One stored block.  ``kind``: 'first', 'middle', 'last' or 'dense'.
    Geometry needed to fill it:
      first : src points = tree range [p0,p1) of the source tree; proxy
              circles ceq (equivalent sources, m points) and cchk (check
              points, m points)
      middle: corig (source-child circle, n points), ceq (m points),
              cchk (target-child circle, m points)
      last  : ceq (source circle, n points); tgt points = tree range
      dense : src range and tgt range"""
    kind: str
    m: int
    n: int
    ri: int = 0          # block row index (COO) / block index (diag)
    ci: int = 0
    src_range: tuple = (0, 0)
    tgt_range: tuple = (0, 0)
    corig: tuple = None
    ceq: tuple = None
    cchk: tuple = None
    data: np.ndarray = None


@dataclass
class Factor:
    kind: str                       # 'DG' (block diagonal) or 'CB' (block COO)
    nbr: int
    nbc: int
    row_off: list
    col_off: list
    blocks: list = field(default_factory=list)


@dataclass
class Product:
    factors: list                   # stored order: [evaluation, ..., first]
    tgt_range: tuple
    src_range: tuple


@dataclass
class Dense:
    block: Block


@dataclass
class BlockDense:
    nr: int
    nc: int
    row_off: list
    col_off: list
    children: list                  # row-major


class Planner:
    """Walks node pairs exactly as bfFacHelm2MakeMultilevel does."""

    def __init__(self, k: float, src: Quadtree, tgt: Quadtree,
                 eps: float = 1e-15, leaf_guard: bool = True):
        self.k = k
        self.src = src
        self.tgt = tgt
        self.eps = eps
        self.leaf_guard = leaf_guard

    # bfFacHelm2MakeMultilevel (fac_helm2.c:943-1002) starts from the nodes
    # at depth 2; a leaf shallower than that (tiny point sets) would leave its
    # points out of every block, so it joins the list in tree order (for
    # trees whose depth-1 nodes are all split this is the reference's list)
    @staticmethod
    def _frontier(tree):
        out = []

        def walk(nd):
            kids = nd.children()
            if nd.depth == 2 or not kids:
                out.append(nd)
            else:
                for ch in kids:
                    walk(ch)
        for ch in tree.root.children():
            walk(ch)
        return out

    def plan(self):
        return self._rec(self._frontier(self.src), self._frontier(self.tgt))

    # facHelm2MakeMultilevel_rec (fac_helm2.c:860-941)
    def _rec(self, src_nodes, tgt_nodes):
        nr, nc = len(tgt_nodes), len(src_nodes)
        children, row_off, col_off = [], [0], [0]
        for i, t in enumerate(tgt_nodes):
            m = t.num_points
            for j, s in enumerate(src_nodes):
                n = s.num_points
                separated = nodes_separated(s, t)
                leafy = self.leaf_guard and (s.is_leaf or t.is_leaf)
                if m * n < MAX_DENSE_MATRIX_SIZE or leafy:
                    mat = self._dense(s, t)
                elif separated:
                    mat = self._separated(s, t)
                else:
                    mat = self._rec(s.children(), t.children())
                children.append(mat)
                if i == 0:
                    col_off.append(col_off[-1] + n)
            row_off.append(row_off[-1] + m)
        return BlockDense(nr, nc, row_off, col_off, children)

    def _dense(self, s, t):
        return Dense(Block("dense", t.num_points, s.num_points,
                           src_range=(s.i0, s.i1), tgt_range=(t.i0, t.i1)))

    def _rank(self, c1, c2):
        return rank_est(self.k, c1, c2, 1.0, self.eps)

    def _all_ranks_ok(self, tgt_node, src_level):
        """allRankEstimatesAreOK (fac_helm2.c:511-530)."""
        tc = tgt_node.circle()
        for s in src_level:
            if self._rank(tc, s.circle()) > s.num_points:
                return False
        return True

    # bfFacHelm2Prepare (fac_helm2.c:551-651)
    def _prepare(self, s, t):
        num_src = s.num_points
        src_levels = self.src.levels_below(s)
        tgt_levels = self.tgt.levels_below(t)
        internal = lambda lv: all(not nd.is_leaf for nd in lv)
        npts = lambda lv: sum(nd.num_points for nd in lv)
        max_allow = t.depth
        if not internal(tgt_levels[0]):
            raise RuntimeError("target node is a leaf")
        ti = 1
        while ti < len(tgt_levels) and internal(tgt_levels[ti]):
            max_allow += 1
            ti += 1
        si = len(src_levels) - 1
        src_depth = src_levels[si][0].depth
        tgt_depth = t.depth
        guard = 0

        def step():
            nonlocal si, src_depth, guard
            if si > 0:
                si -= 1
            src_depth -= 1
            guard += 1
            if guard > 10000:
                raise RuntimeError("level search did not terminate")

        while src_depth > max_allow:
            step()
        while npts(src_levels[si]) != num_src:
            step()
        while not internal(src_levels[si]):
            step()
        while src_depth > tgt_depth and not self._all_ranks_ok(t, src_levels[si]):
            step()
        nf = (src_depth - tgt_depth + 2) if self._all_ranks_ok(t, src_levels[si]) else 0
        return nf, src_levels, si, tgt_levels

    # facHelm2MakeMultilevel_separated + bfFacHelm2Make (fac_helm2.c:653-704, 777-804)
    def _separated(self, s, t):
        nf, src_levels, si, tgt_levels = self._prepare(s, t)
        if nf == 0:
            return self._dense(s, t)
        ti = 0
        fac = [self._first(src_levels[si], tgt_levels[ti])]
        for _ in range(1, nf - 1):
            si = max(si - 1, 0)
            fac.append(self._middle(fac[-1], src_levels[si], tgt_levels[ti]))
            ti = min(ti + 1, len(tgt_levels) - 1)
        fac.append(self._last(fac[-1], src_levels[si], tgt_levels[ti]))
        return Product(list(reversed(fac)), (t.i0, t.i1), (s.i0, s.i1))

    # makeFirstFactor (fac_helm2.c:42-160)
    def _first(self, src_level, tgt_level):
        assert len(tgt_level) == 1
        tc = tgt_level[0].circle()
        row_off, col_off, blocks = [0], [0], []
        for i, sn in enumerate(src_level):
            sc = sn.circle()
            p = self._rank(sc, tc)
            blocks.append(Block("first", p, sn.num_points, ri=i, ci=i,
                                src_range=(sn.i0, sn.i1), ceq=sc, cchk=tc))
            row_off.append(row_off[-1] + p)
            col_off.append(col_off[-1] + sn.num_points)
        return Factor("DG", len(blocks), len(blocks), row_off, col_off, blocks)

    @staticmethod
    def _block_rows(f: Factor, i: int) -> int:
        return f.row_off[i + 1] - f.row_off[i]

    # makeFactor (fac_helm2.c:222-401)
    def _middle(self, prev: Factor, src_level, tgt_level):
        n_tgt_nodes = len(tgt_level)
        n_tgt_children = sum(len(nd.children()) for nd in tgt_level)
        n_src_nodes = len(src_level)
        n_src_children = sum(len(nd.children()) for nd in src_level)
        nbr = n_tgt_children * n_src_nodes
        nbc = n_src_children * n_tgt_nodes
        assert nbc == prev.nbr
        col_off = [0]
        for j in range(nbc):
            col_off.append(col_off[-1] + self._block_rows(prev, j))
        rows = [None] * nbr
        entries = []
        i_offset = 0
        for ti, tn in enumerate(tgt_level):
            tcirc = tn.circle()
            for tch in tn.children():
                tchc = tch.circle()
                j = ti * n_src_children
                for si_, sn in enumerate(src_level):
                    scirc = sn.circle()
                    for sch in sn.children():
                        schc = sch.circle()
                        i = i_offset + si_
                        rank_or = self._rank(schc, tcirc)
                        rank_eq = self._rank(scirc, tchc)
                        rank = rank_or if rank_or > rank_eq else rank_eq
                        if rows[i] is None or rank > rows[i]:
                            rows[i] = rank
                        entries.append((i, j, schc, scirc, tchc))
                        j += 1
                i_offset += n_src_nodes
        row_off = [0]
        for i in range(nbr):
            row_off.append(row_off[-1] + rows[i])
        f = Factor("CB", nbr, nbc, row_off, col_off)
        for (i, j, schc, scirc, tchc) in entries:
            m = row_off[i + 1] - row_off[i]
            n = col_off[j + 1] - col_off[j]
            f.blocks.append(Block("middle", m, n, ri=i, ci=j,
                                  corig=schc, ceq=scirc, cchk=tchc))
        return f

    # makeLastFactor (fac_helm2.c:403-509)
    def _last(self, prev: Factor, src_level, tgt_level):
        assert len(src_level) == 1
        sc = src_level[0].circle()
        row_off, col_off, blocks = [0], [0], []
        for i, tn in enumerate(tgt_level):
            pr = self._block_rows(prev, i)
            blocks.append(Block("last", tn.num_points, pr, ri=i, ci=i,
                                tgt_range=(tn.i0, tn.i1), ceq=sc))
            row_off.append(row_off[-1] + tn.num_points)
            col_off.append(col_off[-1] + pr)
        return Factor("DG", len(blocks), len(blocks), row_off, col_off, blocks)


def plan_text(node) -> str:
    """The plan grammar written by oracle/ref_dump.c."""
    out = []

    def offs(tag, v):
        out.append(tag + "".join(" %d" % x for x in v))

    def rec(nd):
        if isinstance(nd, BlockDense):
            out.append("BD %d %d" % (nd.nr, nd.nc))
            offs("RO", nd.row_off)
            offs("CO", nd.col_off)
            for ch in nd.children:
                rec(ch)
        elif isinstance(nd, Product):
            out.append("PR %d" % len(nd.factors))
            for f in nd.factors:
                rec(f)
        elif isinstance(nd, Factor):
            if nd.kind == "DG":
                out.append("DG %d" % len(nd.blocks))
            else:
                out.append("CB %d %d %d" % (nd.nbr, nd.nbc, len(nd.blocks)))
            offs("RO", nd.row_off)
            offs("CO", nd.col_off)
            for b in nd.blocks:
                if nd.kind == "DG":
                    out.append("B %d %d" % (b.m, b.n))
                else:
                    out.append("B %d %d %d %d" % (b.ri, b.ci, b.m, b.n))
        elif isinstance(nd, Dense):
            out.append("DC %d %d" % (nd.block.m, nd.block.n))
        else:
            raise TypeError(nd)

    rec(node)
    return "\n".join(out) + "\n"


def iter_blocks(node):
    """All stored blocks in plan order (the order of blocks.c128)."""
    if isinstance(node, BlockDense):
        for ch in node.children:
            yield from iter_blocks(ch)
    elif isinstance(node, Product):
        for f in node.factors:
            yield from f.blocks
    elif isinstance(node, Dense):
        yield node.block


# ---------------------------------------------------------------------------
# numeric fill (helm2.c:93-365, mat_dense_complex.c:1768-1849)
# ---------------------------------------------------------------------------
def circle_points(circ, n):
    """bfCircle2SamplePoints / SampleUnitNormals (circle.c:12-58)."""
    pts = np.empty((n, 2))
    nrm = np.empty((n, 2))
    lib().oracle_circle_points(ctypes.c_double(circ[0]), ctypes.c_double(circ[1]),
                               ctypes.c_double(circ[2]), ctypes.c_int64(n),
                               _ptr(pts), _ptr(nrm))
    return pts, nrm


@dataclass
class Helm2:
    k: float
    layer_pot: int = LP_SINGLE
    alpha: complex = 0j
    beta: complex = 0j


def kernel_matrix(helm: Helm2, src, tgt, src_normals=None, tgt_normals=None):
    """bfHelm2GetKernelMatrix (helm2.c:282-319): rows = targets."""
    src = np.ascontiguousarray(src, dtype=np.float64)
    tgt = np.ascontiguousarray(tgt, dtype=np.float64)
    m, n = len(tgt), len(src)
    out = np.empty((m, n), dtype=np.complex128)
    sx, sy = np.ascontiguousarray(src[:, 0]), np.ascontiguousarray(src[:, 1])
    tx, ty = np.ascontiguousarray(tgt[:, 0]), np.ascontiguousarray(tgt[:, 1])
    snx = sny = tnx = tny = None
    if src_normals is not None:
        snx = np.ascontiguousarray(src_normals[:, 0]); sny = np.ascontiguousarray(src_normals[:, 1])
    if tgt_normals is not None:
        tnx = np.ascontiguousarray(tgt_normals[:, 0]); tny = np.ascontiguousarray(tgt_normals[:, 1])
    rc = lib().oracle_kernel_matrix(
        ctypes.c_int(helm.layer_pot), ctypes.c_double(helm.k),
        ctypes.c_double(helm.alpha.real), ctypes.c_double(helm.alpha.imag),
        ctypes.c_double(helm.beta.real), ctypes.c_double(helm.beta.imag),
        _ptr(tx), _ptr(ty), _ptr(tnx), _ptr(tny), ctypes.c_int64(m),
        _ptr(sx), _ptr(sy), _ptr(snx), _ptr(sny), ctypes.c_int64(n), _ptr(out))
    if rc != 0:
        raise NotImplementedError("layer potential %d" % helm.layer_pot)
    return out


def lstsq_pinv(A: np.ndarray, B: np.ndarray, rcut: str = "reference",
               tol: float = None, return_terms: bool = False):
    """bfMatDenseComplexDenseComplexLstSq (mat_dense_complex.c:1768-1849):
    X = V_k S_k^-1 U_k^H B with k = #{sigma_i >= max(m,n) eps sigma_0 + eps}.
    ``rcut="relative"`` keeps sigma_i >= tol * sigma_0 instead (the
    truncation rule of bfTruncSpecGetNumTerms, linalg.c:26-36).
    ``return_terms``: also the number of kept terms and the singular
    values."""
    import scipy.linalg
    m, n = A.shape
    U, S, VH = scipy.linalg.svd(A, full_matrices=False, lapack_driver="gesvd")
    if rcut == "reference":
        t = max(m, n) * EPS_MACH * S[0] + EPS_MACH
    else:
        t = tol * S[0]
    k = 0
    while k < len(S) and not S[k] < t:
        k += 1
    tmp1 = U[:, :k].conj().T @ B
    tmp2 = tmp1 / S[:k, None]
    X = VH[:k, :].conj().T @ tmp2
    return (X, k, S) if return_terms else X


def sketch_width(k: float, ceq, cchk, m: int, scale: float = 1.1, pad: int = 40) -> int:
    """Initial width of the library's randomized re-expansion for a block
    with rank estimate m: scale * k r1 r2 / R + pad rounded up to 32, at most
    m (R: distance of the equivalent and check circles' centres).  The rank
    estimate of helm2.c:14-36 divides by R - r1 - r2 instead."""
    R = float(np.hypot(ceq[0] - cchk[0], ceq[1] - cchk[1]))
    est = k * ceq[2] * cchk[2] / R if R > 0 else float(m)
    w = int(np.ceil((scale * est + pad) / 32.0)) * 32
    return m if w >= m else max(32, w)


def sketch_pinv(A: np.ndarray, B: np.ndarray, width: int, tol: float,
                seed: int = 0):
    """The randomized re-expansion the library runs on the GPU, restated with
    numpy's LAPACK for the CPU checks (test infrastructure): X ~ pinv_cut(A) B
    with the relative cut sigma_i >= tol sigma_0 (linalg.c:26-36) taken on the
    singular values of A restricted to the range of a Gaussian sketch
    A Omega (Halko, Martinsson, Tropp 2011, algorithms 4.1 and 5.1):
    Q = qr(A Omega), Q2 R2 = qr(A^H Q), R2^H = U S V^H, so A ~ (Q U) S (Q2 V)^H
    and X = Q2 V diag(w) S U^H Q^H B.  Returns (X, sigma_min / sigma_max), the
    second being the library's capture test (the sketch reached A's rounding
    floor when it is tiny)."""
    p = A.shape[0]
    rng = np.random.default_rng(seed)
    om = rng.standard_normal((p, width)) + 1j * rng.standard_normal((p, width))
    Q, _ = np.linalg.qr(A @ om)
    Q2, R2 = np.linalg.qr(A.conj().T @ Q)
    U, S, VH = np.linalg.svd(R2.conj().T)
    w = np.where(S >= tol * S.max(), 1.0 / S ** 2, 0.0)
    T = U * S
    X = Q2 @ (VH.conj().T @ (w[:, None] * (T.conj().T @ (Q.conj().T @ B))))
    return X, float(S.min() / S.max())


class Factorization:
    """The oracle's butterfly factorization: plan + filled blocks."""

    def __init__(self, helm: Helm2, src_pts, tgt_pts, src_normals=None,
                 tgt_normals=None, leaf_size: int = 1, eps: float = 1e-15,
                 rcut: str = "reference", fill: bool = True):
        self.helm = helm
        self.src_tree = Quadtree(src_pts, leaf_size)
        self.tgt_tree = Quadtree(tgt_pts, leaf_size)
        self.src_normals = src_normals
        self.tgt_normals = tgt_normals
        self.eps = eps
        self.rcut = rcut
        self.root = Planner(helm.k, self.src_tree, self.tgt_tree, eps).plan()
        sp = np.asarray(self.src_tree.perm, dtype=np.int64)
        tp = np.asarray(self.tgt_tree.perm, dtype=np.int64)
        self.src_perm, self.tgt_perm = sp, tp
        self.src_tree_pts = self.src_tree.points[sp]
        self.tgt_tree_pts = self.tgt_tree.points[tp]
        self.src_tree_nrm = None if src_normals is None else np.asarray(src_normals)[sp]
        self.tgt_tree_nrm = None if tgt_normals is None else np.asarray(tgt_normals)[tp]
        if fill:
            for b in iter_blocks(self.root):
                self.fill_block(b)

    def plan_text(self) -> str:
        return plan_text(self.root)

    def blocks(self):
        return list(iter_blocks(self.root))

    def fill_block(self, b: Block) -> None:
        h = self.helm
        proxy = Helm2(h.k, PROXY_LAYER_POT[h.layer_pot], h.alpha, h.beta)
        sn_all, tn_all = self.src_tree_nrm, self.tgt_tree_nrm
        if b.kind == "dense":
            s0, s1 = b.src_range
            t0, t1 = b.tgt_range
            b.data = kernel_matrix(
                h, self.src_tree_pts[s0:s1], self.tgt_tree_pts[t0:t1],
                None if sn_all is None or h.layer_pot not in USES_SRC_NORMALS else sn_all[s0:s1],
                None if tn_all is None or h.layer_pot not in USES_TGT_NORMALS else tn_all[t0:t1])
        elif b.kind == "last":
            t0, t1 = b.tgt_range
            eq_pts, eq_nrm = circle_points(b.ceq, b.n)
            b.data = kernel_matrix(
                h, eq_pts, self.tgt_tree_pts[t0:t1],
                eq_nrm if h.layer_pot in USES_SRC_NORMALS else None,
                None if tn_all is None or h.layer_pot not in USES_TGT_NORMALS else tn_all[t0:t1])
        else:
            if b.kind == "first":
                s0, s1 = b.src_range
                orig_pts = self.src_tree_pts[s0:s1]
                orig_nrm = None if sn_all is None else sn_all[s0:s1]
            else:
                orig_pts, orig_nrm = circle_points(b.corig, b.n)
            eq_pts, eq_nrm = circle_points(b.ceq, b.m)
            chk_pts, _ = circle_points(b.cchk, b.m)
            use_n = proxy.layer_pot in USES_SRC_NORMALS
            z_orig = kernel_matrix(proxy, orig_pts, chk_pts, orig_nrm if use_n else None)
            z_equiv = kernel_matrix(proxy, eq_pts, chk_pts, eq_nrm if use_n else None)
            b.data = lstsq_pinv(z_equiv, z_orig, self.rcut, self.eps)

    # ---------------- apply (mat.c:183 -> mat_block_dense.c:512 ...) ----------
    def apply(self, X: np.ndarray) -> np.ndarray:
        """Y = A X, rows of X and Y in tree order (the reference's bfMatMul
        contract; callers permute)."""
        X = np.asarray(X, dtype=np.complex128)
        if X.ndim == 1:
            return self.apply(X[:, None])[:, 0]
        return self._apply(self.root, X)

    def _apply(self, nd, X):
        if isinstance(nd, BlockDense):
            Y = np.zeros((nd.row_off[-1], X.shape[1]), dtype=np.complex128)
            for i in range(nd.nr):
                for j in range(nd.nc):
                    ch = nd.children[i * nd.nc + j]
                    Y[nd.row_off[i]:nd.row_off[i + 1]] += self._apply(
                        ch, X[nd.col_off[j]:nd.col_off[j + 1]])
            return Y
        if isinstance(nd, Dense):
            return nd.block.data @ X
        if isinstance(nd, Product):
            V = X
            for f in reversed(nd.factors):
                W = np.zeros((f.row_off[-1], X.shape[1]), dtype=np.complex128)
                for b in f.blocks:
                    r0, r1 = f.row_off[b.ri], f.row_off[b.ri + 1]
                    c0, c1 = f.col_off[b.ci], f.col_off[b.ci + 1]
                    W[r0:r1] += b.data @ V[c0:c1]
                V = W
            return V
        raise TypeError(nd)

    # ---------------- flat description for the C apply port -----------------
    def port_arrays(self):
        """Terms / factors / blocks arrays for oracle_apply_port."""
        terms, factors, fblocks, chunks = [], [], [], []
        off = [0]

        def add_data(a):
            a = np.ascontiguousarray(a, dtype=np.complex128)
            chunks.append(a.ravel())
            o = off[0]
            off[0] += a.size
            return o

        def rec(nd, r0, c0, group):
            if isinstance(nd, BlockDense):
                for i in range(nd.nr):
                    for j in range(nd.nc):
                        g = group if group is not None else i
                        rec(nd.children[i * nd.nc + j], r0 + nd.row_off[i],
                            c0 + nd.col_off[j], g)
            elif isinstance(nd, Dense):
                b = nd.block
                terms.append((0, group, r0, c0, b.m, b.n, 0, 0, add_data(b.data)))
            else:
                ff = len(factors)
                for f in reversed(nd.factors):
                    fb = len(fblocks)
                    for b in f.blocks:
                        fblocks.append((f.row_off[b.ri], f.col_off[b.ci], b.m, b.n,
                                        add_data(b.data)))
                    factors.append((f.row_off[-1], f.col_off[-1], fb, len(f.blocks), 0))
                m = nd.tgt_range[1] - nd.tgt_range[0]
                n = nd.src_range[1] - nd.src_range[0]
                terms.append((1, group, r0, c0, m, n, ff, len(nd.factors), 0))

        rec(self.root, 0, 0, None)
        term_dt = np.dtype([("kind", "<i4"), ("group", "<i4"), ("tgtRow", "<i8"),
                            ("srcRow", "<i8"), ("m", "<i4"), ("n", "<i4"),
                            ("firstFactor", "<i4"), ("numFactors", "<i4"),
                            ("dataOff", "<i8")])
        fac_dt = np.dtype([("rows", "<i4"), ("cols", "<i4"), ("firstBlock", "<i8"),
                           ("numBlocks", "<i4"), ("pad", "<i4")])
        blk_dt = np.dtype([("rowOff", "<i8"), ("colOff", "<i8"), ("m", "<i4"),
                           ("n", "<i4"), ("dataOff", "<i8")])
        return (np.array(terms, dtype=term_dt), np.array(factors, dtype=fac_dt),
                np.array(fblocks, dtype=blk_dt),
                np.concatenate(chunks) if chunks else np.zeros(0, np.complex128))

    def num_entries(self) -> int:
        return sum(b.m * b.n for b in iter_blocks(self.root))


class ApplyPort:
    """The reference's apply restated in C (oracle_kernels.c), timed as the
    CPU baseline."""

    def __init__(self, fac: Factorization = None):
        self.col_major = 0
        if fac is not None:
            self.terms, self.factors, self.fblocks, self.data = fac.port_arrays()
            self.nrows = len(fac.tgt_perm)

    @classmethod
    def from_plan(cls, text: str, data: np.ndarray, col_major: bool, wrap: bool = False):
        """Port over the structure of a plan text (oracle_dump grammar) with
        the blocks stored back to back in plan order in ``data`` --
        row-major, or column-major as in the GPU arena.  ``wrap``: ``data``
        is a stand-in shorter than the plan (timing only: values do not
        change the cost); block offsets wrap around it, every block reading
        its own contiguous m*n entries of it.  It must hold the largest
        block; far larger than the host caches, it streams from memory as
        the real factors would."""
        root = parse_plan(text)
        off = [0]

        def take(m, n):
            o = off[0]
            off[0] += m * n
            if wrap:
                span = data.size - m * n + 1
                if span <= 0:
                    raise ValueError("stand-in data shorter than a block")
                o %= span
            return o

        terms, factors, fblocks = [], [], []

        def rec(nd, r0, c0, group):
            if isinstance(nd, BlockDense):
                for i in range(nd.nr):
                    for j in range(nd.nc):
                        rec(nd.children[i * nd.nc + j], r0 + nd.row_off[i],
                            c0 + nd.col_off[j], group if group is not None else i)
            elif isinstance(nd, Dense):
                b = nd.block
                terms.append((0, group, r0, c0, b.m, b.n, 0, 0, take(b.m, b.n)))
            else:
                ff = len(factors)
                offs = [[take(b.m, b.n) for b in f.blocks] for f in nd.factors]
                for f, fo in zip(reversed(nd.factors), reversed(offs)):
                    fb = len(fblocks)
                    for b, o in zip(f.blocks, fo):
                        fblocks.append((f.row_off[b.ri], f.col_off[b.ci], b.m, b.n, o))
                    factors.append((f.row_off[-1], f.col_off[-1], fb, len(f.blocks), 0))
                m = nd.factors[0].row_off[-1]
                n = nd.factors[-1].col_off[-1]
                terms.append((1, group, r0, c0, m, n, ff, len(nd.factors), 0))

        rec(root, 0, 0, None)
        if off[0] > data.size and not wrap:
            raise ValueError("block data shorter than the plan")
        p = cls()
        term_dt = np.dtype([("kind", "<i4"), ("group", "<i4"), ("tgtRow", "<i8"),
                            ("srcRow", "<i8"), ("m", "<i4"), ("n", "<i4"),
                            ("firstFactor", "<i4"), ("numFactors", "<i4"),
                            ("dataOff", "<i8")])
        fac_dt = np.dtype([("rows", "<i4"), ("cols", "<i4"), ("firstBlock", "<i8"),
                           ("numBlocks", "<i4"), ("pad", "<i4")])
        blk_dt = np.dtype([("rowOff", "<i8"), ("colOff", "<i8"), ("m", "<i4"),
                           ("n", "<i4"), ("dataOff", "<i8")])
        p.terms = np.array(terms, dtype=term_dt)
        p.factors = np.array(factors, dtype=fac_dt)
        p.fblocks = np.array(fblocks, dtype=blk_dt)
        p.data = np.ascontiguousarray(data, dtype=np.complex128)
        p.nrows = root.row_off[-1]
        p.col_major = 1 if col_major else 0
        return p

    def __call__(self, X: np.ndarray, nthreads: int = 1) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.complex128)
        if X.ndim == 1:
            X = X[:, None]
        R = X.shape[1]
        Y = np.empty((self.nrows, R), dtype=np.complex128)
        rc = lib().oracle_apply_port(
            ctypes.c_int64(len(self.terms)), _ptr(self.terms), _ptr(self.factors),
            _ptr(self.fblocks), _ptr(self.data), _ptr(X), _ptr(Y),
            ctypes.c_int64(self.nrows), ctypes.c_int64(R), ctypes.c_int32(nthreads),
            ctypes.c_int32(self.col_major))
        if rc != 0:
            raise MemoryError("apply port failed")
        return Y


def parse_plan_entries(text: str) -> int:
    """Complex entries over all stored blocks of a plan text: the "B" lines
    of block-diagonal (m n) and block-COO (i j m n) factors and the dense
    blocks ("DC m n")."""
    total = 0
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "B":
            total += int(t[-2]) * int(t[-1])
        elif t[0] == "DC":
            total += int(t[1]) * int(t[2])
    return total


def parse_plan(text: str):
    """Inverse of plan_text: the structure (no geometry) of a plan dump."""
    lines = text.split("\n")
    pos = [0]

    def nxt():
        toks = lines[pos[0]].split()
        pos[0] += 1
        return toks

    def ints(toks):
        return [int(t) for t in toks[1:]]

    def rec():
        t = nxt()
        if t[0] == "BD":
            nr, nc = int(t[1]), int(t[2])
            ro, co = ints(nxt()), ints(nxt())
            return BlockDense(nr, nc, ro, co, [rec() for _ in range(nr * nc)])
        if t[0] == "PR":
            return Product([rec() for _ in range(int(t[1]))], None, None)
        if t[0] == "DG":
            nb = int(t[1])
            ro, co = ints(nxt()), ints(nxt())
            blocks = []
            for i in range(nb):
                _, m, n = nxt()
                blocks.append(Block("diag", int(m), int(n), ri=i, ci=i))
            return Factor("DG", nb, nb, ro, co, blocks)
        if t[0] == "CB":
            nr, nc, nb = int(t[1]), int(t[2]), int(t[3])
            ro, co = ints(nxt()), ints(nxt())
            blocks = []
            for _ in range(nb):
                _, ri, ci, m, n = nxt()
                blocks.append(Block("coo", int(m), int(n), ri=int(ri), ci=int(ci)))
            return Factor("CB", nr, nc, ro, co, blocks)
        if t[0] == "DC":
            return Dense(Block("dense", int(t[1]), int(t[2])))
        raise ValueError("bad plan line %r" % t)

    return rec()


# Kapur-Rokhlin end-correction weights (quadrature.c:12-40; Kapur & Rokhlin,
# SIAM J. Numer. Anal. 34 (1997))
KR_WEIGHTS = {
    2: [1.825748064736159, -1.325748064736159],
    6: [4.967362978287758, -16.20501504859126, 25.85153761832639,
        -22.22599466791883, 9.930104998037539, -1.817995878141594],
    10: [7.832432020568779, -4.565161670374749, 1.452168846354677,
         -2.901348302886379, 3.870862162579900, -3.523821383570681,
         2.172421547519342, -8.707796087382991, 2.053584266072635,
         -2.166984103403823],
}


def kernel_pairs(helm: Helm2, src, src_normals, tgt):
    """bfHelm2GetKernelValue(helm, src_q, tgt_q, n_q, NULL) per pair q."""
    src = np.ascontiguousarray(src, dtype=np.float64)
    tgt = np.ascontiguousarray(tgt, dtype=np.float64)
    nrm = np.ascontiguousarray(src_normals, dtype=np.float64)
    out = np.empty(len(src), dtype=np.complex128)
    cols = [np.ascontiguousarray(a) for a in (src[:, 0], src[:, 1], nrm[:, 0], nrm[:, 1],
                                              tgt[:, 0], tgt[:, 1])]
    rc = lib().oracle_kernel_pairs(
        ctypes.c_int(helm.layer_pot), ctypes.c_double(helm.k),
        ctypes.c_double(helm.alpha.real), ctypes.c_double(helm.alpha.imag),
        ctypes.c_double(helm.beta.real), ctypes.c_double(helm.beta.imag),
        *[_ptr(c) for c in cols], ctypes.c_int64(len(src)), _ptr(out))
    if rc != 0:
        raise NotImplementedError("layer potential %d" % helm.layer_pot)
    return out


def kr_correction(helm: Helm2, X, N, offsets, order: int):
    """(rows, cols, vals) of the block KR correction (quadrature.c:124-164,
    with K_helm2 of multiple_scattering_context.c:27-42: source x_i, normal
    n_i, target x_j)."""
    w = KR_WEIGHTS[order]
    rows, cols, srcs, tgts = [], [], [], []
    for b in range(len(offsets) - 1):
        i0, i1 = offsets[b], offsets[b + 1]
        m = i1 - i0
        for i in range(i0, i1):
            for p in range(order):
                for j in (((i + p + 1 - i0) % m) + i0, (((i + m) - p - 1 - i0) % m) + i0):
                    rows.append(i)
                    cols.append(j)
    rows = np.array(rows)
    cols = np.array(cols)
    vals = kernel_pairs(helm, X[rows], N[rows], X[cols])
    weights = np.tile(np.repeat(np.array(w), 2), len(X))
    return rows, cols, weights * vals


def cfie_system_dense(helm: Helm2, X, N, W, offsets, order: int, shift: float = 0.5):
    """Dense A = shift I + (K + C) diag(W) as assembleDenseK
    (multiple_scattering_context.c:407-437) builds it."""
    K = kernel_matrix(helm, X, X, N, None)
    if order:
        r, c, v = kr_correction(helm, X, N, offsets, order)
        np.add.at(K, (r, c), v)
    K = K * np.asarray(W)[None, :]
    K[np.diag_indices(len(X))] += shift
    return K


def dense_rows(helm: Helm2, src_tree_pts, tgt_tree_pts, rows, X,
               src_normals=None, tgt_normals=None, chunk: int = 4096):
    """Rows ``rows`` (tree order) of K X with the dense FP64 kernel, in
    column chunks so large N never materialises the matrix
    (bf_all_blocks.c:122-149 on sampled rows)."""
    X = np.asarray(X, dtype=np.complex128)
    if X.ndim == 1:
        X = X[:, None]
    rows = np.asarray(rows, dtype=np.int64)
    tp = tgt_tree_pts[rows]
    tn = None if tgt_normals is None else tgt_normals[rows]
    Y = np.zeros((len(rows), X.shape[1]), dtype=np.complex128)
    for j0 in range(0, len(src_tree_pts), chunk):
        j1 = min(j0 + chunk, len(src_tree_pts))
        K = kernel_matrix(helm, src_tree_pts[j0:j1], tp,
                          None if src_normals is None else src_normals[j0:j1], tn)
        Y += K @ X[j0:j1]
    return Y
