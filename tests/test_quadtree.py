"""Quadtree build (bfQuadtreeInit, quadtree.c:80-98) through the C ABI's
bfgQuadtreeBuild, host path: the reference's own tree orders (golden
fixtures) and the oracle's, plus the node table's invariants."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from oracle import bf_oracle as O

import butterfly_gb300 as B


@pytest.mark.parametrize("name", list(GOLDEN_CASES))
def test_host_tree_order_matches_reference(name):
    g = load_golden(name)
    (sp, _), (tp, _) = B.quadtree_build([g["src"], g["tgt"]], leaf_size=1)
    assert np.array_equal(sp, g["src_perm"].astype(np.int64))
    assert np.array_equal(tp, g["tgt_perm"].astype(np.int64))


@pytest.mark.parametrize("leaf", [1, 16, 64])
def test_host_tree_order_matches_oracle(leaf):
    pts = O.uniform_square_points(3000, 5)
    (perm, _), = B.quadtree_build([pts], leaf_size=leaf)
    assert np.array_equal(perm, np.asarray(O.Quadtree(pts, leaf_size=leaf).perm, dtype=np.int64))


def check_nodes(pts, perm, nodes, leaf):
    """Children partition their parent's range in quadrant order, every point
    lies in its node's box on the side of the split the quadrant says, and
    nodes below the root (which is always split) are split exactly when they
    hold more than `leaf` points."""
    tp = pts[perm]
    assert nodes[0]["parent"] == -1 and nodes[0]["i0"] == 0 and nodes[0]["i1"] == len(pts)
    for i, nd in enumerate(nodes):
        kids = [c for c in nd["child"] if c >= 0]
        if not kids:
            assert nd["i1"] - nd["i0"] <= leaf
            continue
        assert i == 0 or nd["i1"] - nd["i0"] > leaf
        assert kids == sorted(kids)
        assert nodes[kids[0]]["i0"] == nd["i0"] and nodes[kids[-1]]["i1"] == nd["i1"]
        for a, b in zip(kids, kids[1:]):
            assert nodes[a]["i1"] == nodes[b]["i0"]
        for q, c in enumerate(nd["child"]):
            if c < 0:
                continue
            ch = nodes[c]
            assert ch["parent"] == i and ch["depth"] == nd["depth"] + 1
            x, y = tp[ch["i0"]:ch["i1"], 0], tp[ch["i0"]:ch["i1"], 1]
            left, low = q in (0, 1), q in (0, 2)
            assert np.all((x <= nd["splitX"]) == left)
            assert np.all((y <= nd["splitY"]) == low)


@pytest.mark.parametrize("leaf", [1, 8, 64])
def test_host_tree_node_table(leaf):
    pts = np.concatenate([O.uniform_square_points(700, 2), O.curve_points("ellipse", 300)])
    (perm, nodes), = B.quadtree_build([pts], leaf_size=leaf)
    assert sorted(perm.tolist()) == list(range(len(pts)))
    check_nodes(pts, perm, nodes, leaf)


def test_host_tree_bad_arguments():
    with pytest.raises(B.BfgError):
        B.quadtree_build([np.array([[0.0, np.nan]])])
    with pytest.raises(B.BfgError):
        B.quadtree_build([np.zeros((300, 2))], leaf_size=1)   # identical points: no split ends
