"""GPU quadtree build (bfg_tree.cu) against the host build: the same tree
order and node table, field for field, on point sets with ties on the split
lines, clusters, curves, tiny sets and forests of uneven sets; and
factorizations built on either tree give bit-identical applies."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from oracle import bf_oracle as O
from test_quadtree import check_nodes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return B.default_context(0)


def same_trees(sets, leaf, ctx):
    host = B.quadtree_build(sets, leaf_size=leaf, on_gpu=False)
    gpu = B.quadtree_build(sets, leaf_size=leaf, on_gpu=True, context=ctx)
    for (hp, hn), (gp, gn), pts in zip(host, gpu, sets):
        assert np.array_equal(hp, gp)
        assert hn.tobytes() == gn.tobytes()
        if len(pts) > 1:
            check_nodes(pts, gp, gn, leaf)


def grid_points(n):
    # many points exactly on the split lines of every level
    k = int(np.ceil(np.sqrt(n)))
    g = np.stack(np.meshgrid(np.arange(k), np.arange(k)), -1).reshape(-1, 2)[:n]
    return (g / (k - 1) * 2.0 - 1.0).astype(np.float64)


def blobs(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, size=(8, 2))
    return (c[rng.integers(0, 8, n)] + 0.01 * rng.standard_normal((n, 2))).astype(np.float64)


@pytest.mark.parametrize("name", list(GOLDEN_CASES))
def test_gpu_tree_matches_host_on_golden_points(ctx, name):
    g = load_golden(name)
    same_trees([g["src"], g["tgt"]], 1, ctx)
    (sp, _), = B.quadtree_build([g["src"]], leaf_size=1, on_gpu=True, context=ctx)
    assert np.array_equal(sp, g["src_perm"].astype(np.int64))     # the reference's order


@pytest.mark.parametrize("leaf", [1, 64])
@pytest.mark.parametrize("kind", ["uniform", "ellipse", "grid", "blobs"])
def test_gpu_tree_matches_host(ctx, kind, leaf):
    n = 20000
    pts = {"uniform": lambda: O.uniform_square_points(n, 7),
           "ellipse": lambda: O.curve_points("ellipse", n),
           "grid": lambda: grid_points(n),
           "blobs": lambda: blobs(n, 3)}[kind]()
    same_trees([pts], leaf, ctx)


def test_gpu_tree_tiny_and_degenerate_sets(ctx):
    sets = [np.array([[0.3, 0.4]]), np.array([[0.0, 0.0], [1.0, 1.0]]),
            np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]]),          # collinear
            O.uniform_square_points(5, 1)]
    same_trees(sets, 1, ctx)
    same_trees(sets, 2, ctx)
    # each point twice: separable down to leaves of 2
    dup = np.repeat(O.uniform_square_points(50, 2), 2, axis=0)
    same_trees([dup], 2, ctx)


def test_gpu_forest_of_uneven_sets(ctx):
    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(200), np.log(8000), 40)).astype(int)
    sets = [O.uniform_square_points(int(s), int(i)) if i % 2 else O.curve_points("circle", int(s))
            for i, s in enumerate(sizes)]
    same_trees(sets, 64, ctx)


def test_gpu_tree_identical_points_fail_like_host(ctx):
    with pytest.raises(B.BfgError):
        B.quadtree_build([np.zeros((300, 2))], leaf_size=1, on_gpu=True, context=ctx)


def test_factorization_on_gpu_trees_is_identical(ctx):
    src = O.uniform_square_points(6000, 4)
    tgt = O.curve_points("star", 6000)
    X = torch.from_numpy(O.RefRng(5).complex_randn(6000 * 4).reshape(6000, 4)).cuda()
    ys = []
    for on_gpu in (False, True):
        fac = B.FacHelm2.make_multilevel(B.Helm2(60.0), B.Quadtree(src, leaf_size=32),
                                         B.Quadtree(tgt, leaf_size=32), rank_eps=1e-10,
                                         pinv_tol=1e-10, tree_on_gpu=on_gpu, context=ctx)
        ys.append((fac.perms(), fac.apply(X), fac.apply(X.to(torch.complex64), precision="bf16x3")))
    (p0, y0, z0), (p1, y1, z1) = ys
    assert all(np.array_equal(a, b) for a, b in zip(p0, p1))
    assert torch.equal(y0, y1) and torch.equal(z0, z1)


def test_batched_factorization_on_gpu_trees_is_identical(ctx):
    probs, ks = [], []
    for i, n in enumerate([900, 2500, 1600]):
        probs.append((O.uniform_square_points(n, 20 + i), O.curve_points("circle", n)))
        ks.append(n / 30.0)
    X = None
    ys = []
    for on_gpu in (False, True):
        fac = B.make_batched(B.Helm2(1.0), probs, ks, leaf_size=64, rank_eps=1e-8,
                             pinv_tol=1e-8, tree_on_gpu=on_gpu, context=ctx)
        if X is None:
            X = torch.from_numpy(O.RefRng(6).complex_randn(fac.shape[1] * 2)
                                 .reshape(fac.shape[1], 2)).cuda()
        ys.append((fac.perms(), fac.apply(X)))
    assert all(np.array_equal(a, b) for a, b in zip(ys[0][0], ys[1][0]))
    assert torch.equal(ys[0][1], ys[1][1])
