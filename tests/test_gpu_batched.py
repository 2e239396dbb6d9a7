"""Many independent problems of uneven size factorized and applied in one
batch (the batched workload: sources uniform in [-1,1]^2, targets on a circle
of radius 3, k = N/30): every problem's rows of the batched apply equal that
problem factorized alone, and its structure equals the reference planner's."""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


def test_batched_problems_match_single_factorizations():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.default_context(0)
    rng = B.Rng(42)
    sizes = [int(np.exp(np.log(512) + (np.log(4096) - np.log(512)) * u)) for u in rng.uniform(5)]
    problems, ks = [], []
    for p, n in enumerate(sizes):
        problems.append((B.uniform_square_points(n, 100 + p), B.curve_points("circle", n)))
        ks.append(n / 30.0)
    helm = B.Helm2(1.0)
    fac = B.make_batched(helm, problems, ks, context=ctx)
    assert fac.shape == (sum(sizes), sum(sizes))
    R = 3
    X = B.Rng(7).complex_randn(sum(sizes) * R).reshape(-1, R)
    Y = fac.apply(X)
    text = fac.describe()
    for p, ((src, tgt), k) in enumerate(zip(problems, ks)):
        single = B.FacHelm2.make_multilevel(B.Helm2(k), B.Quadtree(src), B.Quadtree(tgt),
                                            context=ctx)
        s0, s1 = fac.src_offsets[p], fac.src_offsets[p + 1]
        t0, t1 = fac.tgt_offsets[p], fac.tgt_offsets[p + 1]
        y1 = single.apply(np.ascontiguousarray(X[s0:s1]))
        assert rel_err(Y[t0:t1], y1) < 1e-13
        sp, tp = single.perms()
        bsp, btp = fac.perms()
        assert np.array_equal(bsp[s0:s1] - s0, sp)
        assert np.array_equal(btp[t0:t1] - t0, tp)
        assert ("PROBLEM %d\n" % p + single.describe()) in text


def test_batched_problems_against_the_oracle():
    """The batched workload's knobs (leaf 64, tolerance 1e-8 for the rank
    estimate and the relative pseudo-inverse cut) on four uneven problems:
    each problem's rows of the one batched apply against the oracle's own
    factorization of that problem (the reference's algorithm with scipy's
    zgesvd, fac_helm2.c:943-1002) and against dense FP64 rows."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import bf_oracle as O
    ctx = B.default_context(0)
    sizes = [1024, 1733, 2980, 4096]
    problems = [(B.uniform_square_points(n, 300 + p), B.curve_points("circle", n))
                for p, n in enumerate(sizes)]
    ks = [n / 30.0 for n in sizes]
    tol = 1e-8
    fac = B.make_batched(B.Helm2(1.0), problems, ks, leaf_size=64, rank_eps=tol, pinv_tol=tol,
                         context=ctx)
    R = 2
    X = B.Rng(9).complex_randn(sum(sizes) * R).reshape(-1, R)
    Y = fac.apply(X)
    bsp, btp = fac.perms()
    for p, ((src, tgt), k) in enumerate(zip(problems, ks)):
        s0, s1 = fac.src_offsets[p], fac.src_offsets[p + 1]
        t0, t1 = fac.tgt_offsets[p], fac.tgt_offsets[p + 1]
        of = O.Factorization(O.Helm2(k), src, tgt, leaf_size=64, eps=tol, rcut="relative")
        assert np.array_equal(bsp[s0:s1] - s0, of.src_perm)
        assert np.array_equal(btp[t0:t1] - t0, of.tgt_perm)
        yo = of.apply(X[s0:s1])
        assert rel_err(Y[t0:t1], yo) < 1e-6
        rows = np.arange(0, t1 - t0, 7)
        yd = O.dense_rows(O.Helm2(k), of.src_tree_pts, of.tgt_tree_pts, rows, X[s0:s1])
        assert rel_err(Y[t0:t1][rows], yd) < 1e-6
        assert rel_err(yo[rows], yd) < 1e-6
