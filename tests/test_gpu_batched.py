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
