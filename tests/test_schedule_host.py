"""CPU tests of the apply's work decomposition (bfgPlanCheckApply): the
staged program the device kernels execute (32-row items, workspace regions,
shared final regions, the final segmented sum) and every tensor-core chunk
schedule the autotuner can pick (128-row items dealt to persistent CTAs)
give, on seeded block values, the product of a direct walk of the plan's
block structure (fac_helm2.c:943-1002, mat_block_dense.c:512-572 and the
factors' Mul) to rounding.  No GPU involved."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

import butterfly_gb300 as B

TOL = 1e-13   # FP64 sums of the same products in another order


def _check(problems, **kw):
    e_prog, e_tc = B.check_apply_schedule(problems, **kw)
    assert e_prog < TOL and e_tc < TOL, (e_prog, e_tc)


@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_reference_plans(name):
    """The reference's own plans (leaf 1, eps-level ranks) of the golden
    workloads."""
    g = load_golden(name)
    _check([(float(g["k"]), g["src"], g["tgt"])], rhs=3)


@pytest.mark.parametrize("ctas", [1, 7, 152, 608])
def test_workload_knobs_and_cta_counts(ctas):
    """Leaf 64 and a 1e-10 rank tolerance, as the benchmark workloads plan;
    one CTA, a few, one per SM and four per SM."""
    src = B.uniform_square_points(6000, 4)
    tgt = B.curve_points("ellipse", 6000, 3, 2)
    _check([(80.0, src, tgt)], leaf_size=64, rank_eps=1e-10, rhs=2, ctas=ctas)


def test_batched_problems_of_uneven_size():
    """Several independent problems in one plan (one HODBF root each, their
    rows and columns back to back), k = N / 30 as the batched workload."""
    rng = np.random.default_rng(7)
    probs = []
    for p, n in enumerate([300, 1100, 2500, 700, 1800]):
        src = B.uniform_square_points(n, 10 + p)
        tgt = B.curve_points("circle", int(rng.integers(n // 2, n)), 3, 3)
        probs.append((n / 30.0, src, tgt))
    _check(probs, leaf_size=64, rank_eps=1e-8, rhs=4)


@pytest.mark.parametrize("ns,nt", [(1, 1), (1, 5), (3, 1), (2, 2), (7, 900), (900, 7)])
def test_tiny_and_lopsided_point_sets(ns, nt):
    src = B.uniform_square_points(ns, 3)
    tgt = B.curve_points("ellipse", nt, 3, 2)
    _check([(20.0, src, tgt)], leaf_size=8 if max(ns, nt) > 100 else 1, rhs=2)


def test_bad_arguments_are_refused():
    src = B.uniform_square_points(50, 1)
    tgt = B.curve_points("circle", 50)
    for kw in ({"rhs": 0}, {"rhs": 65}, {"ctas": 0}):
        with pytest.raises(B.BfgError):
            B.check_apply_schedule([(10.0, src, tgt)], **kw)
    with pytest.raises(B.BfgError):
        B.check_apply_schedule([(-1.0, src, tgt)])
    bad = src.copy()
    bad[3, 0] = np.nan
    with pytest.raises(B.BfgError):
        B.check_apply_schedule([(10.0, bad, tgt)])


def test_benchmark_workload():
    """The headline workload's plan (65,536 points, k = 512, leaf 64, 1e-10)
    with one CTA per SM: the schedules the benchmark times (about 11 s)."""
    import bench
    cfg = bench.CONFIGS["c2"]
    src = B.uniform_square_points(cfg["n"], 0)
    tgt = B.curve_points(cfg["curve"], cfg["n"], cfg["a"], cfg["b"])
    _check([(cfg["k"], src, tgt)], leaf_size=cfg["leaf"], rank_eps=cfg["tol"], rhs=1, ctas=152)


def test_batched_benchmark_workload():
    """The batched workload at 64 problems (N log-uniform in [1,024, 4,096],
    k = N / 30, leaf 64, 1e-8): one plan with a root per problem (16 s)."""
    import bench
    cfg = bench.CONFIGS["c3s"]
    _, probs, ks = bench.batched_problems(B, cfg)
    _check([(k, s, t) for k, (s, t) in zip(ks, probs)], leaf_size=cfg["leaf"],
           rank_eps=cfg["tol"], rhs=2, ctas=152)
