"""CPU test of the bench's factorization work counts (kernel evaluations
and the SVD flop model) on a hand-made block table."""
import numpy as np

import bench


def test_factorization_work_counts_and_rates():
    # FIRST 4 x 10, MIDDLE 3 x 8, LAST 5 x 3, DENSE 2 x 2
    table = np.array([[0, 4, 10, 0], [1, 3, 8, 40], [2, 5, 3, 64], [3, 2, 2, 79]], np.int64)
    st = {"fillMs": 2.0, "reexpSmemMs": 1.0, "reexpGlobalMs": 3.0}
    w = bench.factorization_work(table, st)
    assert w["fill_evals"] == 5 * 3 + 2 * 2
    assert w["proxy_evals"] == (16 + 40) + (9 + 24)
    assert w["kernel_evals"] == w["fill_evals"] + w["proxy_evals"]
    assert w["fill_evals_per_s"] == 19 / 2e-3
    svd = 22 * 4 ** 3 + 16 * 16 * 10 + 22 * 3 ** 3 + 16 * 9 * 8
    assert w["svd_flops_model"] == svd
    assert np.isclose(w["reexp_tflops_model"], svd / 4e-3 / 1e12)
    assert np.isclose(w["frac_of_nominal_fp64"], w["reexp_tflops_model"] / 1.25)


def test_factorization_work_without_reexpansions():
    table = np.array([[3, 6, 6, 0]], np.int64)
    w = bench.factorization_work(table, {"fillMs": 1.0, "reexpSmemMs": 0.0, "reexpGlobalMs": 0.0})
    assert w["kernel_evals"] == 36 and w["svd_flops_model"] == 0
    assert w["reexp_tflops_model"] is None and w["frac_of_nominal_fp64"] is None
