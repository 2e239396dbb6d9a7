"""CPU tests of the bench's host-side parts: the factorization work counts
(kernel evaluations, the SVD flop model) on a hand-made block table, and the
reference arm's JSON line (the oracle's C port of the reference's apply on
host cores), which needs no GPU."""
import json
import os
import subprocess
import sys

import numpy as np

import bench
from conftest import ROOT


def test_factorization_work_counts_and_rates():
    # FIRST 4 x 10, MIDDLE 3 x 8, LAST 5 x 3, DENSE 2 x 2
    table = np.array([[0, 4, 10, 0], [1, 3, 8, 40], [2, 5, 3, 64], [3, 2, 2, 79]], np.int64)
    st = {"fillMs": 2.0, "reexpSmemMs": 1.0, "reexpGlobalMs": 2.0, "sketchMs": 1.0,
          "reexpSvds": 1, "numSketched": 0}
    w = bench.factorization_work(table, st)
    assert w["fill_evals"] == 5 * 3 + 2 * 2
    assert w["proxy_evals"] == (16 + 40) + (9 + 24)
    assert w["kernel_evals"] == w["fill_evals"] + w["proxy_evals"]
    assert w["fill_evals_per_s"] == 19 / 2e-3
    svd = 22 * 4 ** 3 + 16 * 16 * 10 + 22 * 3 ** 3 + 16 * 9 * 8
    assert w["svd_flops_reference_equivalent"] == svd
    assert w["reexp_s"] == 4e-3 and w["first_middle_blocks"] == 2
    assert w["full_path_svds"] == 1 and w["sketched_blocks"] == 0
    assert np.isclose(w["reference_equivalent_tflops"], svd / 4e-3 / 1e12)


def test_factorization_work_without_reexpansions():
    table = np.array([[3, 6, 6, 0]], np.int64)
    w = bench.factorization_work(table, {"fillMs": 1.0, "reexpSmemMs": 0.0, "reexpGlobalMs": 0.0})
    assert w["kernel_evals"] == 36 and w["svd_flops_reference_equivalent"] == 0
    assert w["reference_equivalent_tflops"] is None


def _bench(args, **env):
    e = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        e.pop(k, None)
    e.update(env)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                          env=e, capture_output=True, text=True, timeout=300)


def test_reference_arm_prints_the_contract_line():
    r = _bench(["--impl", "reference", "--config", "c1", "--steps", "2", "--warmup", "3"])
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["unit"] == "RHS/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert (line["n_gpus"], line["steps"], line["warmup"]) == (1, 2, 3)
    assert line["scaling"] == "weak" and line["vs_baseline"] is None
    assert line["config"]["workload"] == "helmholtz2d_butterfly_apply_c1"
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] == "port" and cpu["cores"] >= 1
    assert cpu["unit"] == "RHS/s" and cpu["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "RHS/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_runs_on_rank_zero_only():
    r = _bench(["--impl", "reference", "--config", "c1", "--steps", "1", "--warmup", "3"],
               RANK="1", WORLD_SIZE="2")
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_batched_reference_arm_is_unavailable():
    r = _bench(["--impl", "reference", "--config", "c3s", "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unavailable"]


def test_cpu_factorization_worker_times_the_oracle_factorization():
    """The CPU factorization leg (child processes on the host cores): the
    oracle's factorization of the 4,096-point workload in full."""
    r = bench.cpu_factorization_worker("c1", 0)
    assert r["full"] is True and r["seconds"] > 0 and r["blocks"] > 100


def test_standin_port_over_a_plan_with_wrapped_values():
    """The reference's apply algorithm over a plan's structure with stand-in
    values in a buffer shorter than the plan: every block reads m n entries
    of it, and the product of constant blocks is the analytic one."""
    from oracle import bf_oracle as O
    src = O.uniform_square_points(2048, 0)
    tgt = O.curve_points("circle", 2048)
    fac = O.Factorization(O.Helm2(40.0), src, tgt, leaf_size=64, eps=1e-8, fill=False)
    text = fac.plan_text()
    entries = O.parse_plan_entries(text)
    assert entries == fac.num_entries()
    big = max(b.m * b.n for b in fac.blocks())
    data = np.full(big + 17, 1e-3 + 0j, dtype=np.complex128)
    port = O.ApplyPort.from_plan(text, data, True, wrap=True)
    full = O.ApplyPort.from_plan(text, np.full(entries, 1e-3 + 0j), True)
    X = O.RefRng(2).complex_randn(2048 * 2).reshape(2048, 2)
    assert np.allclose(port(X, 2), full(X, 2), rtol=1e-13, atol=0)


class _FakeFac:
    """Per-launch times and launch info of a tensor-core apply of several
    RHS tiles: the input's tile-major copy, three stages, the final sum."""
    def __init__(self, ms, info):
        self.ms, self.info = np.asarray(ms, dtype=np.float32), np.asarray(info, dtype=np.int64)

    def apply_timed(self, *args):
        return self.ms

    def launch_info(self, **kw):
        return self.info


class _Ptr:
    def data_ptr(self):
        return 0


def test_launch_roofline_maps_the_dominant_launch_to_its_stage():
    """The roofline's dominant launch is reported with its stage index (the
    input copy before the first stage has no stored entries), which selects
    the ncu DRAM ratio; the algorithmic bytes and rates follow the launch
    info."""
    R = 256
    info = [[0, 1000, 1000], [5000, 1000, 300], [4000, 300, 200], [0, 500, 1000]]
    fac = _FakeFac([0.1, 2.0, 1.5, 0.05], info)
    roof = bench.launch_roofline(fac, _Ptr(), _Ptr(), R, "bf16x3")
    assert roof["kernel"] == "apply launch 1 of 4" and roof["stage"] == 0
    alg = 5000 * 12 + R * 8 * (1000 + 300)
    assert roof["alg_bytes"] == alg
    assert np.isclose(roof["launch_ms"], 2.0)
    assert np.isclose(roof["hbm"]["achieved_gbs"], alg / 2e-3 / 1e9)
    assert np.isclose(roof["tensor"]["achieved_alg_tflops"], 8 * 5000 * R / 2e-3 / 1e12)
    assert np.isclose(sum(roof["launch_share"]), 1.0)
    # no copy launch: the stage index is the launch index; the final sum
    # has no stage
    fac = _FakeFac([2.0, 1.5, 0.05], info[1:])
    assert bench.launch_roofline(fac, _Ptr(), _Ptr(), R, "bf16x3")["stage"] == 0
    fac = _FakeFac([0.1, 0.2, 3.0], info[1:])
    assert bench.launch_roofline(fac, _Ptr(), _Ptr(), R, "fp32")["stage"] is None
