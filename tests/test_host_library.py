"""CPU tests of the product library's host side: the C ABI loads and exports
every declared symbol, and the host-only planner, generator and Hankel
evaluator agree with the reference fixtures and the oracle."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden

import butterfly_gb300 as B
from oracle import bf_oracle as O


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "bfg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(ln for ln in text.split("\n") if not ln.lstrip().startswith("typedef"))
    names = set(re.findall(r"\b(bfg[A-Z]\w*)\s*\(", text))
    types = set(re.findall(r"\}\s*(bfg\w+)\s*;", open(os.path.join(ROOT, "include", "bfg.h")).read()))
    return sorted(names - types - {"bfgStatus"})


def test_library_exports_every_declared_symbol():
    lib = B.lib()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", B.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (bfg\w+)", out))
    assert set(names) <= exported


@pytest.mark.parametrize("name", list(GOLDEN_CASES))
def test_product_plan_matches_reference(name):
    g = load_golden(name)
    sp, tp, txt = B.plan_helm2(float(g["k"]), g["src"], g["tgt"])
    assert np.array_equal(sp, g["src_perm"].astype(np.int64))
    assert np.array_equal(tp, g["tgt_perm"].astype(np.int64))
    assert txt == g["plan"]


@pytest.mark.parametrize("leaf,eps", [(64, 1e-8), (16, 1e-10), (32, 1e-7)])
def test_product_plan_matches_oracle_with_leaf_and_tolerance(leaf, eps):
    src = O.uniform_square_points(4096, 1)
    tgt = O.curve_points("star", 4096)
    sp, tp, txt = B.plan_helm2(96.0, src, tgt, leaf_size=leaf, rank_eps=eps)
    fac = O.Factorization(O.Helm2(96.0), src, tgt, leaf_size=leaf, eps=eps, fill=False)
    assert np.array_equal(sp, fac.src_perm)
    assert np.array_equal(tp, fac.tgt_perm)
    assert txt == fac.plan_text()


def test_product_generator_matches_reference():
    g = np.load(os.path.join(ROOT, "tests", "golden", "rng_seed3.npz"))
    r = B.Rng(int(g["seed"]))
    assert np.array_equal(r.uniform(int(g["n"])), g["uniform"])
    r.seed(int(g["seed"]))
    assert np.array_equal(r.complex_randn(int(g["n"])), g["complex_randn"])
    for name, (curve, n) in GOLDEN_CASES.items():
        gg = load_golden(name)
        assert np.array_equal(B.uniform_square_points(n, 0), gg["src"])
        assert np.array_equal(B.curve_points(curve, n), gg["tgt"])


def glibc_h01(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    h0 = np.empty(2 * len(x))
    h1 = np.empty(2 * len(x))
    O.lib().oracle_h0(x.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(len(x)),
                      h0.ctypes.data_as(ctypes.c_void_p))
    O.lib().oracle_h1(x.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(len(x)),
                      h1.ctypes.data_as(ctypes.c_void_p))
    return h0[0::2] + 1j * h0[1::2], h1[0::2] + 1j * h1[1::2]


def hankel_samples(n=200000, seed=0):
    rng = np.random.default_rng(seed)
    return np.concatenate([10 ** rng.uniform(-4, 4.3, n), np.linspace(0.01, 40, n // 4),
                           [0.25, 20.0, 19.999999999, 20.000000001]])


def test_hankel_evaluator_source_matches_glibc():
    x = hankel_samples()
    b = B.bessel01_host(x)
    g0, g1 = glibc_h01(x)
    e0 = np.abs(b[:, 0] + 1j * b[:, 1] - g0) / np.abs(g0)
    e1 = np.abs(b[:, 2] + 1j * b[:, 3] - g1) / np.abs(g1)
    # |H_nu(x)| has no real zeros, so the relative error is well defined
    assert e0.max() < 1e-13 and e1.max() < 1e-13


def test_host_entry_points_reject_bad_input():
    with pytest.raises(B.BfgError):
        B.bessel01_host(np.array([1.0, -2.0]))
    with pytest.raises(B.BfgError):
        B.plan_helm2(-1.0, np.zeros((4, 2)), np.ones((4, 2)))
    with pytest.raises(ValueError):
        B.plan_helm2(1.0, np.zeros((4, 3)), np.ones((4, 2)))
    # empty point sets are refused, not planned (the reference's tree build
    # has no empty case)
    pts = B.uniform_square_points(10, 3)
    for src, tgt in ((pts[:0], pts), (pts, pts[:0]), (pts[:0], pts[:0])):
        with pytest.raises(B.BfgError):
            B.plan_helm2(10.0, src, tgt)
        with pytest.raises(B.BfgError):
            B.check_apply_schedule([(10.0, src, tgt)])


# every struct the Python mirror passes across the C ABI, by its C name
ABI_STRUCTS = [("bfgHelm2", "_Helm2C"), ("bfgFacOptions", "_FacOptionsC"),
               ("bfgFacStats", "_FacStatsC"), ("bfgQuadtreeNode", "_QuadtreeNodeC"),
               ("bfgGmresResult", "_GmresResultC"), ("bfgRng", "_RngC")]


def test_ctypes_structs_match_header(tmp_path):
    """The ctypes mirrors have the header's size and every field at the
    header's offset with the header's size (a C program compiled against
    include/bfg.h prints them)."""
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "bfg.h"', 'int main(void) {']
    want = []
    for cname, pyname in ABI_STRUCTS:
        cls = getattr(B, pyname)
        lines.append('  printf("%%s %%zu\\n", "%s", sizeof(%s));' % (cname, cname))
        want.append("%s %d" % (cname, ctypes.sizeof(cls)))
        for fname, _ in cls._fields_:
            lines.append('  printf("%%s.%%s %%zu %%zu\\n", "%s", "%s", offsetof(%s, %s), '
                         'sizeof(((%s *)0)->%s));' % (cname, fname, cname, fname, cname, fname))
            f = getattr(cls, fname)
            want.append("%s.%s %d %d" % (cname, fname, f.offset, f.size))
    lines += ['  return 0;', '}']
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    assert [g for g in got if g] == want


@pytest.mark.parametrize("config", ["c2", "c4"])
def test_product_plan_matches_oracle_at_benchmark_sizes(config):
    """The benchmark workloads' plans (c2: 65,536 points, k = 512; c4, the
    metric's 256-RHS target: 262,144 points on the star, k = 2,048) from the
    library's planner and the oracle's, point for point and block for block."""
    import bench
    cfg = bench.CONFIGS[config]
    src = O.uniform_square_points(cfg["n"], 0)
    tgt = O.curve_points(cfg["curve"], cfg["n"], cfg["a"], cfg["b"])
    sp, tp, txt = B.plan_helm2(cfg["k"], src, tgt, leaf_size=cfg["leaf"], rank_eps=cfg["tol"])
    fac = O.Factorization(O.Helm2(cfg["k"]), src, tgt, leaf_size=cfg["leaf"], eps=cfg["tol"],
                          fill=False)
    assert np.array_equal(sp, fac.src_perm)
    assert np.array_equal(tp, fac.tgt_perm)
    assert txt == fac.plan_text()
