"""Generates the golden fixtures in this directory by running the reference
library's own code (built from its sources by oracle/build_ref.sh) through the
driver oracle/_ref/ref_dump.

Run from the repository root, where the reference sources are present:
    oracle/build_ref.sh && python tests/golden/make_golden.py

Each case stores, in one compressed .npz:
  src, tgt            input points (float64, N x 2, original order)
  src_perm, tgt_perm  quadtree permutations (tree position -> original index)
  plan                the factorization's block structure (plan.txt grammar of
                      oracle/ref_dump.c), utf-8 bytes
  x, y_bf             X (tree order, n_src x R) and the reference's A_BF X
  dense_rows, y_dense sampled tree-order rows of the dense FP64 product K X
  k, R, xseed         parameters; stats (factorization/apply seconds, bytes)
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import bf_oracle as O  # noqa: E402

REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
OUT = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # config-1 geometry: uniform sources, circle r=3 targets, k=64
    "c1_circle_n4096_k64": dict(n=4096, k=64.0, curve="circle", R=2, xseed=7, ndense=64),
    # ellipse (3,2) targets, k=128 (the intermediate size of the survey)
    "ellipse_n16384_k128": dict(n=16384, k=128.0, curve="ellipse", R=1, xseed=11, ndense=64),
    # star targets r = 3 + 0.5 cos(5 theta), small
    "star_n2048_k48": dict(n=2048, k=48.0, curve="star", R=3, xseed=5, ndense=48),
}


def run_case(name, n, k, curve, R, xseed, ndense):
    src = O.uniform_square_points(n, 0)
    tgt = O.curve_points(curve, n)
    with tempfile.TemporaryDirectory() as d:
        src.tofile(os.path.join(d, "src.f64"))
        tgt.tofile(os.path.join(d, "tgt.f64"))
        subprocess.check_call([REF_DUMP, "fac", d, repr(k), os.path.join(d, "src.f64"),
                               os.path.join(d, "tgt.f64"), str(R), str(xseed),
                               str(ndense), "0"])
        rd = lambda f, dt: np.fromfile(os.path.join(d, f), dtype=dt)
        plan = open(os.path.join(d, "plan.txt"), "rb").read()
        stats = open(os.path.join(d, "stats.txt")).read()
        np.savez_compressed(
            os.path.join(OUT, name + ".npz"),
            src=src, tgt=tgt,
            src_perm=rd("src_perm.u64", np.uint64).astype(np.uint32),
            tgt_perm=rd("tgt_perm.u64", np.uint64).astype(np.uint32),
            plan=np.frombuffer(plan, dtype=np.uint8),
            x=rd("x.c128", np.complex128).reshape(n, R),
            y_bf=rd("y_bf.c128", np.complex128).reshape(n, R),
            dense_rows=rd("dense_rows.u64", np.uint64).astype(np.int64),
            y_dense=rd("y_dense.c128", np.complex128).reshape(-1, R),
            k=k, R=R, xseed=xseed, stats=np.frombuffer(stats.encode(), dtype=np.uint8))
    print(name, stats.replace("\n", " "))


def run_rng():
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "rng.f64")
        subprocess.check_call([REF_DUMP, "rng", "3", "2001", f])
        v = np.fromfile(f, dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, "rng_seed3.npz"), seed=3, n=2001,
                        uniform=v[:2001], complex_randn=v[2001:].view(np.complex128))
    print("rng_seed3 done")


if __name__ == "__main__":
    if not os.path.exists(REF_DUMP):
        sys.exit("run oracle/build_ref.sh first")
    run_rng()
    for name, kw in CASES.items():
        if len(sys.argv) > 1 and name not in sys.argv[1:]:
            continue
        run_case(name, **kw)
