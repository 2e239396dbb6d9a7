"""The reference-side binding (tests/integration/bfmat_gpu.c): a libbfg
factorization wrapped as the reference's callback operator BfMatFunc
(mat_func.h:5-28), compiled against the reference's own headers and linked
with its library (oracle/_ref, built by oracle/build_ref.sh) and libbfg.
The driver runs the adapter through the reference's bfMatMul (mat.c:183-185)
and bfSolveGMRES (linalg.c:47-317) with the host apply replaced by a CPU
stand-in, so no GPU is needed: products equal the reference's dense product
to 1e-14, GMRES converges through it, and libbfg failures end in the
reference's error handling.  Skipped where the reference build is absent
(the GPU machines: the reference's sources are not there)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_OUT = os.path.join(ROOT, "oracle", "_ref")


def test_bfmat_adapter_through_the_reference(tmp_path):
    root_file = os.path.join(REF_OUT, "reference_root.txt")
    lib = os.path.join(REF_OUT, "libbf_ref.so")
    if not (os.path.exists(root_file) and os.path.exists(lib)):
        pytest.skip("reference build (oracle/build_ref.sh) not present")
    ref = open(root_file).read().strip()
    openblas = open(os.path.join(REF_OUT, "openblas_path.txt")).read().strip()
    if not os.path.isdir(os.path.join(ref, "include", "bf")):
        pytest.skip("reference headers not present")
    from butterfly_gb300 import build
    bfg = build.build()
    exe = str(tmp_path / "bfmat_driver")
    integ = os.path.join(ROOT, "tests", "integration")
    cmd = ["gcc", "-std=gnu11", "-O1", "-Wall", "-Werror", "-Wno-unused-function",
           "-DBF_DOUBLE", "-DBF_LINUX",
           "-I" + os.path.join(ref, "include"), "-I" + os.path.join(ROOT, "oracle", "ref_shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + integ,
           os.path.join(integ, "bfmat_gpu.c"), os.path.join(integ, "bfmat_driver.c"),
           "-o", exe, "-L" + REF_OUT, "-lbf_ref", "-L" + os.path.dirname(bfg), "-lbfg",
           openblas, "-lm", "-Wl,-rpath," + REF_OUT, "-Wl,-rpath," + os.path.dirname(bfg),
           "-Wl,-rpath," + os.path.dirname(openblas)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all ok" in r.stdout
    assert "FAIL" not in r.stdout
