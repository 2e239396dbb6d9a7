"""Builds libbfg.so in-tree with nvcc for sm_103a (GB300).

    python -m butterfly_gb300.build          # or __graft_entry__.build()

Translation units compile in parallel into butterfly_gb300/_build/ and link
into butterfly_gb300/libbfg.so (CUDA runtime linked shared).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbfg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-I" + os.path.join(ROOT, "include")]
SOURCES = ["bfg_kernels.cu", "bfg_plan.cpp", "bfg_api.cpp", "bfg_noalloc.cu", "bfg_solver.cu",
           "bfg_tc.cu", "bfg_tree.cu", "bfg_df64.cu", "bfg_mlp.cu", "bfg_mlp_api.cpp",
           "bfg_check.cpp", "bfg_sketch.cu", "bfg_coarse.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *COMMON, *ARCH, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-v"] if os.environ.get("BFG_PTXAS_VERBOSE") else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if r.stderr.strip() and os.environ.get("BFG_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "bfg.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    # the CUDA runtime is linked shared so that a process that also loads
    # torch's runtime ends up with a single runtime instance
    cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")
    cmd = [nvcc(), "-shared", *ARCH, "-cudart", "shared", "-Xlinker", "-rpath," + cudalib,
           "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
