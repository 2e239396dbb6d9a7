import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["plan"] = out["plan"].tobytes().decode()
    out["stats"] = out["stats"].tobytes().decode() if "stats" in out else ""
    return out


GOLDEN_CASES = {
    "c1_circle_n4096_k64": ("circle", 4096),
    "ellipse_n16384_k128": ("ellipse", 16384),
    "star_n2048_k48": ("star", 2048),
}


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
