"""The GPU's relative pseudo-inverse cut (bfgFacOptions pinvCut = 1: keep
sigma_i >= tol sigma_0, the rule of bfTruncSpecGetNumTerms, linalg.c:26-36)
against the oracle's scipy-zgesvd pseudo-inverse with the same rule, block
by block on MIDDLE blocks where the cut is active (8,192 sources in
[-1,1]^2, 8,192 targets on the star curve, k = 256, leaf 64, tol 1e-8; the
full Jacobi path, FP64 and double-float sweeps).

Bar: Z_shift within 1e-4 of the oracle's.  Keeping one term more or less at
the cut moves Z_shift by more than 1e-3 on these blocks
(tests/test_oracle_cut.py), so the bar pins the kept count."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import bf_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.mark.parametrize("jacobi", ["fp64", "df64"])
def test_relative_cut_blocks_match_the_oracle(jacobi):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.default_context(0)
    k, tol = 256.0, 1e-8
    src = O.uniform_square_points(8192, 0)
    tgt = O.curve_points("star", 8192)
    fac = B.FacHelm2.make_multilevel(B.Helm2(k), B.Quadtree(src, leaf_size=64),
                                     B.Quadtree(tgt, leaf_size=64), rank_eps=tol,
                                     pinv_tol=tol, sketch=False, jacobi=jacobi, context=ctx)
    st = fac.stats()
    assert st["jacobiNotConverged"] == 0
    # blocks with the same Z_equiv share one SVD; the checks below cover
    # members of shared groups as well as their leaders
    assert 0 < st["reexpSvds"] < st["numFirst"] + st["numMiddle"]
    of = O.Factorization(O.Helm2(k), src, tgt, leaf_size=64, eps=tol, rcut="relative",
                         fill=False)
    tab, ent = fac.blocks()
    mids = [(row, ob) for row, ob in zip(tab, of.blocks()) if ob.kind == "middle"]
    h = O.Helm2(k)
    for (kind, m, n, off), ob in mids[::97][:12]:
        assert kind == 1 and (m, n) == (ob.m, ob.n)
        Z = ent[off:off + m * n].reshape(n, m).T
        eq, _ = O.circle_points(ob.ceq, m)
        chk, _ = O.circle_points(ob.cchk, m)
        orig, _ = O.circle_points(ob.corig, n)
        Ze = O.kernel_matrix(h, eq, chk)
        Zo = O.kernel_matrix(h, orig, chk)
        Xo, terms, _ = O.lstsq_pinv(Ze, Zo, "relative", tol, return_terms=True)
        assert 0 < terms < m
        assert rel_err(Z, Xo) < 1e-4
