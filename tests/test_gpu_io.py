"""Saved factorizations (bfgFacSave / bfgFacLoad): a reloaded factorization
has the same plan, permutations and factors, so its applies equal the
original's bit for bit; batched factorizations round-trip too; files of
another format, truncated files and missing files are refused with status
codes."""
import os

import numpy as np
import pytest

from conftest import load_golden
from oracle import bf_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return B.default_context(0)


def _same_operator(a, b, n_cols, precs=("fp64", "bf16x3")):
    assert a.describe() == b.describe()
    for pa, pb in zip(a.perms(), b.perms()):
        assert np.array_equal(pa, pb)
    X = torch.from_numpy(O.RefRng(31).complex_randn(n_cols * 5).reshape(n_cols, 5)).cuda()
    for p in precs:
        Xp = X if p == "fp64" else X.to(torch.complex64)
        assert torch.equal(a.apply(Xp, precision=p), b.apply(Xp, precision=p))


def test_save_load_round_trip(ctx, tmp_path):
    g = load_golden("star_n2048_k48")
    fac = B.FacHelm2.make_multilevel(B.Helm2(float(g["k"])), B.Quadtree(g["src"], leaf_size=8),
                                     B.Quadtree(g["tgt"], leaf_size=8), rank_eps=1e-10,
                                     pinv_tol=1e-10, context=ctx)
    path = str(tmp_path / "star.bfgfac")
    fac.save(path)
    assert os.path.getsize(path) > fac.stats()["arenaEntries"] * 16
    back = B.load_fac(path, context=ctx)
    assert back.shape == fac.shape
    assert back.stats()["arenaEntries"] == fac.stats()["arenaEntries"]
    assert back.stats()["maxRank"] == fac.stats()["maxRank"]
    _same_operator(fac, back, fac.shape[1])


def test_save_load_combined_field_with_normals(ctx, tmp_path):
    pts, nrm, w, off, _ = B.scattering_geometry(num=6, k=30.0, ppw=12, rmin=0.2, rmax=0.4,
                                                box=2.0, gap=0.1, seed=5)
    helm = B.Helm2(30.0, B.LayerPot.CombinedField, alpha=-30j, beta=1.0)
    fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm), B.Quadtree(pts), context=ctx)
    path = str(tmp_path / "cfie.bfgfac")
    fac.save(path)
    _same_operator(fac, B.load_fac(path, context=ctx), fac.shape[1], precs=("fp64",))


def test_save_load_batched(ctx, tmp_path):
    rng = B.Rng(8)
    sizes = [int(v) for v in 600 + 900 * rng.uniform(4)]
    problems = [(B.uniform_square_points(n, 50 + j), B.curve_points("circle", n)) for j, n in
                enumerate(sizes)]
    fac = B.make_batched(B.Helm2(1.0), problems, [n / 30.0 for n in sizes], leaf_size=16,
                         rank_eps=1e-10, pinv_tol=1e-10, context=ctx)
    path = str(tmp_path / "batch.bfgfac")
    fac.save(path)
    _same_operator(fac, B.load_fac(path, context=ctx), fac.shape[1])


def test_load_refuses_bad_files(ctx, tmp_path):
    g = load_golden("star_n2048_k48")
    fac = B.FacHelm2.make_multilevel(B.Helm2(float(g["k"])), B.Quadtree(g["src"]),
                                     B.Quadtree(g["tgt"]), context=ctx)
    path = tmp_path / "ok.bfgfac"
    fac.save(str(path))
    data = path.read_bytes()
    bad = tmp_path / "bad.bfgfac"
    bad.write_bytes(b"NOTAFAC!" + data[8:])
    with pytest.raises(B.BfgError) as e:
        B.load_fac(str(bad), context=ctx)
    assert e.value.status == 1
    bad.write_bytes(data[: len(data) // 2])
    with pytest.raises(B.BfgError) as e:
        B.load_fac(str(bad), context=ctx)
    assert e.value.status == 2
    with pytest.raises(B.BfgError):
        B.load_fac(str(tmp_path / "missing.bfgfac"), context=ctx)
