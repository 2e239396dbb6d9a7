"""Edge cases of the factorization and apply through the C ABI: tiny and
lopsided point sets (compared with the dense kernel), a single right-hand
side in every precision, strided operands, and inputs the reference cannot
factor (duplicate points) or calls with bad shapes, which must return status
codes and leave the context usable."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import bf_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return B.default_context(0)


def _dense_check(ctx, src, tgt, k, tol, **kw):
    fac = B.FacHelm2.make_multilevel(B.Helm2(k), B.Quadtree(src, leaf_size=kw.get("leaf", 1)),
                                     B.Quadtree(tgt, leaf_size=kw.get("leaf", 1)), context=ctx)
    X = O.RefRng(5).complex_randn(len(src) * 3).reshape(len(src), 3)
    y = fac.apply(X, original_order=True)
    yd = B.kernel_matrix(B.Helm2(k), src, tgt, context=ctx) @ X
    assert rel_err(y, yd) < tol
    return fac


@pytest.mark.parametrize("ns,nt", [(1, 1), (1, 5), (3, 1), (2, 2)])
def test_tiny_point_sets(ctx, ns, nt):
    src = B.uniform_square_points(ns, 3)
    tgt = B.curve_points("circle", nt)
    _dense_check(ctx, src, tgt, 10.0, 1e-13)


def test_lopsided_point_sets(ctx):
    # few sources, many targets and the reverse (leaf size 8 splits deeply)
    _dense_check(ctx, B.uniform_square_points(7, 4), B.curve_points("ellipse", 900, 3, 2), 20.0,
                 1e-10, leaf=8)
    _dense_check(ctx, B.uniform_square_points(900, 4), B.curve_points("ellipse", 7, 3, 2), 20.0,
                 1e-10, leaf=8)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x3", "bf16x2"])
def test_single_rhs_and_strided_operands_every_precision(ctx, prec):
    n = 1500
    src = B.uniform_square_points(n, 6)
    tgt = B.curve_points("circle", n)
    fac = B.FacHelm2.make_multilevel(B.Helm2(30.0), B.Quadtree(src, leaf_size=16),
                                     B.Quadtree(tgt, leaf_size=16), context=ctx)
    dt = torch.complex128 if prec == "fp64" else torch.complex64
    tol = {"fp64": 1e-14, "fp32": 1e-5, "bf16x3": 3e-6, "bf16x2": 2e-3}[prec]
    X = torch.from_numpy(O.RefRng(9).complex_randn(n * 4).reshape(n, 4)).cuda()
    y64 = fac.apply(X)
    # one column, taken from a 4-column matrix (leading dimension 4)
    Xs = X.to(dt)
    Y = torch.zeros((n, 3), dtype=dt, device="cuda")      # leading dimension 3
    # the raw-pointer call runs on the context's stream: put it on torch's,
    # behind the fill of Y and the applies above (they share the workspace)
    with fac.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
        fac.apply_device(Xs[:, 1:].data_ptr(), 4, 1, Y.data_ptr(), 3, prec)
    torch.cuda.synchronize()
    y = Y[:, 0].cpu().numpy().astype(np.complex128)
    assert rel_err(y, y64[:, 1].cpu().numpy()) < tol
    assert torch.count_nonzero(Y[:, 1:]).item() == 0      # untouched columns


def test_duplicate_points_and_bad_shapes_return_errors(ctx):
    src = np.zeros((100, 2))                                # every point the same
    with pytest.raises(B.BfgError) as e:
        B.FacHelm2.make_multilevel(B.Helm2(5.0), B.Quadtree(src), B.Quadtree(src + 1.0),
                                   context=ctx)
    assert e.value.status == 2
    src = B.uniform_square_points(300, 1)
    tgt = B.curve_points("circle", 300)
    fac = B.FacHelm2.make_multilevel(B.Helm2(5.0), B.Quadtree(src), B.Quadtree(tgt), context=ctx)
    X = torch.zeros((300, 2), dtype=torch.complex128, device="cuda")
    Y = torch.zeros_like(X)
    lib = B.lib()
    assert lib.bfgFacApply(fac.handle, 0, B._VP(X.data_ptr()), 1, 2, B._VP(Y.data_ptr()), 2, 0) == 1
    assert lib.bfgFacApply(fac.handle, 0, B._VP(X.data_ptr()), 2, 0, B._VP(Y.data_ptr()), 2, 0) == 1
    assert lib.bfgFacApply(fac.handle, 7, B._VP(X.data_ptr()), 2, 2, B._VP(Y.data_ptr()), 2, 0) == 3
    # the context still works
    y = fac.apply(O.RefRng(2).complex_randn(300))
    assert np.all(np.isfinite(y))
