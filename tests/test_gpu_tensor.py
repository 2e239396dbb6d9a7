"""Split-BF16 tensor-core apply (tcgen05, precisions "bf16x2" and "bf16x3")
against the FP64 apply, which matches the reference's own A_BF X to 1e-10,
and against the reference's golden outputs.

Tolerances (relative Frobenius error):
  * bf16x3 -- 3e-6: three bf16 planes keep ~24 significant bits of every
    factor entry and right-hand side (FP32 storage keeps 24), accumulated in
    FP32 by the tensor cores;
  * bf16x2 -- 2e-3: two planes keep ~16 bits.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import bf_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402

TOL = {"bf16x3": 3e-6, "bf16x2": 2e-3}


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return B.default_context(0)


_facs = {}


def golden_fac(name, ctx):
    if name not in _facs:
        g = load_golden(name)
        fac = B.FacHelm2.make_multilevel(B.Helm2(float(g["k"])), B.Quadtree(g["src"]),
                                         B.Quadtree(g["tgt"]), context=ctx)
        _facs[name] = (g, fac)
    return _facs[name]


@pytest.mark.parametrize("prec", ["bf16x3", "bf16x2"])
@pytest.mark.parametrize("R", [1, 5, 16, 40, 64])
def test_tensor_apply_close_to_fp64(ctx, prec, R):
    g, fac = golden_fac("c1_circle_n4096_k64", ctx)
    X = O.RefRng(11 + R).complex_randn(4096 * R).reshape(4096, R)
    Xd = torch.from_numpy(X).cuda()
    y64 = fac.apply(Xd).cpu().numpy()
    y = fac.apply(Xd.to(torch.complex64), precision=prec).cpu().numpy().astype(np.complex128)
    assert rel_err(y, y64) < TOL[prec]


@pytest.mark.parametrize("name", ["star_n2048_k48", "ellipse_n16384_k128"])
def test_tensor_apply_matches_reference_output(ctx, name):
    """bf16x3 against the reference's own A_BF X (golden fixture)."""
    g, fac = golden_fac(name, ctx)
    y = fac.apply(torch.from_numpy(g["x"]).cuda().to(torch.complex64), precision="bf16x3")
    y = y.cpu().numpy().astype(np.complex128)
    assert rel_err(y, g["y_bf"].reshape(y.shape)) < TOL["bf16x3"]


def test_tensor_apply_is_deterministic(ctx):
    g, fac = golden_fac("star_n2048_k48", ctx)
    X = torch.from_numpy(O.RefRng(3).complex_randn(2048 * 16).reshape(2048, 16)).cuda()
    X = X.to(torch.complex64)
    y1 = fac.apply(X, precision="bf16x3")
    y2 = fac.apply(X, precision="bf16x3")
    assert torch.equal(y1, y2)


@pytest.mark.parametrize("prec", ["bf16x3", "bf16x2"])
def test_tensor_apply_columns_are_independent(ctx, prec):
    """Within one tile width (16 RHS for R <= 16, 32 above) a column's
    result depends on nothing but that column: not on its place in the tile,
    its neighbours or the partial last tile.  The two widths sum the plane
    products in different groupings, so across them the results agree to
    rounding."""
    g, fac = golden_fac("star_n2048_k48", ctx)
    X = O.RefRng(4).complex_randn(2048 * 45).reshape(2048, 45)
    Xd = torch.from_numpy(X).cuda().to(torch.complex64)
    # 16-RHS tiles: R = 13 against single columns
    y13 = fac.apply(Xd[:, :13].contiguous(), precision=prec).cpu().numpy()
    for c in (0, 7, 12):
        yc = fac.apply(Xd[:, c:c + 1].contiguous(), precision=prec).cpu().numpy()
        assert np.array_equal(y13[:, c:c + 1], yc)
    # 32-RHS tiles: R = 45 (a partial second tile) against R = 17 applies
    # holding the column first
    y45 = fac.apply(Xd, precision=prec).cpu().numpy()
    for c in (0, 15, 16, 31, 32, 44):
        Xc = torch.cat([Xd[:, c:c + 1], Xd[:, 20:36]], dim=1).contiguous()
        yc = fac.apply(Xc, precision=prec).cpu().numpy()
        assert np.array_equal(y45[:, c:c + 1], yc[:, :1])
    assert rel_err(y45[:, :13].astype(np.complex128), y13.astype(np.complex128)) < \
        TOL[prec] / 3


def test_tensor_apply_host_operands_and_original_order(ctx):
    g, fac = golden_fac("star_n2048_k48", ctx)
    sp, tp = fac.perms()
    x_tree = g["x"]
    x_orig = np.empty_like(x_tree)
    x_orig[sp] = x_tree
    y_tree = fac.apply(x_tree, precision="bf16x3")              # host complex128 path
    y_orig = fac.apply(x_orig, precision="bf16x3", original_order=True)
    assert rel_err(y_orig[tp], y_tree) < 1e-12
    assert rel_err(y_tree, g["y_bf"].reshape(y_tree.shape)) < TOL["bf16x3"]


@pytest.mark.parametrize("R", [45, 64])
def test_tensor_apply_host_operands_with_several_tiles(ctx, R):
    """With more than one RHS tile the host-operand applies convert their
    input straight into the tile-major layout (the device apply and the
    original-order gather take it row-major): the same arithmetic, so the
    same bits, for a partial last tile (45) and full tiles (64), through
    the synchronous and the pipelined host calls."""
    g, fac = golden_fac("star_n2048_k48", ctx)
    sp, tp = fac.perms()
    x = np.ascontiguousarray(O.RefRng(60 + R).complex_randn(2048 * R).reshape(2048, R))
    y_dev = fac.apply(torch.from_numpy(x).cuda().to(torch.complex64),
                      precision="bf16x3").cpu().numpy().astype(np.complex128)
    y_host = fac.apply(x, precision="bf16x3")
    assert np.array_equal(y_host, y_dev)
    x_orig = np.empty_like(x)
    x_orig[sp] = x
    y_orig = fac.apply(x_orig, precision="bf16x3", original_order=True)
    assert np.array_equal(y_orig[tp], y_host)
    lib = B.lib()
    xp = torch.from_numpy(x).pin_memory()
    yp = torch.zeros((2048, R), dtype=torch.complex128).pin_memory()
    ctx.check(lib.bfgFacApplyHostAsync(fac.handle, B.PRECISIONS["bf16x3"], B._VP(xp.data_ptr()),
                                       R, R, B._VP(yp.data_ptr()), R, 0))
    ctx.check(lib.bfgFacApplyHostWait(fac.handle))
    assert np.array_equal(yp.numpy(), y_host)


@pytest.mark.parametrize("R", [16, 64])
def test_tensor_apply_timed_launch_count(ctx, R):
    """One tile: the stages and the final sum; more tiles: the input's
    tile-major copy first (no stored entries, every input row)."""
    g, fac = golden_fac("star_n2048_k48", ctx)
    X = torch.zeros((2048, R), dtype=torch.complex64, device="cuda")
    Y = torch.empty_like(X)
    torch.cuda.synchronize()
    ms = fac.apply_timed(X.data_ptr(), R, R, Y.data_ptr(), R, "bf16x3")
    info = fac.launch_info(precision="bf16x3", rhs=R)
    assert len(ms) == len(info)
    stages = len(fac.launch_info()) - 1
    if R <= 32:
        assert len(info) == stages + 1
        assert np.array_equal(info, fac.launch_info())
    else:
        assert len(info) == stages + 2
        assert info[0, 0] == 0 and info[0, 1] == info[0, 2] == 2048
        assert np.array_equal(info[1:], fac.launch_info())
    assert torch.count_nonzero(Y).item() == 0


# ---- double-float (df64): FP64 accuracy from FP32 arithmetic ----
@pytest.mark.parametrize("R", [1, 3, 16])
def test_df64_apply_matches_fp64(ctx, R):
    g, fac = golden_fac("ellipse_n16384_k128", ctx)
    n = fac.shape[1]
    X = torch.from_numpy(O.RefRng(31 + R).complex_randn(n * R).reshape(n, R)).cuda()
    y64 = fac.apply(X)
    ydf = fac.apply(X, precision="df64")
    assert ydf.dtype == torch.complex128
    # double-float keeps ~48 significant bits: agreement far below FP32's
    assert rel_err(ydf.cpu().numpy(), y64.cpu().numpy()) < 1e-12


def test_df64_apply_reference_output_and_original_order(ctx):
    g, fac = golden_fac("star_n2048_k48", ctx)
    y = fac.apply(g["x"], precision="df64")                # host complex128 path
    assert rel_err(y, g["y_bf"].reshape(y.shape)) < 1e-12
    sp, tp = fac.perms()
    x_orig = np.empty_like(g["x"])
    x_orig[sp] = g["x"]
    y_orig = fac.apply(x_orig, precision="df64", original_order=True)
    assert np.array_equal(y_orig[tp], y)


def test_df64_apply_is_deterministic_and_timed(ctx):
    g, fac = golden_fac("star_n2048_k48", ctx)
    X = torch.from_numpy(O.RefRng(8).complex_randn(2048 * 2).reshape(2048, 2)).cuda()
    assert torch.equal(fac.apply(X, precision="df64"), fac.apply(X, precision="df64"))
    Y = torch.empty_like(X)
    ms = fac.apply_timed(X.data_ptr(), 2, 2, Y.data_ptr(), 2, "df64")
    assert len(ms) == len(fac.launch_info())


@pytest.mark.parametrize("prec", ["fp64", "df64", "bf16x3"])
def test_pipelined_host_apply_matches_synchronous(ctx, prec):
    """bfgFacApplyHostAsync: several calls in flight (two staging slots, a
    third call waits on the device), the same results as bfgFacApplyHost."""
    g, fac = golden_fac("star_n2048_k48", ctx)
    lib = B.lib()
    P = B.PRECISIONS[prec]
    R = 4
    Xs = [np.ascontiguousarray(O.RefRng(40 + i).complex_randn(2048 * R).reshape(2048, R))
          for i in range(5)]
    Xp = [torch.from_numpy(x).pin_memory() for x in Xs]
    Yp = [torch.zeros((2048, R), dtype=torch.complex128).pin_memory() for _ in Xs]
    for x, y in zip(Xp, Yp):
        ctx.check(lib.bfgFacApplyHostAsync(fac.handle, P, B._VP(x.data_ptr()), R, R,
                                           B._VP(y.data_ptr()), R, 0))
    ctx.check(lib.bfgFacApplyHostWait(fac.handle))
    for x, y in zip(Xs, Yp):
        assert np.array_equal(y.numpy(), fac.apply(x, precision=prec))


@pytest.mark.parametrize("R", [16, 24, 64])
def test_autotune_keeps_results_and_never_slows_the_apply(ctx, R):
    """bfgFacAutotune picks the RHS tile width and re-deals chunks to CTAs.
    An item stays on one CTA with its chunks in order, so within a width the
    results are bit-identical; a change of width regroups the plane
    products' sums, within rounding.  The default is a candidate, so the
    tuned stages sum to no more than the default ones."""
    g, fac = golden_fac("ellipse_n16384_k128", ctx)
    X = torch.from_numpy(O.RefRng(50).complex_randn(16384 * R).reshape(16384, R)).cuda()
    X = X.to(torch.complex64)
    assert fac.rhs_tile("bf16x3", R) == (16 if R <= 16 else 32)
    y0 = fac.apply(X, precision="bf16x3")
    times = fac.autotune("bf16x3", R)
    assert times.shape[0] == len(fac.launch_info()) - 1          # stages, not the final sum
    assert times[:, 1].sum() <= times[:, 0].sum()
    rt = fac.rhs_tile("bf16x3", R)
    assert rt in (16, 32)
    y1 = fac.apply(X, precision="bf16x3")
    if rt == (16 if R <= 16 else 32):
        assert torch.equal(y1, y0)
    else:
        assert rel_err(y1.cpu().numpy().astype(np.complex128),
                       y0.cpu().numpy().astype(np.complex128)) < TOL["bf16x3"] / 3
    # the choice holds for this R only
    assert fac.rhs_tile("bf16x3", R + 1) == (16 if R + 1 <= 16 else 32)
    with pytest.raises(B.BfgError):
        fac.autotune("fp32", 16)
    with pytest.raises(B.BfgError):
        fac.rhs_tile("fp32", 16)


def test_double_float_jacobi_factorization(ctx):
    """The re-expansion SVDs' Jacobi sweeps in double-float: the same
    operator as with FP64 sweeps (relative cut 1e-10), checked against dense
    FP64 kernel rows; every block converges; cuts below 1e-10 are refused."""
    src = O.uniform_square_points(6000, 4)
    tgt = O.curve_points("ellipse", 6000)
    X = torch.from_numpy(O.RefRng(60).complex_randn(6000 * 4).reshape(6000, 4)).cuda()
    facs = {a: B.FacHelm2.make_multilevel(B.Helm2(80.0), B.Quadtree(src, leaf_size=32),
                                          B.Quadtree(tgt, leaf_size=32), rank_eps=1e-10,
                                          pinv_tol=1e-10, jacobi=a, context=ctx)
            for a in ("fp64", "df64")}
    # every block converges within the sweep cap in both arithmetics (this
    # problem has blocks in every re-expansion mode, ranks up to 361)
    assert facs["fp64"].stats()["jacobiNotConverged"] == 0
    assert facs["df64"].stats()["jacobiNotConverged"] == 0
    y64 = facs["fp64"].apply(X).cpu().numpy()
    ydf = facs["df64"].apply(X).cpu().numpy()
    assert rel_err(ydf, y64) < 1e-9
    rows = np.arange(0, 6000, 97)
    yd = facs["df64"].dense_rows(rows, X, 4).cpu().numpy()
    assert rel_err(ydf[rows], yd) < 1e-8
    for tol in (None, 1e-11):   # the eps-level default cut, and one below 1e-10
        kw = {} if tol is None else {"pinv_tol": tol}
        with pytest.raises(B.BfgError):
            B.FacHelm2.make_multilevel(B.Helm2(80.0), B.Quadtree(src, leaf_size=32),
                                       B.Quadtree(tgt, leaf_size=32), jacobi="df64",
                                       context=ctx, **kw)
