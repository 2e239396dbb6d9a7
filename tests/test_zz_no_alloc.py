"""bfgFacApplyNoAlloc: the apply for callers that cannot allocate GPU memory
(device memory reserved up front by another allocator, or a path where
cudaMalloc's possible synchronisation is not acceptable).  Its workspace is a
static device array inside the library, so this file runs last: it must pass
whether run alone in a fresh process or after every other test.

The check: through the C ABI, two calls in a row (different inputs) give
what the allocating entry point bfgFacApply gives, within the FP64 apply
tolerance of the other GPU tests; too many right-hand sides are refused."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


def _no_alloc(fac, X, Y, R, flags=0):
    lib = B.lib()
    fn = lib.bfgFacApplyNoAlloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                   ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32]
    fn.restype = ctypes.c_int
    with fac.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
        return fn(fac.handle, X.data_ptr(), R, R, Y.data_ptr(), R, flags)


def test_no_alloc_apply_matches_apply_on_consecutive_calls():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.default_context(0)
    g = load_golden("star_n2048_k48")
    fac = B.FacHelm2.make_multilevel(B.Helm2(float(g["k"])), B.Quadtree(g["src"]),
                                     B.Quadtree(g["tgt"]), context=ctx)
    n = fac.shape[1]
    R = 3
    # on a fresh factorization the no-alloc calls (tree and original order)
    # leave the factorization's own workspace and gather buffers unallocated
    X0 = torch.from_numpy(B.Rng(10).complex_randn(n * R).reshape(n, R)).cuda()
    Y0 = torch.empty_like(X0)
    ctx.check(_no_alloc(fac, X0, Y0, R), "first no-alloc call")
    ctx.check(_no_alloc(fac, X0, Y0, R, flags=B.APPLY_ORIGINAL_ORDER), "original order")
    torch.cuda.synchronize()
    assert fac.stats()["applyBufferBytes"] == 0
    Y0_ref = fac.apply(X0, original_order=True)
    assert fac.stats()["applyBufferBytes"] > 0                # the allocating path did allocate
    assert rel_err(Y0.cpu().numpy(), Y0_ref.cpu().numpy()) < 1e-13
    for call, seed in enumerate((11, 12)):
        X = torch.from_numpy(B.Rng(seed).complex_randn(n * R).reshape(n, R)).cuda()
        Y_ref = fac.apply(X)                                  # allocating entry point
        Y = torch.full_like(Y_ref, complex(float("nan"), float("nan")))
        st = _no_alloc(fac, X, Y, R)
        ctx.check(st, "bfgFacApplyNoAlloc call %d" % call)
        torch.cuda.synchronize()
        assert rel_err(Y.cpu().numpy(), Y_ref.cpu().numpy()) < 1e-13
    # the golden reference output too (tree-order rows)
    X = torch.from_numpy(g["x"]).cuda()
    Y = torch.empty_like(X)
    ctx.check(_no_alloc(fac, X, Y, X.shape[1]))
    torch.cuda.synchronize()
    assert rel_err(Y.cpu().numpy(), g["y_bf"]) < 1e-10
    # original point order, as the allocating path does it
    Y_ref = fac.apply(X, original_order=True)
    ctx.check(_no_alloc(fac, X, Y, X.shape[1], flags=B.APPLY_ORIGINAL_ORDER))
    torch.cuda.synchronize()
    assert rel_err(Y.cpu().numpy(), Y_ref.cpu().numpy()) < 1e-13
    # a workspace larger than the static array is refused, not overrun
    Rbig = 4096
    Xb = torch.zeros((n, Rbig), dtype=torch.complex128, device="cuda")
    Yb = torch.zeros_like(Xb)
    st = _no_alloc(fac, Xb, Yb, Rbig)
    assert st == 5                                            # BFG_ERROR_OUT_OF_RANGE
    assert "static limit" in B.lib().bfgGetErrorString(ctx.handle).decode()
    # a right-hand-side count whose workspace size would overflow 64 bits is
    # refused the same way, before any device work (the operands are never read)
    Rhuge = 1 << 62
    fn = B.lib().bfgFacApplyNoAlloc
    for flags in (0, B.APPLY_ORIGINAL_ORDER):
        st = fn(fac.handle, Xb.data_ptr(), Rhuge, Rhuge, Yb.data_ptr(), Rhuge, flags)
        assert st == 5
        assert "static limit" in B.lib().bfgGetErrorString(ctx.handle).decode()
