"""The tensor-core apply's bounded waits.  Every mbarrier wait of the
split-BF16 kernel gives up after a limit (1 s by default); the CTA then
drains the copies and tensor-core products it has in flight, frees its
tensor memory and ends, and the apply returns BFG_ERROR_TIMEOUT (33).  The
test hook bfgFacSetTcWaitLimit sets the limit to 0, so every wait that is
not already satisfied gives up at once: the path runs without any fault or
hang being provoked.  Checked: the status (after an asynchronous apply by
bfgFacSynchronize, and by the synchronising timed apply), then that the
factorization is still usable -- at the default limit the next applies
equal the ones before the timeout bit for bit (bf16x3 and bf16x2)."""
import pytest

from conftest import load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.mark.parametrize("R", [16, 32])
def test_zero_wait_limit_times_out_and_the_factorization_recovers(R):
    """R = 16 runs the 16-RHS tile kernel, R = 32 the 32-RHS one (its own
    warp roles: one MMA warp, eight extractor warps)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.default_context(0)
    g = load_golden("ellipse_n16384_k128")
    fac = B.FacHelm2.make_multilevel(B.Helm2(float(g["k"])), B.Quadtree(g["src"]),
                                     B.Quadtree(g["tgt"]), context=ctx)
    n = fac.shape[1]
    X = torch.from_numpy(B.Rng(21).complex_randn(n * R).reshape(n, R)).cuda().to(torch.complex64)
    lib = B.lib()
    Y = torch.empty_like(X)
    for prec in ("bf16x3", "bf16x2"):
        y0 = fac.apply(X, precision=prec)       # on torch's stream
        torch.cuda.synchronize()
        fac.synchronize()
        ctx.check(lib.bfgFacSetTcWaitLimit(fac.handle, 0))
        # the asynchronous apply: reported by the next check of the stream
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
        with pytest.raises(B.BfgError) as e:
            fac.synchronize()
        assert e.value.status == 33                       # BFG_ERROR_TIMEOUT
        # a synchronising call reports it itself
        with pytest.raises(B.BfgError) as e:
            fac.apply_timed(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
        assert e.value.status == 33
        ctx.check(lib.bfgFacSetTcWaitLimit(fac.handle, 1_000_000_000))
        for _ in range(2):
            y1 = fac.apply(X, precision=prec)
            torch.cuda.synchronize()
            fac.synchronize()
            assert torch.equal(y0, y1)
