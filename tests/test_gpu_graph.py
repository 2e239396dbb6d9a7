"""An apply captured in a CUDA graph (the library launches on the context's
stream; the workspace exists from an earlier apply, so nothing is allocated
while capturing) replays to the same result as a direct apply, bit for bit,
in every precision and for single and multiple right-hand sides."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import bf_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.fixture(scope="module")
def fac():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.Context(0)
    g = load_golden("star_n2048_k48")
    return B.FacHelm2.make_multilevel(B.Helm2(float(g["k"])), B.Quadtree(g["src"]),
                                      B.Quadtree(g["tgt"]), context=ctx)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x3"])
@pytest.mark.parametrize("R", [1, 16])
def test_captured_apply_replays_the_direct_result(fac, prec, R):
    n = fac.shape[1]
    dt = torch.complex128 if prec == "fp64" else torch.complex64
    X = torch.from_numpy(O.RefRng(21 + R).complex_randn(n * R).reshape(n, R)).cuda().to(dt)
    Yd = torch.empty((fac.shape[0], R), dtype=dt, device="cuda")
    Yg = torch.empty_like(Yd)
    stream = torch.cuda.Stream()
    fac.ctx.set_stream(stream.cuda_stream)
    try:
        with torch.cuda.stream(stream):
            fac.apply_device(X.data_ptr(), R, R, Yd.data_ptr(), R, prec)   # sizes the workspace
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            fac.apply_device(X.data_ptr(), R, R, Yg.data_ptr(), R, prec)
        Yg.zero_()
        with torch.cuda.stream(stream):
            for _ in range(2):
                graph.replay()
        stream.synchronize()
    finally:
        fac.ctx.set_stream(0)
    assert torch.equal(Yg, Yd)
