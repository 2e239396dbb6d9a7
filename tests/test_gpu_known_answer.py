"""The GPU multiple-scattering solve against the point-source known answer
(examples/simple/helm2_bie.c:60-210): the butterfly-factorized
combined-field operator with the Kapur-Rokhlin correction, block-Jacobi
flexible GMRES on the GPU, and the exterior field of its density (evaluated
by the oracle) converging to the exact field of the interior sources at the
KR rule's order -- the same errors as the oracle's dense solve."""
import numpy as np
import pytest

import known_answer as KA

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return B.default_context(0)


def _gpu_error(ctx, ppw):
    pts, nrm, w, off, srcs, tgt = KA.geometry(ppw)
    helm = B.Helm2(KA.K, B.LayerPot.CombinedField, alpha=-1j * KA.K, beta=1.0)
    fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm), B.Quadtree(pts), context=ctx)
    sys_ = B.System(fac, pts, nrm, w, off, kr_order=6, diag_shift=0.5)
    sys_.build_block_jacobi()
    b = torch.from_numpy(KA.exact_field(srcs, pts)).cuda()
    x, info = B.solve_gmres(sys_, b, tol=1e-10, max_num_iter=400, precond="block_jacobi")
    assert info["converged"] == 1 and info["trueRelResidual"] < 1e-9
    return KA.field_error(pts, nrm, w, x.cpu().numpy(), srcs, tgt)


def test_point_sources_inside_scatterers(ctx):
    e12, e24 = _gpu_error(ctx, 12), _gpu_error(ctx, 24)
    # the oracle's dense solve gives 9.3e-3 and 1.13e-4
    assert e12 < 2e-2 and e24 < 3e-4
    assert e12 / e24 > 30
