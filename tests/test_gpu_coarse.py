"""The two-level preconditioner on the GPU (bfg_coarse.cu) against the CPU
oracle (oracle/coarse_oracle.py) on the dense multiple-scattering system of
16 circles with C5's statistics (radii 0.05-0.15, gap 0.05, k = 200, 12
points per wavelength, the 16-circle layout of tests/test_coarse_oracle.py;
3,963 unknowns).

Bars:
  * the coarse dimension equals the oracle's mode count from the weights;
  * A_c = Phi^H A Phi within 1e-4 of the oracle's dense FP64 A_c (the GPU
    applies the butterfly part in split-BF16, ~1e-6, and accumulates the
    coarse quantities in FP32);
  * the block Gauss-Jordan inverse: ||A_c^-1 A_c - I|| / sqrt(dim) < 1e-4;
  * the coarse correction Phi A_c^-1 Phi^H r within 1e-4 of the oracle's;
  * FGMRES with the two-level preconditioner converges to a 1e-8 true
    residual in at most the oracle's multiplicative iteration count + 2,
    its solution within 1e-6 of the dense solve."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import bf_oracle as O
from oracle import coarse_oracle as C

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402

K = 200.0
EXTRA = 5


@pytest.fixture(scope="module")
def problem():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.default_context(0)
    pts, nrm, w, off, circles = B.scattering_geometry(num=16, k=K, ppw=12, rmin=0.05, rmax=0.15,
                                                      box=1.0, gap=0.05, seed=0)
    helm = B.Helm2(K, B.LayerPot.CombinedField, alpha=-1j * K, beta=1.0)
    fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm, leaf_size=64),
                                     B.Quadtree(pts, leaf_size=64), rank_eps=1e-10,
                                     pinv_tol=1e-10, context=ctx)
    sys_ = B.System(fac, pts, nrm, w, off, kr_order=6, diag_shift=0.5)
    sys_.build_block_jacobi()
    dim = sys_.build_coarse(EXTRA)
    ohelm = O.Helm2(K, O.LP_COMBINED_FIELD, -1j * K, 1.0)
    A = O.cfie_system_dense(ohelm, pts, nrm, w, off, 6, 0.5)
    q = C.mode_counts_from_weights(w, off, K, EXTRA)
    coarse = C.FourierCoarse(A, off, circles, K, modes=q)
    d = np.array([np.cos(0.7), np.sin(0.7)])
    b = -np.exp(1j * K * (pts @ d))                 # incident plane wave (setUpRhs)
    return dict(sys=sys_, dim=dim, A=A, coarse=coarse, b=b, off=off)


def test_coarse_operator_and_inverse(problem):
    p = problem
    assert p["dim"] == p["coarse"].dim
    ac, ai = p["sys"].coarse_matrices()
    ac = ac.cpu().numpy().astype(np.complex128)
    ai = ai.cpu().numpy().astype(np.complex128)
    assert rel_err(ac, p["coarse"].Ac) < 1e-4
    eye = np.eye(p["dim"])
    assert np.linalg.norm(ai @ ac - eye) / np.sqrt(p["dim"]) < 1e-4


def test_coarse_correction_matches_the_oracle(problem):
    p = problem
    r = O.RefRng(12).complex_randn(len(p["b"]))
    z = p["sys"].apply_coarse(torch.from_numpy(r).cuda()).cpu().numpy()
    assert rel_err(z, p["coarse"].correction(r)) < 1e-4


@pytest.mark.parametrize("prec", ["fp64", "df64"])
def test_two_level_fgmres(problem, prec):
    p = problem
    A, b, sys_ = p["A"], p["b"], p["sys"]
    m_bj = C.block_jacobi(A, p["off"])
    _, it_oracle = C.fgmres(lambda v: A @ v, b, C.multiplicative(lambda v: A @ v, m_bj,
                                                                 p["coarse"]),
                            tol=1e-8, max_iter=200)
    sys_.set_apply_precision(prec)
    x, info = B.solve_gmres(sys_, torch.from_numpy(b).cuda(), tol=1e-8, max_num_iter=200,
                            precond="two_level")
    _, info_bj = B.solve_gmres(sys_, torch.from_numpy(b).cuda(), tol=1e-8, max_num_iter=400,
                               precond="block_jacobi")
    sys_.set_apply_precision("fp64")
    assert info["converged"] and info["trueRelResidual"] < 1e-8
    assert info["iterations"] <= it_oracle + 2
    assert info["iterations"] * 4 <= info_bj["iterations"]
    xs = np.linalg.solve(A, b)
    assert rel_err(x.cpu().numpy(), xs) < 1e-6
