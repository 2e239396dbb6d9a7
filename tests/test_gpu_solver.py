"""GPU tests of the boundary-integral system A = 1/2 I + (K + C) diag(w)
(combined field, Kapur-Rokhlin order 6), its block-Jacobi preconditioner and
FGMRES, against the CPU oracle's dense assembly of the same operator
(multiple_scattering_context.c:407-437 restated) and numpy's dense solve."""
import ctypes

import numpy as np
import pytest

from conftest import rel_err
from oracle import bf_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402

K = 40.0


@pytest.fixture(scope="module")
def problem():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = B.default_context(0)
    pts, nrm, w, off, circles = B.scattering_geometry(num=8, k=K, ppw=12, rmin=0.2, rmax=0.4,
                                                      box=2.0, gap=0.1, seed=3)
    helm = B.Helm2(K, B.LayerPot.CombinedField, alpha=-1j * K, beta=1.0)
    fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm), B.Quadtree(pts), context=ctx)
    sys_ = B.System(fac, pts, nrm, w, off, kr_order=6, diag_shift=0.5)
    ohelm = O.Helm2(K, O.LP_COMBINED_FIELD, -1j * K, 1.0)
    A = O.cfie_system_dense(ohelm, pts, nrm, w, off, 6, 0.5)
    d = np.array([np.cos(0.7), np.sin(0.7)])
    b = -np.exp(1j * K * (pts @ d))                 # incident plane wave (setUpRhs)
    return dict(ctx=ctx, pts=pts, nrm=nrm, w=w, off=off, fac=fac, sys=sys_, A=A, b=b)


def test_system_apply_matches_dense_oracle(problem):
    A, sys_ = problem["A"], problem["sys"]
    x = O.RefRng(9).complex_randn(A.shape[0])
    y = sys_.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel_err(y, A @ x) < 1e-9


def test_block_jacobi_inverts_the_diagonal_blocks(problem):
    A, sys_, off = problem["A"], problem["sys"], problem["off"]
    sys_.build_block_jacobi()
    r = O.RefRng(10).complex_randn(A.shape[0])
    z = sys_.apply_block_jacobi(torch.from_numpy(r).cuda()).cpu().numpy()
    zo = np.concatenate([np.linalg.solve(A[a:b, a:b], r[a:b]) for a, b in zip(off[:-1], off[1:])])
    # the blocks come from the dense kernel, the same as the oracle's
    assert rel_err(z, zo) < 1e-11


@pytest.mark.parametrize("precond", ["none", "block_jacobi"])
def test_gmres_solution_matches_dense_solve(problem, precond):
    A, sys_, b = problem["A"], problem["sys"], problem["b"]
    if precond == "block_jacobi":
        sys_.build_block_jacobi()
    # without a preconditioner the multiple-scattering operator needs many
    # iterations; full GMRES terminates within n steps
    x, info = B.solve_gmres(sys_, torch.from_numpy(b).cuda(), tol=1e-10, max_num_iter=A.shape[0],
                            precond=precond)
    assert info["converged"] == 1
    assert info["trueRelResidual"] < 1e-9
    xo = np.linalg.solve(A, b)
    assert rel_err(x.cpu().numpy(), xo) < 1e-7
    problem.setdefault("iters", {})[precond] = info["iterations"]


def test_preconditioning_reduces_iterations_and_user_callback(problem):
    sys_, b = problem["sys"], problem["b"]
    sys_.build_block_jacobi()
    lib = B._solver_sigs()

    def user(r, z, stream):                     # the same block-Jacobi, via the callback
        st = lib.bfgSystemApplyBlockJacobi(sys_.handle, ctypes.c_void_p(r), ctypes.c_void_p(z))
        if st != 0:
            raise RuntimeError("precond failed")

    bt = torch.from_numpy(b).cuda()
    _, i_none = B.solve_gmres(sys_, bt, tol=1e-8, max_num_iter=len(b), precond="none")
    _, i_bj = B.solve_gmres(sys_, bt, tol=1e-8, max_num_iter=400, precond="block_jacobi")
    _, i_cb = B.solve_gmres(sys_, bt, tol=1e-8, max_num_iter=400, precond=user)
    assert i_bj["iterations"] < i_none["iterations"]
    # the built-in preconditioner applies an FP32 copy of the same inverses
    # (the callback here uses the FP64 ones): a flexible solver may take an
    # iteration more or less, no more
    assert abs(i_cb["iterations"] - i_bj["iterations"]) <= 2
    assert i_cb["trueRelResidual"] < 1e-7


def test_kr_correction_restates_reference(problem):
    """The oracle's KR entries (restating quadrature.c and K_helm2) are what
    the reference adds: spot-check one row against the formula."""
    pts, nrm, off = problem["pts"], problem["nrm"], problem["off"]
    h = O.Helm2(K, O.LP_COMBINED_FIELD, -1j * K, 1.0)
    r, c, v = O.kr_correction(h, pts, nrm, off, 6)
    i = 5
    m = off[1] - off[0]
    sel = r == i
    assert sel.sum() == 12
    j = (i + 1) % m
    k = O.kernel_pairs(h, pts[[i]], nrm[[i]], pts[[j]])[0]
    assert np.isclose(v[sel][0], O.KR_WEIGHTS[6][0] * k)


def test_df64_system_apply_and_gmres(problem):
    """Double-float matvecs (FP32 arithmetic, ~48 bits): the system apply
    within 1e-12 of FP64, and FGMRES on them reaches the same solution with a
    true FP64 residual below the tolerance."""
    A, sys_, b = problem["A"], problem["sys"], problem["b"]
    x = torch.from_numpy(O.RefRng(12).complex_randn(A.shape[0])).cuda()
    y64 = sys_.apply(x)
    sys_.set_apply_precision("df64")
    try:
        ydf = sys_.apply(x)
        assert rel_err(ydf.cpu().numpy(), y64.cpu().numpy()) < 1e-12
        sys_.build_block_jacobi()
        xs, info = B.solve_gmres(sys_, torch.from_numpy(b).cuda(), tol=1e-10, max_num_iter=400,
                                 precond="block_jacobi")
    finally:
        sys_.set_apply_precision("fp64")
    assert info["converged"] == 1 and info["trueRelResidual"] < 1e-9
    assert rel_err(xs.cpu().numpy(), np.linalg.solve(A, b)) < 1e-7
    with pytest.raises(B.BfgError):
        sys_.set_apply_precision("fp32")
