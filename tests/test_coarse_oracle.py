"""The two-level preconditioner oracle (oracle/coarse_oracle.py) on the
dense multiple-scattering system of 16 circles with C5's statistics (radii
0.05-0.15, gap 0.05, k = 200, 12 points per wavelength, C5's density of
circles): its FGMRES reproduces the dense solve, and a per-circle Fourier
coarse space of the radiating modes cuts block-Jacobi's iterations several
times over (measured: 79 -> 29 additive, 8 multiplicative)."""
import numpy as np
import pytest

import butterfly_gb300 as B
from oracle import bf_oracle as O
from oracle import coarse_oracle as C

K = 200.0


@pytest.fixture(scope="module")
def system():
    pts, nrm, w, off, circles = B.scattering_geometry(num=16, k=K, ppw=12, rmin=0.05, rmax=0.15,
                                                      box=1.0, gap=0.05, seed=0)
    helm = O.Helm2(K, O.LP_COMBINED_FIELD, -1j * K, 1.0)
    A = O.cfie_system_dense(helm, pts, nrm, w, off, 6, 0.5)
    d = np.array([np.cos(0.7), np.sin(0.7)])
    b = -np.exp(1j * K * (pts @ d))             # incident plane wave (setUpRhs)
    return A, b, off, circles


def _solve(A, b, precond):
    x, it = C.fgmres(lambda v: A @ v, b, precond, tol=1e-8, max_iter=400)
    res = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    return x, it, res


def test_fgmres_matches_the_dense_solve(system):
    A, b, off, _ = system
    x, it, res = _solve(A, b, C.block_jacobi(A, off))
    assert res < 1e-8
    xs = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-6
    assert 60 <= it <= 100                      # measured 79


def test_fourier_coarse_space_cuts_iterations(system):
    A, b, off, circles = system
    m_bj = C.block_jacobi(A, off)
    _, it_bj, _ = _solve(A, b, m_bj)
    coarse = C.FourierCoarse(A, off, circles, K, extra=0)
    assert coarse.dim < 0.2 * len(b)            # measured 692 of 3,963
    _, it_add, res_add = _solve(A, b, C.additive(m_bj, coarse))
    _, it_mul, res_mul = _solve(A, b, C.multiplicative(lambda v: A @ v, m_bj, coarse))
    assert res_add < 1e-8 and res_mul < 1e-8
    assert it_add * 2 <= it_bj                  # measured 29 against 79
    assert it_mul * 6 <= it_bj                  # measured 8


def test_block_gauss_jordan_inverts_the_coarse_operator(system):
    """The GPU's algorithm for A_c^-1: block pivots on the circles' mode
    blocks, no pivoting across blocks.  On the coarse operator of the CFIE
    it agrees with LAPACK's inverse to rounding."""
    A, b, off, circles = system
    w = np.concatenate([np.full(int(off[i + 1] - off[i]), 2 * np.pi * circles[i][2] /
                                (off[i + 1] - off[i])) for i in range(len(off) - 1)])
    q = C.mode_counts_from_weights(w, off, K, extra=5)
    assert q == [min(int(np.ceil(K * c[2])) + 5, (int(off[i + 1] - off[i]) - 1) // 2)
                 for i, c in enumerate(circles)]
    coarse = C.FourierCoarse(A, off, circles, K, modes=q)
    Ainv = C.block_gauss_jordan(coarse.Ac, coarse.start)
    ref = np.linalg.inv(coarse.Ac)
    assert np.linalg.norm(Ainv - ref) / np.linalg.norm(ref) < 1e-10
    # and on a matrix that needs row exchanges inside a block
    rng = np.random.default_rng(3)
    M = rng.standard_normal((12, 12)) + 1j * rng.standard_normal((12, 12))
    M[:4, :4] = 6 * np.fliplr(np.eye(4))      # zero diagonal: block 0 needs row exchanges
    M += 8 * np.eye(12) * (np.arange(12) >= 4)
    Minv = C.block_gauss_jordan(M, [0, 4, 8, 12])
    assert np.linalg.norm(Minv @ M - np.eye(12)) < 1e-10
