"""The relative pseudo-inverse cut (the tolerance semantics of
bfTruncSpecGetNumTerms, linalg.c:26-36: keep sigma_k while
sigma_k >= tol * sigma_0, singular values in descending order) as the oracle
applies it with scipy's zgesvd, on a constructed spectrum with a singular
value exactly at the cut and on real re-expansion blocks.  The GPU kernels'
cut is checked against this oracle in tests/test_gpu_cut.py."""
import numpy as np

from oracle import bf_oracle as O


def reference_num_terms(S, tol):
    """linalg.c:26-36, restated."""
    k = 0
    while k < len(S) and S[k] >= tol * S[0]:
        k += 1
    return k


def test_cut_keeps_singular_values_at_the_threshold():
    """A diagonal matrix, whose SVD LAPACK returns exactly: a singular value
    equal to tol * sigma_0 is kept (>=), the ones below it are cut."""
    tol = 1e-8
    S = np.array([2.0, 1.0, 3e-3, 2.0 * tol, 1.0 * tol, 0.5 * tol])
    A = np.diag(S).astype(np.complex128)
    B = np.arange(12.0).reshape(6, 2) + 1j
    X, k, Sc = O.lstsq_pinv(A, B, "relative", tol, return_terms=True)
    assert np.array_equal(Sc, S)
    assert k == reference_num_terms(Sc, tol) == 4
    # the kept part solves its rows exactly, the cut rows are left at zero
    assert np.allclose(X[:4], B[:4] / S[:4, None], rtol=1e-15, atol=0)
    assert not np.any(X[4:])


def test_cut_count_on_reexpansion_blocks():
    k, tol = 256.0, 1e-8
    src = O.uniform_square_points(8192, 0)
    tgt = O.curve_points("star", 8192)
    ts, tt = O.Quadtree(src, 64), O.Quadtree(tgt, 64)
    root = O.Planner(k, ts, tt, eps=tol).plan()
    blocks = [b for b in O.iter_blocks(root) if b.kind == "middle"][::97][:12]
    h = O.Helm2(k)
    for b in blocks:
        eq, _ = O.circle_points(b.ceq, b.m)
        chk, _ = O.circle_points(b.cchk, b.m)
        orig, _ = O.circle_points(b.corig, b.n)
        Ze = O.kernel_matrix(h, eq, chk)
        Zo = O.kernel_matrix(h, orig, chk)
        X, n, S = O.lstsq_pinv(Ze, Zo, "relative", tol, return_terms=True)
        assert n == reference_num_terms(S, tol)
        assert 0 < n < b.m                          # the cut is active on these blocks
        # dropping or adding the term at the cut changes the solution by far
        # more than the GPU kernels' agreement bar (tests/test_gpu_cut.py)
        U, _, VH = np.linalg.svd(Ze)
        for k2 in (n - 1, n + 1):
            X2 = VH[:k2].conj().T @ ((U[:, :k2].conj().T @ Zo) / S[:k2, None])
            assert np.linalg.norm(X2 - X) / np.linalg.norm(X) > 1e-3
