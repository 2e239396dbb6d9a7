"""The learned preconditioner's CPU oracle (oracle/mlp_oracle.py): its
analytic gradient against central finite differences, its Adam step against
the published update, and its chunk features on a hand-made case."""
import numpy as np

from oracle import mlp_oracle as M


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    shape = (6, 5, 4)
    n = M.layout(*shape)[-1]
    p = rng.standard_normal(n) * 0.5
    X = rng.standard_normal((7, 6))
    T = rng.standard_normal((7, 4))
    loss, g = M.loss_and_grad(p, X, T, shape)
    h = 1e-6
    fd = np.empty(n)
    for i in range(n):
        e = np.zeros(n)
        e[i] = h
        fd[i] = (M.loss_and_grad(p + e, X, T, shape)[0] - M.loss_and_grad(p - e, X, T, shape)[0]) / (2 * h)
    assert np.max(np.abs(fd - g)) < 1e-7 * max(1.0, np.max(np.abs(g)))
    assert loss > 0


def test_adam_first_step_moves_by_lr():
    # the first bias-corrected step is lr * g / (|g| + eps) ~ lr * sign(g)
    p = np.zeros(3)
    g = np.array([2.0, -0.5, 1e-3])
    q, m, v = M.adam_step(p, g, np.zeros(3), np.zeros(3), 1, 0.01)
    assert np.allclose(q, -0.01 * np.sign(g), rtol=1e-4)


def test_chunk_features():
    off = np.array([0, 3, 8])
    r = np.arange(8) + 1j * np.arange(8)[::-1]
    z = 2 * r
    e = 3 * r
    F, T, S = M.learned_pairs(r, z, e, off, 4)
    assert F.shape == (3, 16) and T.shape == (3, 8)          # chunks [0,3), [3,7), [7,8)
    assert np.isclose(abs(S[0]), np.linalg.norm(r[0:3]))
    w = 1 / S                                                 # conj(p) / s
    assert np.allclose(F[0, 0:6:2], (r[0:3] * w[0]).real) and np.all(F[0, 6:8] == 0)
    assert np.allclose(F[1, 8:16:2], (z[3:7] * w[1]).real)
    d = (e[7] - z[7]) * w[2]
    assert np.allclose(T[2, 0:2], [d.real, d.imag])
    # a complex scaling of the inputs leaves the features unchanged
    F2, T2, _ = M.learned_pairs((0.3 - 2j) * r, (0.3 - 2j) * z, (0.3 - 2j) * e, off, 4)
    assert np.allclose(F2, F) and np.allclose(T2, T)
