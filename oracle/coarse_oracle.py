"""Test infrastructure -- a CPU oracle for two-level preconditioning of the
multiple-scattering system (dense, float64).

Only ``tests/`` may import it, as the reference for a GPU two-level
preconditioner and for the iteration counts that motivate one.  Block-Jacobi
(the reference's assemblePreconditioner, multiple_scattering_context.c:
545-634) inverts each scatterer's self-interaction; what it leaves is the
coupling between scatterers.  A coarse space of the low-order Fourier modes
of every circle, e^{i m theta}, |m| <= ceil(k r) + extra (the modes that
radiate), carries most of that coupling:

  additive:        z = M_bj r + Phi A_c^-1 Phi^H r
  multiplicative:  z1 = Phi A_c^-1 Phi^H r,  z = z1 + M_bj (r - A z1)

with A_c = Phi^H A Phi, inverted by block Gauss-Jordan elimination over the
circles' mode blocks (block_gauss_jordan, the GPU's algorithm).  The solver
is right-preconditioned flexible GMRES
(the method's FGMRES, linalg.c:47-317 with the preconditioner on the right)
with classical Gram-Schmidt and a second orthogonalisation pass.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla


def fgmres(apply_a, b, precond, tol=1e-8, max_iter=1000):
    """Right-preconditioned FGMRES from x0 = 0: (x, iterations) with
    ||b - A x|| <= tol ||b|| by the Arnoldi estimate."""
    n = len(b)
    beta = float(np.linalg.norm(b))
    if beta == 0.0:
        return np.zeros(n, complex), 0
    V = np.zeros((n, max_iter + 1), complex)
    Z = np.zeros((n, max_iter), complex)
    H = np.zeros((max_iter + 1, max_iter), complex)
    cs = np.zeros(max_iter)                 # Givens cosines (real)
    sn = np.zeros(max_iter, complex)        # Givens sines
    g = np.zeros(max_iter + 1, complex)
    g[0] = beta
    V[:, 0] = b / beta
    for j in range(max_iter):
        Z[:, j] = precond(V[:, j])
        w = apply_a(Z[:, j])
        for _ in range(2):                  # CGS, twice
            h = V[:, :j + 1].conj().T @ w
            w = w - V[:, :j + 1] @ h
            H[:j + 1, j] += h
        H[j + 1, j] = np.linalg.norm(w)
        if H[j + 1, j] > 0:
            V[:, j + 1] = w / H[j + 1, j]
        for i in range(j):                  # earlier rotations on the new column
            t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
            H[i + 1, j] = -np.conj(sn[i]) * H[i, j] + cs[i] * H[i + 1, j]
            H[i, j] = t
        a, c = H[j, j], H[j + 1, j]
        den = math.hypot(abs(a), abs(c))
        if abs(a) == 0.0:
            cs[j], sn[j] = 0.0, 1.0
        else:
            cs[j] = abs(a) / den
            sn[j] = (a / abs(a)) * np.conj(c) / den
        H[j, j] = cs[j] * a + sn[j] * c
        H[j + 1, j] = 0.0
        g[j + 1] = -np.conj(sn[j]) * g[j]
        g[j] = cs[j] * g[j]
        if abs(g[j + 1]) <= tol * beta or H[j + 1, j] == 0 and j + 1 == n:
            y = sla.solve_triangular(H[:j + 1, :j + 1], g[:j + 1])
            return Z[:, :j + 1] @ y, j + 1
    y = sla.solve_triangular(H[:max_iter, :max_iter], g[:max_iter])
    return Z[:, :max_iter] @ y, max_iter


def block_jacobi(A, offsets):
    """z = blockdiag(A_bb)^-1 r over the curves' point ranges."""
    inv = [np.linalg.inv(A[offsets[b]:offsets[b + 1], offsets[b]:offsets[b + 1]])
           for b in range(len(offsets) - 1)]

    def apply(r):
        z = np.empty_like(r)
        for b, ib in enumerate(inv):
            z[offsets[b]:offsets[b + 1]] = ib @ r[offsets[b]:offsets[b + 1]]
        return z
    return apply


def mode_counts_from_weights(weights, offsets, k, extra=0):
    """Modes |m| <= q_b per curve from its quadrature weights: q_b =
    min(ceil(k L_b / 2 pi) + extra, (n_b - 1) / 2), L_b = sum of the curve's
    weights (its length: 2 pi r for a circle, so q_b = ceil(k r) + extra),
    as bfgSystemBuildCoarse counts them."""
    q = []
    for b in range(len(offsets) - 1):
        nb = int(offsets[b + 1] - offsets[b])
        L = float(np.sum(weights[offsets[b]:offsets[b + 1]]))
        q.append(max(0, min(int(math.ceil(k * L / (2.0 * math.pi))) + extra, (nb - 1) // 2)))
    return q


def block_gauss_jordan(A, starts):
    """The inverse of A by block Gauss-Jordan elimination with the diagonal
    blocks [starts[b], starts[b+1]) as pivots in order (partial pivoting only
    inside a block's own inverse), as the GPU inverts A_c: for block K and
    the rest O,
      P = A_KK^-1;  A_KO <- P A_KO;  A_OO <- A_OO - A_OK A_KO;
      A_OK <- -A_OK P;  A_KK <- P."""
    A = np.array(A, dtype=complex)
    for b in range(len(starts) - 1):
        K = slice(int(starts[b]), int(starts[b + 1]))
        P = np.linalg.inv(A[K, K])
        T = P @ A[K, :]
        U = A[:, K].copy()
        U[K, :] = 0
        A -= U @ T
        A[:, K] = -U @ P
        A[K, :] = T
        A[K, K] = P
    return A


class FourierCoarse:
    """The per-circle Fourier coarse space and its exact coarse solve.

    circles: (num, 3) rows (cx, cy, r); offsets: curve point ranges (each
    circle sampled at equispaced angles 2 pi j / n_b, as scattering_geometry
    places them); modes per circle |m| <= min(ceil(k r) + extra, (n_b-1)/2)."""

    def __init__(self, A, offsets, circles, k, extra=0, modes=None):
        self.offsets = np.asarray(offsets)
        self.bases, start = [], [0]
        for b in range(len(offsets) - 1):
            nb = int(offsets[b + 1] - offsets[b])
            q = modes[b] if modes is not None else \
                min(int(math.ceil(k * circles[b][2])) + extra, (nb - 1) // 2)
            th = 2.0 * np.pi * np.arange(nb) / nb
            self.bases.append(np.exp(1j * np.outer(th, np.arange(-q, q + 1))) / math.sqrt(nb))
            start.append(start[-1] + 2 * q + 1)
        self.start = np.asarray(start)
        self.dim = int(start[-1])
        AP = np.empty((A.shape[0], self.dim), complex)
        for b, Pb in enumerate(self.bases):
            AP[:, start[b]:start[b + 1]] = A[:, offsets[b]:offsets[b + 1]] @ Pb
        self.Ac = self.restrict_rows(AP)
        self.lu = sla.lu_factor(self.Ac)

    def restrict(self, r):
        """Phi^H r."""
        return np.concatenate([Pb.conj().T @ r[self.offsets[b]:self.offsets[b + 1]]
                               for b, Pb in enumerate(self.bases)])

    def restrict_rows(self, M):
        out = np.empty((self.dim, M.shape[1]), complex)
        for b, Pb in enumerate(self.bases):
            out[self.start[b]:self.start[b + 1]] = \
                Pb.conj().T @ M[self.offsets[b]:self.offsets[b + 1]]
        return out

    def prolong(self, y):
        """Phi y."""
        z = np.empty(self.offsets[-1], complex)
        for b, Pb in enumerate(self.bases):
            z[self.offsets[b]:self.offsets[b + 1]] = Pb @ y[self.start[b]:self.start[b + 1]]
        return z

    def correction(self, r):
        """Phi A_c^-1 Phi^H r."""
        return self.prolong(sla.lu_solve(self.lu, self.restrict(r)))


def additive(m_bj, coarse):
    return lambda r: m_bj(r) + coarse.correction(r)


def multiplicative(apply_a, m_bj, coarse):
    def apply(r):
        z1 = coarse.correction(r)
        return z1 + m_bj(r - apply_a(z1))
    return apply
