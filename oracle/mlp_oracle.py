"""CPU oracle for the learned preconditioner (test infrastructure only: the
tests use it to check the GPU kernels; nothing in the product path imports
it).  Float64 numpy restatement of bfgMlp* (butterfly_gb300/csrc/bfg_mlp.cu,
bfg_mlp_api.cpp) and of the chunk features and targets of
bfgSystemLearnedPairs (bfg_solver.cu).  The reference has no learned
preconditioner (it preconditions with block-Jacobi only,
multiple_scattering_context.c:545-634), so there is nothing of the
reference's to pin this oracle to; it is pinned by finite differences
instead (tests/test_mlp_oracle.py)."""
import numpy as np


def layout(n_in, n_hid, n_out):
    """Offsets of W1, b1, W2, b2, W3, b3 in the flat parameter array."""
    sizes = [n_in * n_hid, n_hid, n_hid * n_hid, n_hid, n_hid * n_out, n_out]
    off = np.concatenate([[0], np.cumsum(sizes)])
    return off


def unpack(params, n_in, n_hid, n_out):
    p = np.asarray(params, dtype=np.float64)
    o = layout(n_in, n_hid, n_out)
    W1 = p[o[0]:o[1]].reshape(n_in, n_hid)
    b1 = p[o[1]:o[2]]
    W2 = p[o[2]:o[3]].reshape(n_hid, n_hid)
    b2 = p[o[3]:o[4]]
    W3 = p[o[4]:o[5]].reshape(n_hid, n_out)
    b3 = p[o[5]:o[6]]
    return W1, b1, W2, b2, W3, b3


def forward(params, X, shape):
    """y = relu(relu(x W1 + b1) W2 + b2) W3 + b3 for every row x of X."""
    W1, b1, W2, b2, W3, b3 = unpack(params, *shape)
    H1 = np.maximum(X @ W1 + b1, 0.0)
    H2 = np.maximum(H1 @ W2 + b2, 0.0)
    return H2 @ W3 + b3, H1, H2


def loss_and_grad(params, X, T, shape):
    """mean_b 0.5 ||y_b - t_b||^2 and its gradient (flat, parameter layout)."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(params, *shape)
    Y, H1, H2 = forward(params, X, shape)
    B = X.shape[0]
    D = Y - T
    loss = 0.5 * np.sum(D * D) / B
    dY = D / B
    gW3 = H2.T @ dY
    gb3 = dY.sum(0)
    dH2 = (dY @ W3.T) * (H2 > 0)
    gW2 = H1.T @ dH2
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2.T) * (H1 > 0)
    gW1 = X.T @ dH1
    gb1 = dH1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def adam_step(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma and Ba 2015); returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def chunks(offsets, chunk):
    """(start, length) of the chunks of `chunk` consecutive points of each
    curve [offsets[b], offsets[b+1])."""
    out = []
    for a, b in zip(offsets[:-1], offsets[1:]):
        for s in range(int(a), int(b), chunk):
            out.append((s, min(chunk, int(b) - s)))
    return out


def learned_pairs(r, zbj, e, offsets, chunk):
    """Features conj(p) (r_c, zbj_c) / s and targets conj(p) (e_c - zbj_c) / s
    of every chunk, s = ||r_c||, p the phase of sum_t |r_t| r_t, as
    interleaved (re, im) pairs zero-padded to `chunk`; S = (s, p) per chunk."""
    ch = chunks(offsets, chunk)
    F = np.zeros((len(ch), 4 * chunk))
    T = np.zeros((len(ch), 2 * chunk))
    S = np.zeros(len(ch), dtype=np.complex128)
    for c, (s, L) in enumerate(ch):
        rc, zc = r[s:s + L], zbj[s:s + L]
        sN = np.sqrt(np.sum(np.abs(rc) ** 2))
        rho = np.sum(np.abs(rc) * rc)
        p = rho / abs(rho) if abs(rho) > 0 else 1.0
        w = np.conj(p) / sN if sN > 0 else 0.0
        S[c] = sN * p
        F[c, 0:2 * L:2], F[c, 1:2 * L:2] = (rc * w).real, (rc * w).imag
        F[c, 2 * chunk:2 * chunk + 2 * L:2] = (zc * w).real
        F[c, 2 * chunk + 1:2 * chunk + 2 * L:2] = (zc * w).imag
        if e is not None:
            d = (e[s:s + L] - zc) * w
            T[c, 0:2 * L:2], T[c, 1:2 * L:2] = d.real, d.imag
    return F, T, S
