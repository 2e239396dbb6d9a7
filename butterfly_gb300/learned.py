"""Learned right preconditioner for flexible GMRES on the multiple-scattering
system (a GB300 addition; the reference preconditions with block-Jacobi
only, multiple_scattering_context.c:545-634).

The network (bfgMlp*, hand-written FP32 kernels in csrc/bfg_mlp.cu) maps, for
every chunk of `chunk` consecutive points of a curve, the chunk's residual
and block-Jacobi output (scaled by 1 / ||r_chunk||) to a correction added to
the block-Jacobi output.  Training pairs come from the method's own GMRES
solves: for an iterate x_j of a solve of A x = b with solution x*, the
residual r_j = b - A x_j and the exact correction e_j = x* - x_j = A^-1 r_j.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import (BfgError, Context, _I64, _VP, _ptr, _solver_sigs, default_context, lib,
               solve_gmres)

_F32P = ctypes.POINTER(ctypes.c_float)


def _sigs():
    L = _solver_sigs()
    if getattr(L, "_mlp_sigs", False):
        return L
    sig = {
        "bfgMlpCreate": [_VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
                         ctypes.POINTER(_VP)],
        "bfgMlpDestroy": [_VP],
        "bfgMlpGetShape": [_VP, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                           ctypes.POINTER(ctypes.c_int32)],
        "bfgMlpNumParams": [_VP, ctypes.POINTER(_I64)],
        "bfgMlpGetParams": [_VP, _VP],
        "bfgMlpSetParams": [_VP, _VP],
        "bfgMlpForward": [_VP, _VP, _I64, _VP],
        "bfgMlpGradients": [_VP, _VP, _VP, _I64, _VP, ctypes.POINTER(ctypes.c_double)],
        "bfgMlpTrainStep": [_VP, _VP, _VP, _I64, ctypes.c_float, ctypes.POINTER(ctypes.c_double)],
        "bfgSystemSetLearnedPreconditioner": [_VP, _VP, ctypes.c_int32],
        "bfgSystemLearnedNumChunks": [_VP, ctypes.POINTER(_I64)],
        "bfgSystemLearnedPairs": [_VP, _VP, _VP, _VP, _VP],
    }
    for name, args in sig.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = ctypes.c_int
    L._mlp_sigs = True
    return L


def _check(st, what):
    if st != 0:
        raise BfgError(st, what)


class Mlp:
    """n_in -> n_hidden -> n_hidden -> n_out perceptron with ReLU, FP32 on the
    GPU (bfgMlpCreate).  Arrays: torch float32 CUDA tensors, row-major."""

    def __init__(self, n_in: int, n_hidden: int, n_out: int, seed: int = 0,
                 context: Context | None = None):
        self.ctx = context or default_context()
        h = _VP()
        _check(_sigs().bfgMlpCreate(self.ctx.handle, n_in, n_hidden, n_out, seed, ctypes.byref(h)),
               "mlp create")
        self.handle = h
        self.shape = (n_in, n_hidden, n_out)
        n = _I64()
        _check(_sigs().bfgMlpNumParams(h, ctypes.byref(n)), "mlp params")
        self.num_params = n.value

    def close(self):
        if getattr(self, "handle", None) and lib() is not None:
            _sigs().bfgMlpDestroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self):
        import torch
        return self.ctx.on_stream(torch.cuda.current_stream().cuda_stream)

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, dtype=np.float32)
        _check(_sigs().bfgMlpGetParams(self.handle, _ptr(p)), "mlp get")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError("expected %d parameters" % self.num_params)
        _check(_sigs().bfgMlpSetParams(self.handle, _ptr(p)), "mlp set")

    def forward(self, X):
        import torch
        X = X.to(torch.float32).contiguous()
        Y = torch.empty((X.shape[0], self.shape[2]), dtype=torch.float32, device=X.device)
        with self._stream():
            _check(_sigs().bfgMlpForward(self.handle, _VP(X.data_ptr()), X.shape[0],
                                         _VP(Y.data_ptr())), "mlp forward")
        return Y

    def gradients(self, X, T):
        """(loss, gradient as a float32 numpy array); no update."""
        g = np.empty(self.num_params, dtype=np.float32)
        loss = ctypes.c_double()
        with self._stream():
            _check(_sigs().bfgMlpGradients(self.handle, _VP(X.data_ptr()), _VP(T.data_ptr()),
                                           X.shape[0], _ptr(g), ctypes.byref(loss)), "mlp grad")
        return loss.value, g

    def train_step(self, X, T, lr: float) -> float:
        loss = ctypes.c_double()
        with self._stream():
            _check(_sigs().bfgMlpTrainStep(self.handle, _VP(X.data_ptr()), _VP(T.data_ptr()),
                                           X.shape[0], float(lr), ctypes.byref(loss)), "mlp step")
        return loss.value


def set_learned(system, mlp: Mlp, chunk: int):
    """Makes `mlp` the system's learned preconditioner (solve_gmres with
    precond="learned"); block-Jacobi must be built."""
    system._check(_sigs().bfgSystemSetLearnedPreconditioner(system.handle, mlp.handle, chunk),
                  "learned preconditioner")
    system._learned = mlp      # keeps the network alive while the system uses it


def num_chunks(system) -> int:
    n = _I64()
    system._check(_sigs().bfgSystemLearnedNumChunks(system.handle, ctypes.byref(n)), "chunks")
    return n.value


def learned_pairs(system, r, e=None):
    """(features, targets) of residual r and exact correction e (device
    complex128 vectors, original point order); targets None without e."""
    import torch
    mlp = system._learned
    nc = num_chunks(system)
    F = torch.empty((nc, mlp.shape[0]), dtype=torch.float32, device="cuda")
    T = torch.empty((nc, mlp.shape[2]), dtype=torch.float32, device="cuda") if e is not None else None
    with system.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
        system._check(_sigs().bfgSystemLearnedPairs(
            system.handle, _VP(r.data_ptr()), _VP(e.data_ptr()) if e is not None else None,
            _VP(F.data_ptr()), _VP(T.data_ptr()) if T is not None else None), "learned pairs")
    return F, T


def collect_pairs(system, b, iterates=(0, 10, 30, 80), tol=1e-10):
    """Training pairs of one right-hand side: the full solve gives x*; the
    iterates x_j of solves stopped after j iterations give r_j = b - A x_j
    and e_j = x* - x_j.  Uses block-Jacobi (the network is not needed)."""
    import torch
    xs, info = solve_gmres(system, b, tol=tol, max_num_iter=3000, precond="block_jacobi")
    F, T = [], []
    for j in iterates:
        if j == 0:
            xj = torch.zeros_like(b)
        else:
            xj, _ = solve_gmres(system, b, tol=1e-30, max_num_iter=j, precond="block_jacobi")
        rj = b - system.apply(xj)
        f, t = learned_pairs(system, rj, xs - xj)
        F.append(f)
        T.append(t)
    return torch.cat(F), torch.cat(T), int(info["iterations"])


def train(mlp: Mlp, F, T, epochs: int = 40, batch: int = 2048, lr: float = 1e-3, seed: int = 0):
    """Adam on shuffled mini-batches; returns the mean loss of each epoch."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = F.shape[0]
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g).to(F.device)
        tot, cnt = 0.0, 0
        for a in range(0, n, batch):
            idx = perm[a:a + batch]
            x = F.index_select(0, idx).contiguous()
            t = T.index_select(0, idx).contiguous()
            tot += mlp.train_step(x, t, lr) * len(idx)
            cnt += len(idx)
        losses.append(tot / max(cnt, 1))
    return losses
