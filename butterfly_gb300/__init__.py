"""butterfly_gb300 -- GB300-native multilevel butterfly factorization of the
2-D Helmholtz kernel G(x, y) = (i/4) H0(k |x - y|), and its application to
vectors, on one GPU.

The Python surface mirrors the reference's Cython wrapper
(wrappers/python/butterfly.pyx): ``Helm2`` (273-305), ``LayerPot`` (330-354),
``FacHelm2.make_multilevel`` (211-220) and ``Mat.__matmul__`` (384-396).
Everything runs through the C ABI of ``libbfg.so`` (include/bfg.h); there is
no CPU fallback -- without the compiled library every call raises.
"""
from __future__ import annotations

import atexit
import ctypes
import enum
import os
import weakref
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libbfg.so")

BFG_OK = 0
APPLY_ORIGINAL_ORDER = 1
PRECISIONS = {"fp64": 0, "fp32": 1, "bf16x2": 2, "bf16x3": 3, "df64": 4}
# precisions whose vectors are complex128
_C128_PRECISIONS = ("fp64", "df64")
STATUS_NAMES = {0: "OK", 1: "INVALID_ARGUMENTS", 2: "RUNTIME", 3: "NOT_IMPLEMENTED",
                4: "MEMORY", 5: "OUT_OF_RANGE", 8: "INCOMPATIBLE_SHAPES", 32: "CUDA",
                33: "TIMEOUT", 34: "NUMERICAL"}


class BfgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, message))
        self.status = status


class _Helm2C(ctypes.Structure):
    _fields_ = [("k", ctypes.c_double), ("layerPot", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("alphaRe", ctypes.c_double),
                ("alphaIm", ctypes.c_double), ("betaRe", ctypes.c_double),
                ("betaIm", ctypes.c_double)]


class _FacOptionsC(ctypes.Structure):
    _fields_ = [("leafSize", ctypes.c_int64), ("rankEps", ctypes.c_double),
                ("pinvCut", ctypes.c_int32), ("treeOnGpu", ctypes.c_int32),
                ("pinvTol", ctypes.c_double), ("jacobiArith", ctypes.c_int32),
                ("sketch", ctypes.c_int32)]


class _QuadtreeNodeC(ctypes.Structure):
    _fields_ = [("xmin", ctypes.c_double), ("ymin", ctypes.c_double),
                ("xmax", ctypes.c_double), ("ymax", ctypes.c_double),
                ("splitX", ctypes.c_double), ("splitY", ctypes.c_double),
                ("i0", ctypes.c_int64), ("i1", ctypes.c_int64),
                ("parent", ctypes.c_int32), ("depth", ctypes.c_int32),
                ("child", ctypes.c_int32 * 4)]


QUADTREE_NODE_DTYPE = np.dtype([("xmin", "f8"), ("ymin", "f8"), ("xmax", "f8"), ("ymax", "f8"),
                                ("splitX", "f8"), ("splitY", "f8"), ("i0", "i8"), ("i1", "i8"),
                                ("parent", "i4"), ("depth", "i4"), ("child", "i4", (4,))])


class _FacStatsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "numRows", "numCols", "numBlocks", "numFirst", "numMiddle", "numLast",
        "numDense", "numProducts", "arenaEntries", "numStages", "numItems",
        "maxRank", "jacobiNotConverged")] + [(n, ctypes.c_double) for n in (
            "factorMs", "flopsPerRhs", "fillMs", "reexpSmemMs", "reexpGlobalMs")] + [
        (n, ctypes.c_int64) for n in (
            "numSketched", "sketchRetries", "sketchFallbacks", "sketchMaxWidth")] + [
        (n, ctypes.c_double) for n in ("sketchMs", "sketchMeanWidth")] + [
        ("applyBufferBytes", ctypes.c_int64), ("sketchPhaseMs", ctypes.c_double * 8),
        ("reexpSvds", ctypes.c_int64), ("sketchGroups", ctypes.c_int64)]


class _RngC(ctypes.Structure):
    _fields_ = [("s", ctypes.c_uint64 * 4)]


_lib = None
_VP = ctypes.c_void_p
_I64 = ctypes.c_int64


def lib() -> ctypes.CDLL:
    """The compiled library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise BfgError(2, "libbfg.so is missing; run __graft_entry__.build() "
                          "(or python -m butterfly_gb300.build)")
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "bfgContextCreate": [ctypes.c_int32, ctypes.POINTER(_VP)],
        "bfgContextDestroy": [_VP],
        "bfgContextSetStream": [_VP, _VP],
        "bfgContextGetStream": [_VP, ctypes.POINTER(_VP)],
        "bfgContextSynchronize": [_VP],
        "bfgFacOptionsDefault": [ctypes.POINTER(_FacOptionsC)],
        "bfgFacHelm2MakeMultilevel": [_VP, ctypes.POINTER(_Helm2C), _VP, _VP, _I64, _VP, _VP,
                                      _I64, ctypes.POINTER(_FacOptionsC), ctypes.POINTER(_VP)],
        "bfgFacHelm2MakeBatched": [_VP, ctypes.POINTER(_Helm2C), _VP, _I64, _VP, _VP, _VP, _VP,
                                   _VP, _VP, ctypes.POINTER(_FacOptionsC), ctypes.POINTER(_VP)],
        "bfgFacDestroy": [_VP],
        "bfgFacSave": [_VP, ctypes.c_char_p],
        "bfgFacLoad": [_VP, ctypes.c_char_p, ctypes.POINTER(_VP)],
        "bfgFacGetShape": [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
        "bfgFacGetPerms": [_VP, _VP, _VP],
        "bfgFacNumBytes": [_VP, ctypes.POINTER(_I64)],
        "bfgFacGetStats": [_VP, ctypes.POINTER(_FacStatsC)],
        "bfgFacDescribe": [_VP, ctypes.c_char_p, _I64, ctypes.POINTER(_I64)],
        "bfgFacCopyBlocks": [_VP, _VP, _I64, _VP, _I64],
        "bfgFacApply": [_VP, ctypes.c_int, _VP, _I64, _I64, _VP, _I64, ctypes.c_uint32],
        "bfgFacApplyHost": [_VP, ctypes.c_int, _VP, _I64, _I64, _VP, _I64, ctypes.c_uint32],
        "bfgFacApplyHostAsync": [_VP, ctypes.c_int, _VP, _I64, _I64, _VP, _I64, ctypes.c_uint32],
        "bfgFacApplyHostWait": [_VP],
        "bfgFacApplyTimed": [_VP, ctypes.c_int, _VP, _I64, _I64, _VP, _I64, ctypes.c_uint32,
                             _VP, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)],
        "bfgFacDenseRows": [_VP, _VP, _I64, _VP, _I64, _I64, _VP, _I64],
        "bfgFacGetLaunchInfo": [_VP, ctypes.c_uint32, _VP, ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_int32)],
        "bfgHelm2KernelMatrix": [_VP, ctypes.POINTER(_Helm2C), _VP, _VP, _I64, _VP, _VP, _I64,
                                 _VP],
        "bfgBessel01": [_VP, _VP, _I64, _VP],
        "bfgMeasureFp64Rate": [_VP, ctypes.POINTER(ctypes.c_double)],
        "bfgFacSetTcWaitLimit": [_VP, ctypes.c_uint64],
        "bfgFacSynchronize": [_VP],
        "bfgPlanHelm2": [ctypes.c_double, _VP, _I64, _VP, _I64, ctypes.POINTER(_FacOptionsC),
                         _VP, _VP, ctypes.c_char_p, _I64, ctypes.POINTER(_I64)],
        "bfgBessel01Host": [_VP, _I64, _VP],
        "bfgPlanCheckApply": [_VP, _I64, _VP, _VP, _VP, _VP, ctypes.POINTER(_FacOptionsC),
                              ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, _VP],
        "bfgFacPrepare": [_VP, ctypes.c_int32],
        "bfgFacAutotune": [_VP, ctypes.c_int32, _I64, _VP, ctypes.c_int32,
                           ctypes.POINTER(ctypes.c_int32)],
        "bfgFacGetRhsTile": [_VP, ctypes.c_int32, _I64, ctypes.POINTER(ctypes.c_int32)],
        "bfgFacGetApplyLaunches": [_VP, ctypes.c_int32, _I64, ctypes.c_uint32, _VP,
                                   ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)],
        "bfgQuadtreeBuild": [_VP, _VP, _VP, _I64, _I64, ctypes.c_int32, _VP, _VP, _I64, _VP],
        "bfgRngSeed": [ctypes.POINTER(_RngC), ctypes.c_uint64],
        "bfgRngUniform1": [ctypes.POINTER(_RngC)],
        "bfgRngUniform": [ctypes.POINTER(_RngC), _I64, _VP],
        "bfgRngComplexRandn": [ctypes.POINTER(_RngC), _I64, _VP],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.bfgGetErrorString.argtypes = [_VP]
    L.bfgGetErrorString.restype = ctypes.c_char_p
    L.bfgFacOptionsDefault.restype = None
    L.bfgRngSeed.restype = None
    L.bfgRngUniform.restype = None
    L.bfgRngComplexRandn.restype = None
    L.bfgRngUniform1.restype = ctypes.c_double
    _lib = L
    return L


def _ptr(a):
    return None if a is None else _VP(a.ctypes.data)


# ---------------------------------------------------------------------------
class Context:
    """One CUDA device and one stream (bfgContextCreate)."""

    def __init__(self, device: int = 0):
        h = _VP()
        st = lib().bfgContextCreate(device, ctypes.byref(h))
        if st != BFG_OK:
            raise BfgError(st, "could not create a context on device %d" % device)
        self.handle = h
        self.device = device
        _live_contexts.add(self)

    def check(self, st: int, what: str = ""):
        if st != BFG_OK:
            msg = lib().bfgGetErrorString(self.handle).decode()
            raise BfgError(st, (what + ": " if what else "") + msg)

    def set_stream(self, cuda_stream_ptr: int | None):
        """Launch on this cudaStream_t (0 = CUDA's legacy default stream)."""
        self.check(lib().bfgContextSetStream(self.handle, _VP(cuda_stream_ptr or 0)))

    def get_stream(self) -> int:
        v = _VP()
        self.check(lib().bfgContextGetStream(self.handle, ctypes.byref(v)))
        return v.value or 0

    def synchronize(self):
        self.check(lib().bfgContextSynchronize(self.handle))

    def on_stream(self, cuda_stream_ptr: int):
        """Context manager: launch on the given stream, then restore."""
        ctx = self

        class _On:
            def __enter__(self_):
                self_.prev = ctx.get_stream()
                ctx.set_stream(cuda_stream_ptr)

            def __exit__(self_, *exc):
                ctx.set_stream(self_.prev)

        return _On()

    def close(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.bfgContextDestroy(self.handle)
        self.handle = None

    def __del__(self):
        self.close()


_default_ctx = {}
_live_contexts = weakref.WeakSet()
_live_facs = weakref.WeakSet()


def _release_all():
    """Destroy every factorization, then every context, before the CUDA
    runtime is torn down at interpreter exit."""
    for f in list(_live_facs):
        f.close()
    for c in list(_live_contexts):
        c.close()
    _default_ctx.clear()


atexit.register(_release_all)


def default_context(device: int = 0) -> Context:
    if device not in _default_ctx:
        _default_ctx[device] = Context(device)
    return _default_ctx[device]


class LayerPot(enum.IntEnum):
    """BfLayerPotential (layer_pot.h:52-65)."""
    Single = 1
    PvDouble = 2
    PvNormalDerivSingle = 3
    CombinedField = 5
    S = 1
    D = 2
    Sp = 3


@dataclass
class Helm2:
    """BfHelm2 (helm2.h:10-15)."""
    k: float
    layer_pot: LayerPot = LayerPot.Single
    alpha: complex = 0j
    beta: complex = 0j

    def _c(self) -> _Helm2C:
        return _Helm2C(float(self.k), int(self.layer_pot), 0, self.alpha.real,
                       self.alpha.imag, self.beta.real, self.beta.imag)


@dataclass
class Quadtree:
    """Points (N, 2) with optional unit normals; the library builds the tree
    with the reference's rule (quadtree.c:80-98) when factorizing."""
    points: np.ndarray
    normals: np.ndarray | None = None
    leaf_size: int = 1


def _xy(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != 2:
        raise ValueError("points/normals must have shape (N, 2)")
    return a


class FacHelm2:
    """bfFacHelm2MakeMultilevel (fac_helm2.c:943-1002) on the GPU."""

    def __init__(self):
        raise TypeError("FacHelm2 can't be instantiated")

    @staticmethod
    def make_multilevel(helm: Helm2, src_tree: Quadtree, tgt_tree: Quadtree | None = None,
                        *, rank_eps: float = 1e-15, pinv_tol: float | None = None,
                        tree_on_gpu: bool = False, jacobi: str = "fp64",
                        sketch: bool = True, context: Context | None = None) -> "Fac":
        tgt_tree = src_tree if tgt_tree is None else tgt_tree
        if src_tree.leaf_size != tgt_tree.leaf_size:
            raise ValueError("both trees must use the same leaf size")
        ctx = context or default_context()
        src, tgt = _xy(src_tree.points), _xy(tgt_tree.points)
        sn, tn = _xy(src_tree.normals), _xy(tgt_tree.normals)
        opts = _FacOptionsC()
        lib().bfgFacOptionsDefault(ctypes.byref(opts))
        opts.leafSize = int(src_tree.leaf_size)
        opts.rankEps = float(rank_eps)
        opts.treeOnGpu = 1 if tree_on_gpu else 0
        opts.jacobiArith = {"fp64": 0, "df64": 1}[jacobi]
        opts.sketch = 1 if sketch else 0
        if pinv_tol is not None:
            opts.pinvCut, opts.pinvTol = 1, float(pinv_tol)
        h = _VP()
        hc = helm._c()
        ctx.check(lib().bfgFacHelm2MakeMultilevel(
            ctx.handle, ctypes.byref(hc), _ptr(src), _ptr(sn), len(src), _ptr(tgt), _ptr(tn),
            len(tgt), ctypes.byref(opts), ctypes.byref(h)), "make_multilevel")
        return Fac(ctx, h, helm)


def make_batched(helm: Helm2, problems, ks, *, leaf_size: int = 1, rank_eps: float = 1e-15,
                 pinv_tol: float | None = None, context: Context | None = None,
                 tree_on_gpu: bool = False, jacobi: str = "fp64", sketch: bool = True) -> "Fac":
    """Factorize many independent problems in one go (bfgFacHelm2MakeBatched).
    ``problems``: list of (src, tgt) or (src, tgt, src_normals, tgt_normals);
    ``ks``: wavenumber per problem.  The result applies diag(A_0, ..., A_P-1);
    ``fac.src_offsets`` / ``fac.tgt_offsets`` locate each problem's rows."""
    ctx = context or default_context()
    srcs = [_xy(p[0]) for p in problems]
    tgts = [_xy(p[1]) for p in problems]
    sn = [_xy(p[2]) if len(p) > 2 and p[2] is not None else None for p in problems]
    tn = [_xy(p[3]) if len(p) > 3 and p[3] is not None else None for p in problems]
    so = np.concatenate([[0], np.cumsum([len(a) for a in srcs])]).astype(np.int64)
    to = np.concatenate([[0], np.cumsum([len(a) for a in tgts])]).astype(np.int64)
    src = np.ascontiguousarray(np.concatenate(srcs))
    tgt = np.ascontiguousarray(np.concatenate(tgts))
    snc = None if any(a is None for a in sn) else np.ascontiguousarray(np.concatenate(sn))
    tnc = None if any(a is None for a in tn) else np.ascontiguousarray(np.concatenate(tn))
    kk = np.ascontiguousarray(ks, dtype=np.float64)
    if len(kk) != len(problems):
        raise ValueError("one wavenumber per problem")
    opts = _FacOptionsC()
    lib().bfgFacOptionsDefault(ctypes.byref(opts))
    opts.leafSize = int(leaf_size)
    opts.rankEps = float(rank_eps)
    opts.treeOnGpu = 1 if tree_on_gpu else 0
    opts.jacobiArith = {"fp64": 0, "df64": 1}[jacobi]
    opts.sketch = 1 if sketch else 0
    if pinv_tol is not None:
        opts.pinvCut, opts.pinvTol = 1, float(pinv_tol)
    h = _VP()
    hc = helm._c()
    ctx.check(lib().bfgFacHelm2MakeBatched(ctx.handle, ctypes.byref(hc), _ptr(kk), len(kk),
                                           _ptr(src), _ptr(snc), _ptr(so), _ptr(tgt), _ptr(tnc),
                                           _ptr(to), ctypes.byref(opts), ctypes.byref(h)),
              "make_batched")
    fac = Fac(ctx, h, helm)
    fac.src_offsets, fac.tgt_offsets = so, to
    return fac


class Fac:
    """A GPU-resident butterfly factorization: the BfMat returned by
    bfFacHelm2MakeMultilevel, with ``@`` = bfMatMul (mat.c:183-185)."""

    def __init__(self, ctx: Context, handle, helm: Helm2):
        self.ctx, self.handle, self.helm = ctx, handle, helm
        _live_facs.add(self)
        r, c = _I64(), _I64()
        ctx.check(lib().bfgFacGetShape(handle, ctypes.byref(r), ctypes.byref(c)))
        self.shape = (r.value, c.value)
        self._perms = None

    def close(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.bfgFacDestroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def autotune(self, precision: str = "bf16x3", rhs: int = 16):
        """bfgFacAutotune: the tensor-core apply's RHS tile width and
        per-stage schedules for `rhs` right-hand sides, picked by timing;
        returns (default ms, tuned ms) per stage."""
        out = np.zeros(64, dtype=np.float64)
        ns = ctypes.c_int32()
        self.ctx.check(lib().bfgFacAutotune(self.handle, PRECISIONS[precision], int(rhs),
                                            _ptr(out), len(out), ctypes.byref(ns)), "autotune")
        return out[:2 * ns.value].reshape(-1, 2)

    def rhs_tile(self, precision: str = "bf16x3", rhs: int = 16) -> int:
        """bfgFacGetRhsTile: the RHS tile width (16 or 32) the tensor-core
        apply of `rhs` right-hand sides uses."""
        t = ctypes.c_int32()
        self.ctx.check(lib().bfgFacGetRhsTile(self.handle, PRECISIONS[precision], int(rhs),
                                              ctypes.byref(t)), "rhs tile")
        return int(t.value)

    def prepare(self, precision: str):
        """Builds the precision's copy of the factors now (bfgFacPrepare)."""
        self.ctx.check(lib().bfgFacPrepare(self.handle, PRECISIONS[precision]), "prepare")

    # -- structure ---------------------------------------------------------
    def perms(self):
        if self._perms is None:
            sp = np.empty(self.shape[1], dtype=np.int64)
            tp = np.empty(self.shape[0], dtype=np.int64)
            self.ctx.check(lib().bfgFacGetPerms(self.handle, _ptr(sp), _ptr(tp)))
            self._perms = (sp, tp)
        return self._perms

    @property
    def src_perm(self):
        return self.perms()[0]

    @property
    def tgt_perm(self):
        return self.perms()[1]

    def num_bytes(self) -> int:
        v = _I64()
        self.ctx.check(lib().bfgFacNumBytes(self.handle, ctypes.byref(v)))
        return v.value

    def stats(self) -> dict:
        s = _FacStatsC()
        self.ctx.check(lib().bfgFacGetStats(self.handle, ctypes.byref(s)))
        out = {name: getattr(s, name) for name, _ in s._fields_}
        out["sketchPhaseMs"] = list(out["sketchPhaseMs"])
        return out

    def describe(self) -> str:
        n = _I64()
        self.ctx.check(lib().bfgFacDescribe(self.handle, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value + 1)
        self.ctx.check(lib().bfgFacDescribe(self.handle, buf, n.value + 1, ctypes.byref(n)))
        return buf.value.decode()

    def blocks(self):
        """(table, entries): table rows (kind, m, n, offset), entries the
        complex128 arena (each block column-major)."""
        st = self.stats()
        ent = np.empty(max(1, st["arenaEntries"]), dtype=np.complex128)
        tab = np.empty((st["numBlocks"], 4), dtype=np.int64)
        self.ctx.check(lib().bfgFacCopyBlocks(self.handle, _ptr(ent), st["arenaEntries"],
                                              _ptr(tab), st["numBlocks"]))
        return tab, ent

    def block_table(self) -> np.ndarray:
        """Rows (kind, m, n, offset) of every stored block in plan order,
        without copying the factors; kinds 0..3 = FIRST, MIDDLE, LAST, DENSE."""
        tab = np.empty((self.stats()["numBlocks"], 4), dtype=np.int64)
        self.ctx.check(lib().bfgFacCopyBlocks(self.handle, None, 0, _ptr(tab), len(tab)))
        return tab

    # -- apply -------------------------------------------------------------
    def save(self, path: str):
        """Writes the factorization (inputs and FP64 factors) to ``path``;
        ``load_fac`` rebuilds it without factorizing again."""
        self.ctx.check(lib().bfgFacSave(self.handle, os.fsencode(path)), "save")

    def apply(self, X, precision: str = "fp64", original_order: bool = False):
        """Y = A X.  numpy complex128 X -> host path (copies inside);
        torch CUDA X -> device path on the context's stream."""
        prec = PRECISIONS[precision]
        flags = APPLY_ORIGINAL_ORDER if original_order else 0
        if isinstance(X, np.ndarray):
            squeeze = X.ndim == 1
            Xh = np.ascontiguousarray(X.reshape(X.shape[0], -1), dtype=np.complex128)
            if Xh.shape[0] != self.shape[1]:
                raise ValueError("X has %d rows, expected %d" % (Xh.shape[0], self.shape[1]))
            R = Xh.shape[1]
            Y = np.empty((self.shape[0], R), dtype=np.complex128)
            self.ctx.check(lib().bfgFacApplyHost(self.handle, prec, _ptr(Xh), R, R, _ptr(Y), R,
                                                 flags), "apply")
            return Y[:, 0] if squeeze else Y
        import torch
        squeeze = X.dim() == 1
        Xd = X.reshape(X.shape[0], -1)
        want = torch.complex128 if precision in _C128_PRECISIONS else torch.complex64
        if Xd.dtype != want or not Xd.is_contiguous():
            Xd = Xd.to(want).contiguous()
        if Xd.shape[0] != self.shape[1]:
            raise ValueError("X has %d rows, expected %d" % (Xd.shape[0], self.shape[1]))
        R = Xd.shape[1]
        Y = torch.empty((self.shape[0], R), dtype=want, device=Xd.device)
        # run on torch's current stream so torch work before and after is ordered
        with self.ctx.on_stream(torch.cuda.current_stream(Xd.device).cuda_stream):
            self.apply_device(Xd.data_ptr(), R, R, Y.data_ptr(), R, precision, original_order)
        return Y[:, 0] if squeeze else Y

    def apply_device(self, x_ptr: int, ldx: int, R: int, y_ptr: int, ldy: int,
                     precision: str = "fp64", original_order: bool = False):
        """Y = A X on raw device pointers (bfgFacApply), on the context's
        stream -- not torch's: order it against torch work with
        ``ctx.on_stream``.  Applies of one factorization share its workspace."""
        flags = APPLY_ORIGINAL_ORDER if original_order else 0
        self.ctx.check(lib().bfgFacApply(self.handle, PRECISIONS[precision], _VP(x_ptr), ldx, R,
                                         _VP(y_ptr), ldy, flags), "apply")

    def apply_timed(self, x_ptr: int, ldx: int, R: int, y_ptr: int, ldy: int,
                    precision: str = "fp64", original_order: bool = False):
        """Per-launch device milliseconds of one apply."""
        flags = APPLY_ORIGINAL_ORDER if original_order else 0
        cap = 256
        ms = np.zeros(cap, dtype=np.float32)
        n = ctypes.c_int32()
        self.ctx.check(lib().bfgFacApplyTimed(self.handle, PRECISIONS[precision], _VP(x_ptr), ldx,
                                              R, _VP(y_ptr), ldy, flags, _ptr(ms), cap,
                                              ctypes.byref(n)), "apply_timed")
        return ms[:n.value].copy()

    def synchronize(self):
        """Waits for the context's stream and raises BfgError(33,
        BFG_ERROR_TIMEOUT) if an asynchronous tensor-core apply gave up on a
        bounded wait (bfgFacSynchronize)."""
        self.ctx.check(lib().bfgFacSynchronize(self.handle), "synchronize")

    def launch_info(self, original_order: bool = False, precision: str = "fp64",
                    rhs: int = 1) -> np.ndarray:
        """(entries, rows_in, rows_out) per launch of one apply in this
        precision with `rhs` right-hand sides (bfgFacGetApplyLaunches)."""
        cap = 256
        info = np.zeros((cap, 3), dtype=np.int64)
        n = ctypes.c_int32()
        self.ctx.check(lib().bfgFacGetApplyLaunches(
            self.handle, PRECISIONS[precision], int(rhs),
            APPLY_ORIGINAL_ORDER if original_order else 0, _ptr(info), cap,
            ctypes.byref(n)), "launch_info")
        return info[:n.value].copy()

    def __matmul__(self, X):
        return self.apply(X)

    def dense_rows(self, rows, X_dev, R: int):
        """Rows (tree order) of K X in FP64 on the GPU; X_dev a torch
        complex128 CUDA tensor (tree order)."""
        import torch
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        out = torch.empty((len(rows), R), dtype=torch.complex128, device=X_dev.device)
        with self.ctx.on_stream(torch.cuda.current_stream(X_dev.device).cuda_stream):
            self.ctx.check(lib().bfgFacDenseRows(self.handle, _ptr(rows), len(rows),
                                                 _VP(X_dev.data_ptr()), R, R,
                                                 _VP(out.data_ptr()), R), "dense_rows")
        return out


def load_fac(path: str, helm: Helm2 | None = None, context: Context | None = None) -> "Fac":
    """A factorization saved by ``Fac.save``, rebuilt on the context's GPU
    (bfgFacLoad).  ``helm`` only labels the Python object."""
    ctx = context or default_context()
    h = _VP()
    ctx.check(lib().bfgFacLoad(ctx.handle, os.fsencode(path), ctypes.byref(h)), "load")
    return Fac(ctx, h, helm)


def kernel_matrix(helm: Helm2, src, tgt, src_normals=None, tgt_normals=None,
                  context: Context | None = None) -> np.ndarray:
    """bfHelm2GetKernelMatrix (helm2.c:282-319) evaluated on the GPU."""
    ctx = context or default_context()
    src, tgt = _xy(src), _xy(tgt)
    sn, tn = _xy(src_normals), _xy(tgt_normals)
    out = np.empty((len(tgt), len(src)), dtype=np.complex128)
    hc = helm._c()
    ctx.check(lib().bfgHelm2KernelMatrix(ctx.handle, ctypes.byref(hc), _ptr(src), _ptr(sn),
                                         len(src), _ptr(tgt), _ptr(tn), len(tgt), _ptr(out)),
              "kernel_matrix")
    return out


def measure_fp64_rate(context: Context | None = None) -> float:
    """The device's measured FP64 FMA rate in TFLOP/s (bfgMeasureFp64Rate)."""
    ctx = context or default_context()
    v = ctypes.c_double()
    ctx.check(lib().bfgMeasureFp64Rate(ctx.handle, ctypes.byref(v)), "measure_fp64_rate")
    return float(v.value)


def bessel01(x, context: Context | None = None) -> np.ndarray:
    """(J0, Y0, J1, Y1) at x > 0 from the device evaluator."""
    ctx = context or default_context()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty((len(x), 4))
    ctx.check(lib().bfgBessel01(ctx.handle, _ptr(x), len(x), _ptr(out)), "bessel01")
    return out


def plan_helm2(k: float, src, tgt, leaf_size: int = 1, rank_eps: float = 1e-15):
    """Host-only: (src_perm, tgt_perm, plan_text) of the factorization the
    library would build -- no GPU involved."""
    src, tgt = _xy(src), _xy(tgt)
    opts = _FacOptionsC()
    lib().bfgFacOptionsDefault(ctypes.byref(opts))
    opts.leafSize, opts.rankEps = int(leaf_size), float(rank_eps)
    sp = np.empty(len(src), dtype=np.int64)
    tp = np.empty(len(tgt), dtype=np.int64)
    n = _I64()
    st = lib().bfgPlanHelm2(float(k), _ptr(src), len(src), _ptr(tgt), len(tgt),
                            ctypes.byref(opts), _ptr(sp), _ptr(tp), None, 0, ctypes.byref(n))
    if st != BFG_OK:
        raise BfgError(st, "plan_helm2 failed")
    buf = ctypes.create_string_buffer(n.value + 1)
    st = lib().bfgPlanHelm2(float(k), _ptr(src), len(src), _ptr(tgt), len(tgt),
                            ctypes.byref(opts), None, None, buf, n.value + 1, ctypes.byref(n))
    if st != BFG_OK:
        raise BfgError(st, "plan_helm2 failed")
    return sp, tp, buf.value.decode()


def check_apply_schedule(problems, leaf_size: int = 1, rank_eps: float = 1e-15, rhs: int = 4,
                         ctas: int = 152, seed: int = 1):
    """Host-only self-check of the apply's work decomposition
    (bfgPlanCheckApply), no GPU involved.  problems: a list of (k, src, tgt)
    planned as one factorization (one problem) or a batched one.  Returns
    (staged-program difference, worst chunk-schedule difference), each the
    relative Frobenius distance from a direct evaluation of the plan's
    structure on seeded block values."""
    ks = np.array([float(p[0]) for p in problems], dtype=np.float64)
    srcs = [_xy(p[1]) for p in problems]
    tgts = [_xy(p[2]) for p in problems]
    so = np.concatenate([[0], np.cumsum([len(a) for a in srcs])]).astype(np.int64)
    to = np.concatenate([[0], np.cumsum([len(a) for a in tgts])]).astype(np.int64)
    src = np.ascontiguousarray(np.concatenate(srcs))
    tgt = np.ascontiguousarray(np.concatenate(tgts))
    opts = _FacOptionsC()
    lib().bfgFacOptionsDefault(ctypes.byref(opts))
    opts.leafSize, opts.rankEps = int(leaf_size), float(rank_eps)
    err = np.zeros(2, dtype=np.float64)
    st = lib().bfgPlanCheckApply(_ptr(ks), len(problems), _ptr(src), _ptr(so), _ptr(tgt),
                                 _ptr(to), ctypes.byref(opts), int(rhs), int(ctas), int(seed),
                                 _ptr(err))
    if st != BFG_OK:
        raise BfgError(st, "check_apply_schedule failed")
    return float(err[0]), float(err[1])


def quadtree_build(point_sets, leaf_size: int = 1, on_gpu: bool = False,
                   context: Context | None = None):
    """bfQuadtreeInit (quadtree.c:80-98) of each (N_t, 2) point set, on the
    GPU in one pass over all sets (on_gpu) or on the host: a list of
    (perm, nodes) per set, perm the tree order (indices into the set), nodes
    a QUADTREE_NODE_DTYPE array numbered as the reference's recursive build
    creates them."""
    sets = [_xy(p) for p in point_sets]
    off = np.zeros(len(sets) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(p) for p in sets])
    xy = np.ascontiguousarray(np.concatenate(sets) if sets else np.zeros((0, 2)))
    ctx = (context or default_context()) if on_gpu else context
    h = ctx.handle if ctx is not None else None
    perm = np.empty(int(off[-1]), dtype=np.int64)
    noff = np.empty(len(sets) + 1, dtype=np.int64)
    L = lib()
    st = L.bfgQuadtreeBuild(h, _ptr(xy), _ptr(off), len(sets), int(leaf_size), int(bool(on_gpu)),
                            _ptr(perm), None, 0, _ptr(noff))
    if st != BFG_OK:
        raise BfgError(st, "quadtree_build: " + (L.bfgGetErrorString(h).decode() if h else "failed"))
    nodes = np.zeros(int(noff[-1]), dtype=QUADTREE_NODE_DTYPE)
    st = L.bfgQuadtreeBuild(h, _ptr(xy), _ptr(off), len(sets), int(leaf_size), int(bool(on_gpu)),
                            _ptr(perm), _ptr(nodes), len(nodes), _ptr(noff))
    if st != BFG_OK:
        raise BfgError(st, "quadtree_build: " + (L.bfgGetErrorString(h).decode() if h else "failed"))
    return [(perm[off[t]:off[t + 1]].copy(), nodes[noff[t]:noff[t + 1]].copy())
            for t in range(len(sets))]


def bessel01_host(x) -> np.ndarray:
    """The device evaluator's source run on the CPU."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty((len(x), 4))
    st = lib().bfgBessel01Host(_ptr(x), len(x), _ptr(out))
    if st != BFG_OK:
        raise BfgError(st, "bessel01_host failed")
    return out


class Rng:
    """The reference's seeded generator (rand.c:19-76), explicit state."""

    def __init__(self, seed: int = 0):
        self._s = _RngC()
        self.seed(seed)

    def seed(self, seed: int):
        lib().bfgRngSeed(ctypes.byref(self._s), ctypes.c_uint64(seed))

    def uniform(self, n: int) -> np.ndarray:
        out = np.empty(n)
        lib().bfgRngUniform(ctypes.byref(self._s), n, _ptr(out))
        return out

    def complex_randn(self, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.complex128)
        lib().bfgRngComplexRandn(ctypes.byref(self._s), n, _ptr(out))
        return out


def uniform_square_points(n: int, seed: int) -> np.ndarray:
    """n points iid uniform in [-1,1]^2 from the seeded generator (x then y)."""
    return (2.0 * Rng(seed).uniform(2 * n) - 1.0).reshape(n, 2)


def curve_points(kind: str, n: int, a: float = 3.0, b: float = 2.0, amp: float = 0.5,
                 lobes: int = 5) -> np.ndarray:
    """Points equispaced in the curve parameter, theta_i = (2 pi / n) i."""
    theta = (6.283185307179586 / n) * np.arange(n, dtype=np.float64)
    if kind == "circle":
        return np.stack([a * np.cos(theta), a * np.sin(theta)], axis=1)
    if kind == "ellipse":
        return np.stack([a * np.cos(theta), b * np.sin(theta)], axis=1)
    if kind == "star":
        r = a + amp * np.cos(lobes * theta)
        return np.stack([r * np.cos(theta), r * np.sin(theta)], axis=1)
    raise ValueError(kind)


# ---------------------------------------------------------------------------
# boundary-integral systems and GMRES
# ---------------------------------------------------------------------------
class _GmresResultC(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("relResidual", ctypes.c_double),
                ("trueRelResidual", ctypes.c_double), ("seconds", ctypes.c_double),
                ("converged", ctypes.c_int32), ("reserved", ctypes.c_int32)]


PRECOND = {"none": 0, "block_jacobi": 1, "user": 2, "learned": 3, "two_level": 4}
_PRECOND_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p)


def _solver_sigs():
    L = lib()
    if getattr(L, "_solver_sigs", False):
        return L
    sig = {
        "bfgSystemCreate": [_VP, _VP, ctypes.POINTER(_Helm2C), _VP, _VP, _VP, _VP, _I64,
                            ctypes.c_int32, ctypes.c_double, ctypes.POINTER(_VP)],
        "bfgSystemDestroy": [_VP],
        "bfgSystemApply": [_VP, _VP, _VP],
        "bfgSystemBuildBlockJacobi": [_VP],
        "bfgSystemApplyBlockJacobi": [_VP, _VP, _VP],
        "bfgSystemSetApplyPrecision": [_VP, ctypes.c_int32],
        "bfgSystemBuildCoarse": [_VP, ctypes.c_int32, ctypes.POINTER(_I64)],
        "bfgSystemCoarseMatrices": [_VP, _VP, _VP],
        "bfgSystemApplyCoarse": [_VP, _VP, _VP],
        "bfgSolveGmres": [_VP, _VP, _VP, ctypes.c_double, _I64, ctypes.c_int32, _PRECOND_FN,
                          _VP, ctypes.POINTER(_GmresResultC)],
    }
    for name, args in sig.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = ctypes.c_int
    L.bfgSystemGetErrorString.argtypes = [_VP]
    L.bfgSystemGetErrorString.restype = ctypes.c_char_p
    L._solver_sigs = True
    return L


class System:
    """A = diag_shift I + (K + C) diag(w) on a factorization K (original point
    order): the operator of the reference's assembleButterfliedK
    (multiple_scattering_context.c:457-507)."""

    def __init__(self, fac: "Fac", points, normals, weights, curve_offsets,
                 kr_order: int = 6, diag_shift: float = 0.5):
        L = _solver_sigs()
        self.fac, self.ctx = fac, fac.ctx
        pts, nrm = _xy(points), _xy(normals)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        off = np.ascontiguousarray(curve_offsets, dtype=np.int64)
        h = _VP()
        hc = fac.helm._c()
        st = L.bfgSystemCreate(self.ctx.handle, fac.handle, ctypes.byref(hc), _ptr(pts), _ptr(nrm),
                               _ptr(w), _ptr(off), len(off) - 1, int(kr_order), float(diag_shift),
                               ctypes.byref(h))
        if st != BFG_OK:
            raise BfgError(st, "bfgSystemCreate failed")
        self.handle = h
        self.n = len(pts)
        _live_facs.add(self)

    def _check(self, st, what):
        if st != BFG_OK:
            msg = _solver_sigs().bfgSystemGetErrorString(self.handle).decode()
            raise BfgError(st, "%s: %s" % (what, msg))

    def close(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.bfgSystemDestroy(self.handle)
        self.handle = None

    def __del__(self):
        self.close()

    def _stream(self, t):
        import torch
        return self.ctx.on_stream(torch.cuda.current_stream(t.device).cuda_stream)

    def apply(self, x):
        import torch
        x = x.to(torch.complex128).contiguous()
        y = torch.empty_like(x)
        with self._stream(x):
            self._check(_solver_sigs().bfgSystemApply(self.handle, _VP(x.data_ptr()),
                                                      _VP(y.data_ptr())), "apply")
        return y

    def set_apply_precision(self, precision: str):
        """Arithmetic of the butterfly part of the system apply (and so of
        the GMRES iterations): "fp64" or "df64" (double-float, ~1e-13 of
        FP64 at FP32 rates).  The solver's final true residual is FP64."""
        import torch
        with self.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
            self._check(_solver_sigs().bfgSystemSetApplyPrecision(self.handle,
                                                                 PRECISIONS[precision]),
                        "apply precision")

    def build_block_jacobi(self):
        import torch
        with self.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
            self._check(_solver_sigs().bfgSystemBuildBlockJacobi(self.handle), "block-Jacobi")

    def apply_block_jacobi(self, r):
        import torch
        r = r.to(torch.complex128).contiguous()
        z = torch.empty_like(r)
        with self._stream(r):
            self._check(_solver_sigs().bfgSystemApplyBlockJacobi(self.handle, _VP(r.data_ptr()),
                                                                 _VP(z.data_ptr())), "precond")
        return z

    def build_coarse(self, extra_modes: int = 5) -> int:
        """The two-level preconditioner's coarse space (bfgSystemBuildCoarse):
        every curve's Fourier modes |m| <= ceil(k L / 2 pi) + extra_modes,
        A_c = Phi^H A Phi and its inverse on the GPU.  Returns the coarse
        dimension.  Use with solve_gmres(..., precond="two_level") after
        build_block_jacobi()."""
        import torch
        d = _I64()
        with self.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
            self._check(_solver_sigs().bfgSystemBuildCoarse(self.handle, int(extra_modes),
                                                            ctypes.byref(d)), "coarse space")
        self.coarse_dim = int(d.value)
        return self.coarse_dim

    def coarse_matrices(self):
        """(A_c, A_c^-1) as device complex64 tensors (dim x dim)."""
        import torch
        D = self.coarse_dim
        ac = torch.empty((D, D), dtype=torch.complex64, device="cuda")
        ai = torch.empty_like(ac)
        with self.ctx.on_stream(torch.cuda.current_stream().cuda_stream):
            self._check(_solver_sigs().bfgSystemCoarseMatrices(self.handle, _VP(ac.data_ptr()),
                                                               _VP(ai.data_ptr())), "coarse")
        return ac, ai

    def apply_coarse(self, r):
        """z = Phi A_c^-1 Phi^H r (device complex128)."""
        import torch
        r = r.to(torch.complex128).contiguous()
        z = torch.empty_like(r)
        with self._stream(r):
            self._check(_solver_sigs().bfgSystemApplyCoarse(self.handle, _VP(r.data_ptr()),
                                                            _VP(z.data_ptr())), "coarse")
        return z


def solve_gmres(system: System, b, x0=None, tol: float = 1e-8, max_num_iter: int = None,
                precond="block_jacobi"):
    """Right-preconditioned flexible GMRES on the GPU (bfSolveGMRES,
    linalg.c:47-317, with the preconditioner on the right).  ``precond``:
    "none", "block_jacobi", "learned", "two_level" (System.build_coarse), or
    a callable (r_ptr, z_ptr, stream_ptr) -> None applying z = M r to device
    complex128 vectors.  Returns (x, info)."""
    import torch
    L = _solver_sigs()
    b = b.to(torch.complex128).contiguous()
    x = torch.zeros_like(b) if x0 is None else x0.to(torch.complex128).contiguous().clone()
    m = system.n if max_num_iter is None else int(max_num_iter)
    fn = _PRECOND_FN()
    mode = PRECOND["user"] if callable(precond) else PRECOND[precond]
    if callable(precond):
        def _cb(user, r, z, stream):
            try:
                precond(r, z, stream)
                return 0
            except Exception:           # reported as a runtime error
                return 2
        fn = _PRECOND_FN(_cb)
    res = _GmresResultC()
    with system.ctx.on_stream(torch.cuda.current_stream(b.device).cuda_stream):
        st = L.bfgSolveGmres(system.handle, _VP(b.data_ptr()), _VP(x.data_ptr()), float(tol), m,
                             mode, fn, None, ctypes.byref(res))
    system._check(st, "gmres")
    info = {name: getattr(res, name) for name, _ in res._fields_ if name != "reserved"}
    return x, info


def scattering_geometry(num: int = 64, k: float = 200.0, ppw: float = 12.0,
                        rmin: float = 0.05, rmax: float = 0.15, box: float = 2.0,
                        gap: float = 0.05, seed: int = 0, max_tries: int = 1000000):
    """Circular scatterers placed by seeded rejection sampling in
    [-box, box]^2 with gaps >= gap, radii uniform in [rmin, rmax]; each
    discretised like bfEllipseSampleLinspaced (ellipse.c) with
    n = floor(perimeter / h) + 1 points (multiple_scattering_context.c:
    351-353), h = 2 pi / (ppw k).  Returns (points, normals, weights,
    offsets, circles)."""
    rng = Rng(seed)
    circles = []
    tries = 0
    while len(circles) < num:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d scatterers" % num)
        r = rmin + (rmax - rmin) * rng.uniform(1)[0]
        u = rng.uniform(2)
        cx = -box + r + (2 * (box - r)) * u[0]
        cy = -box + r + (2 * (box - r)) * u[1]
        if all(np.hypot(cx - c[0], cy - c[1]) >= r + c[2] + gap for c in circles):
            circles.append((cx, cy, r))
    h = 2 * np.pi / (ppw * k)
    pts, nrm, wts, off = [], [], [], [0]
    for cx, cy, r in circles:
        n = int(np.floor(2 * np.pi * r / h)) + 1
        dt = 6.283185307179586 / n
        th = dt * np.arange(n)
        c, s = np.cos(th), np.sin(th)
        pts.append(np.stack([cx + r * c, cy + r * s], 1))
        nrm.append(np.stack([c, s], 1))
        wts.append(np.full(n, dt * r))
        off.append(off[-1] + n)
    return (np.concatenate(pts), np.concatenate(nrm), np.concatenate(wts),
            np.array(off, dtype=np.int64), np.array(circles))


from . import learned  # noqa: E402,F401  (learned preconditioner)
