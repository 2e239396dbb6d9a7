"""The randomized re-expansion (the library's path for FIRST/MIDDLE blocks
whose rank estimate far exceeds the numerical rank of Z_equiv), restated
with numpy's LAPACK, against the reference's pseudo-inverse least squares
(helm2.c:321-365, mat_dense_complex.c:1768-1849) restated by the oracle with
scipy's zgesvd, on real blocks of a workload where the path is taken.

Bars: the same least-squares residual (within 1.5x + 1e-13), solutions
within 1e-8 (cut 1e-7) of each other, and the capture ratio (smallest over
largest sketched singular value) under the library's threshold."""
import numpy as np

from oracle import bf_oracle as O


def _blocks(N, k, curve, eps, leaf=64):
    src = O.uniform_square_points(N, 0)
    tgt = O.curve_points(curve, N)
    ts, tt = O.Quadtree(src, leaf), O.Quadtree(tgt, leaf)
    root = O.Planner(k, ts, tt, eps=eps).plan()
    src_tree_pts = ts.points[np.asarray(ts.perm, dtype=np.int64)]
    out = []
    for b in O.iter_blocks(root):
        if b.kind not in ("first", "middle") or b.m < 256:
            continue
        w = O.sketch_width(k, b.ceq, b.cchk, b.m)
        if w <= 0.5 * b.m:
            out.append((b, w))
    return out, src_tree_pts


def test_sketched_pseudo_inverse_matches_the_reference_rule():
    k, tol = 256.0, 1e-7
    blocks, src_pts = _blocks(8192, k, "star", tol)
    assert len(blocks) >= 8
    h = O.Helm2(k)
    for b, w in blocks[:4]:
        eq, _ = O.circle_points(b.ceq, b.m)
        chk, _ = O.circle_points(b.cchk, b.m)
        if b.kind == "first":
            orig = src_pts[b.src_range[0]:b.src_range[1]]
        else:
            orig, _ = O.circle_points(b.corig, b.n)
        Ze = O.kernel_matrix(h, eq, chk)
        Zo = O.kernel_matrix(h, orig, chk)
        Xf = O.lstsq_pinv(Ze, Zo, "relative", tol)
        Xs, ratio = O.sketch_pinv(Ze, Zo, w, tol)
        rf = np.linalg.norm(Ze @ Xf - Zo) / np.linalg.norm(Zo)
        rs = np.linalg.norm(Ze @ Xs - Zo) / np.linalg.norm(Zo)
        assert w < b.m / 2
        assert ratio < 1e-10                      # the library's capture bar at cut 1e-7
        assert rs <= 1.5 * rf + 1e-13
        assert np.linalg.norm(Xs - Xf) / np.linalg.norm(Xf) < 1e-8


def test_too_narrow_sketch_fails_the_capture_test():
    """A sketch narrower than the numerical rank keeps singular values far
    above the rounding floor: the library then sketches again, wider."""
    k, tol = 256.0, 1e-7
    blocks, _ = _blocks(8192, k, "star", tol)
    b, w = blocks[0]
    eq, _ = O.circle_points(b.ceq, b.m)
    chk, _ = O.circle_points(b.cchk, b.m)
    Ze = O.kernel_matrix(O.Helm2(k), eq, chk)
    _, ratio = O.sketch_pinv(Ze, Ze[:, :8], 32, tol)
    assert ratio > 1e-10
