"""The oracle's combined-field system with the Kapur-Rokhlin correction
(cfie_system_dense: kernel fills, quadrature.c KR weights, 1/2 I) against
the point-source known answer: solved densely, its exterior field converges
to the exact one at the KR rule's order (6)."""
import numpy as np

import known_answer as KA
from oracle import bf_oracle as O


def _dense_error(ppw):
    pts, nrm, w, off, srcs, tgt = KA.geometry(ppw)
    A = O.cfie_system_dense(KA.cfie_helm_oracle(), pts, nrm, w, off, 6, 0.5)
    sigma = np.linalg.solve(A, KA.exact_field(srcs, pts))
    return KA.field_error(pts, nrm, w, sigma, srcs, tgt)


def test_point_sources_inside_scatterers():
    e12, e24 = _dense_error(12), _dense_error(24)
    # measured 9.3e-3 and 1.13e-4: a factor 2^6.4 per halving of h
    assert e12 < 2e-2 and e24 < 3e-4
    assert e12 / e24 > 30
