"""The point-source known answer for the multiple-scattering solve (the
construction of the reference's examples/simple/helm2_bie.c:60-210): point
sources placed inside scatterers radiate a field that solves the exterior
Helmholtz problem, so with that field as the boundary data the
combined-field density, evaluated outside the scatterers, must reproduce it
to the discretization's accuracy.  Shared by the oracle's CPU test and the
GPU solver's test."""
import numpy as np

import butterfly_gb300 as B
from oracle import bf_oracle as O

K = 40.0


def geometry(ppw):
    """8 circles (the solver tests' layout), sources inside circles 0 and 3,
    exterior targets on a ring around the layout."""
    pts, nrm, w, off, circles = B.scattering_geometry(num=8, k=K, ppw=ppw, rmin=0.2, rmax=0.4,
                                                      box=2.0, gap=0.1, seed=3)
    c0, c3 = circles[0], circles[3]
    srcs = np.array([[c0[0] + 0.3 * c0[2], c0[1] - 0.2 * c0[2]],
                     [c3[0] - 0.1 * c3[2], c3[1] + 0.4 * c3[2]]])
    th = np.linspace(0.0, 2.0 * np.pi, 200, endpoint=False)
    tgt = np.stack([3.5 * np.cos(th), 3.5 * np.sin(th)], 1)
    return pts, nrm, w, off, srcs, tgt


AMPLITUDES = np.array([1.0, 0.5 - 0.7j])


def exact_field(srcs, x):
    single = O.Helm2(K)
    return sum(a * O.kernel_matrix(single, srcs[i:i + 1], x)[:, 0]
               for i, a in enumerate(AMPLITUDES))


def cfie_helm_oracle():
    return O.Helm2(K, O.LP_COMBINED_FIELD, -1j * K, 1.0)


def field_error(pts, nrm, w, sigma, srcs, tgt):
    """Relative l2 error, on the targets, of the combined-field potential
    of density sigma (trapezoid weights w) against the exact field."""
    u = O.kernel_matrix(cfie_helm_oracle(), pts, tgt, nrm, None) @ (np.asarray(w) * sigma)
    ue = exact_field(srcs, tgt)
    return float(np.linalg.norm(u - ue) / np.linalg.norm(ue))
