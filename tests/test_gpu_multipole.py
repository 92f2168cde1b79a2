"""Multipole and ellipsoid DEP forces (forceMultipole_*, forceEllipsoid_*,
src/force.c:65-322,572-825) against the reference's own values
(tests/golden/multipole.npz, made by tests/golden/make_golden.py from the
reference build): both small scenes, three points, orders 1-5 and the
ellipsoid analyses 10 and 11, through the flat API and the drop-in
signatures (including the reference's in-place rescaling of the particle's
material for analysis 11)."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from depsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu

TOL = 1e-10   # relative to the largest component of the reference's force


def _rel(a, b):
    return float(np.abs(np.asarray(a) - b).max() / np.abs(b).max())


@pytest.mark.parametrize("nen", [6, 3])
def test_multipole_and_ellipsoid_match_reference(gpu, nen):
    g = golden("multipole.npz")
    sc = scenes.small(nen=nen)
    x = g[f"x_{nen}"]
    pts = g["points"]
    for o in range(1, 6):
        F = api.force_multipole(sc, x, pts, o, float(g["R"]))
        for k in range(len(pts)):
            assert _rel(F[k], g[f"multipole_{nen}"][k, o - 1]) < TOL, (o, k)
    for a, an in enumerate((10, 11)):
        F = api.force_ellipsoid(sc, x, pts, an, g["axis"])
        for k in range(len(pts)):
            assert _rel(F[k], g[f"ellipsoid_{nen}"][k, a]) < TOL, (an, k)


def test_dropin_signatures(gpu):
    g = golden("multipole.npz")
    sc = scenes.small(nen=6)
    L = gpu
    C.c_uint.in_dll(L, "nNodes").value = sc.N
    C.c_uint.in_dll(L, "nElems").value = sc.E
    nodes = np.ascontiguousarray(sc.nodes)
    elems = np.ascontiguousarray(sc.elems, dtype=np.uint32)
    x = np.ascontiguousarray(g["x_6"])
    mat = np.ascontiguousarray(sc.mat[:2]).copy()
    prob = np.array([sc.freq])
    F = np.zeros(3)
    p = np.ascontiguousarray(g["points"][1])
    L.forceMultipole_tria6(C.c_uint(3), C.c_double(1.0), p.ctypes.data_as(C.c_void_p), api.row_pointers(nodes),
                           api.row_pointers(elems), x.ctypes.data_as(C.c_void_p), api.row_pointers(mat),
                           prob.ctypes.data_as(C.c_void_p), F.ctypes.data_as(C.c_void_p))
    assert _rel(F, g["multipole_6"][1, 2]) < TOL
    axis = np.ascontiguousarray(g["axis"]).copy()
    L.forceEllipsoid_tria6(C.c_uint(11), C.c_uint(1), axis.ctypes.data_as(C.c_void_p),
                           p.ctypes.data_as(C.c_void_p), api.row_pointers(nodes), api.row_pointers(elems),
                           x.ctypes.data_as(C.c_void_p), api.row_pointers(mat), prob.ctypes.data_as(C.c_void_p),
                           F.ctypes.data_as(C.c_void_p))
    assert _rel(F, g["ellipsoid_6"][1, 1]) < TOL
    # the reference's analysis 11 leaves the particle's material scaled by a c / (2 c + a)
    cs = axis[0] * axis[2] / (2 * axis[2] + axis[0])
    assert np.allclose(mat[1], sc.mat[1] * cs, rtol=1e-15)
