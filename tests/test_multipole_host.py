"""Host-side parts of the multipole / ellipsoid force (no GPU): the
committed reference values pinned against the live reference build where its
sources are present, and the depolarisation factors (src/force.c:236-258, a
64-point Gauss-Legendre rule over [0, 100 a_k^2]) against the same rule in
numpy."""
import numpy as np
import pytest

from conftest import golden
from depsolver_gb300 import api, scenes


def test_fixture_matches_live_reference(ref):
    g = golden("multipole.npz")
    for nen in (6, 3):
        sc = scenes.small(nen=nen)
        x = g[f"x_{nen}"]
        for k, p in enumerate(g["points"]):
            for o in (1, 3, 5):
                assert np.array_equal(ref.force_multipole(sc, x, o, 1.0, p), g[f"multipole_{nen}"][k, o - 1])
            for a, an in enumerate((10, 11)):
                assert np.array_equal(ref.force_ellipsoid(sc, x, an, g["axis"], p), g[f"ellipsoid_{nen}"][k, a])


def _depol_numpy(axis):
    t, w = np.polynomial.legendre.leggauss(64)
    a2 = np.asarray(axis, dtype=np.float64) ** 2
    L = np.zeros(3)
    for k in range(3):
        X1 = 100 * a2[k]
        x = 0.5 * (1 + t) * X1
        f = 1.0 / ((x + a2[k]) * np.sqrt((x + a2[0]) * (x + a2[1]) * (x + a2[2])))
        L[k] = 0.5 * np.prod(axis) * 0.5 * X1 * np.dot(w, f)
    return L


@pytest.mark.parametrize("axis", [(1.0, 1.0, 1.0), (1.0, 0.9, 0.8), (2.0, 1.0, 0.5), (1e-6, 2e-6, 3e-6)])
def test_depolarization_factors(native, axis):
    L = api.depolarization(axis)
    assert np.allclose(L, _depol_numpy(axis), rtol=1e-12, atol=0)
    assert abs(L.sum() - 1.0) < 0.1


def test_depolarization_sphere_is_symmetric(native):
    L = api.depolarization([1.0, 1.0, 1.0])
    assert L[0] == L[1] == L[2]
