"""The quad8 extension without a GPU.  The reference has no quad8 integrals,
so the oracle's quad8 restatement (oracle/port/quad8.c) is pinned here to
fields known in closed form instead of reference outputs: a sphere held at
1 V alone (potential R / r outside, normal field V / R on the surface) and
a dielectric sphere in a near-uniform field (induced dipole with the
Clausius-Mossotti factor).  Also the deck reader and the node normals for
quad8 meshes."""
import numpy as np
import pytest

from depsolver_gb300 import api, scenes


def test_cubed_sphere_mesh():
    n, e = scenes.cubed_sphere(2)
    assert n.shape == (74, 3) and e.shape == (24, 8)
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-15)
    assert np.array_equal(np.unique(e), np.arange(74))          # every node used
    c0, c1, c2, c3 = (n[e[:, k]] for k in range(4))
    out = np.einsum("ij,ij->i", np.cross(c2 - c0, c3 - c1), c0 + c1 + c2 + c3)
    assert (out > 0).all()                                       # normals outward


def test_oracle_conducting_sphere(port):
    sc = scenes.conductor_sphere(4)
    A, B = port.assemble(sc, full=True)
    x = port.gauss(A, B)
    pts = np.array([[2.0, 0.0, 0.0], [0.0, 3.0, 0.0], [1.5, 1.5, 1.5]])
    r = np.linalg.norm(pts, axis=1)
    phi = port.potential(sc, x, pts)[:, 0]
    assert np.abs(phi * r - 1.0).max() < 3e-3
    E = port.field(sc, x, pts)[:, 0::2]
    assert np.abs(E - pts / r[:, None] ** 3).max() < 1e-3
    # on the surface: the principal value plus the jump, once
    En = np.einsum("ij,ij->i", port.field(sc, x, sc.nodes[:40])[:, 0::2], sc.nodes[:40])
    assert np.abs(En - 1.0).max() < 0.12


def test_oracle_dielectric_sphere_dipole(port):
    ep, em = 10.0, 1.0
    sc = scenes.sphere_between_plates(2, 4, nen=8, plate_side=40.0, plate_z=8.0, medium=(0.0, em),
                                      particle=(0.0, ep), freq=1e6)
    A, B = port.assemble(sc, full=True)
    x = port.gauss(A, B)
    pts = np.array([[0.0, 0.0, 1.6], [0.0, 0.0, -1.6], [0.0, 0.0, 2.0]])
    r = np.linalg.norm(pts, axis=1)
    phi = port.potential(sc, x, pts)[:, 0]
    (E0, p), *_ = np.linalg.lstsq(np.stack([-pts[:, 2], pts[:, 2] / r ** 3], 1), phi, rcond=None)
    K = (ep - em) / (ep + 2 * em)
    assert abs(p / E0 - K) < 0.06 * K


@pytest.mark.parametrize("nen", [8])
def test_reader_round_trip_quad8(native, tmp_path, nen):
    sc = scenes.small(nen=nen)
    scenes.write_bem(sc, str(tmp_path))
    d = api.read_bem(str(tmp_path))
    assert d["nen"] == 8
    assert np.array_equal(d["elems"], sc.elems) and np.array_equal(d["nodes"], sc.nodes)


def test_node_normals_quad8(native, port):
    sc = scenes.small(nen=8)
    n = api.node_normals(sc)
    for i in (0, 5, sc.particles[0][0], sc.particles[0][0] + 7, sc.N - 1):
        assert np.allclose(n[i], port.node_normal(sc, i), atol=1e-14)
    p0, p1 = sc.particles[0][:2]
    c = sc.nodes[p0:p1].mean(axis=0)
    assert (np.einsum("ij,ij->i", n[p0:p1], sc.nodes[p0:p1] - c) > 0).all()
