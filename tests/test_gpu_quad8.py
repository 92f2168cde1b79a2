"""The quad8 extension on the GPU, against the oracle's quad8 restatement
(oracle/port/quad8.c; the reference has no quad8 integrals) and against
closed-form fields: assembly of both forms, the solve, field and potential
off and on the mesh, the Maxwell-stress force; a conducting sphere and a
dielectric sphere in a near-uniform field."""
import numpy as np
import pytest

from conftest import relerr
from depsolver_gb300 import _native, api, scenes

pytestmark = pytest.mark.gpu

ASM_TOL = 1e-12   # relative to the largest entry
SOL_TOL = 1e-10


@pytest.mark.parametrize("full", [False, True])
def test_quad8_assembly_matches_oracle(gpu, port, full):
    sc = scenes.small(nen=8)
    A, B = api.electric_form(sc, full=full)
    Ap, Bp = port.assemble(sc, full=full)
    assert relerr(A, Ap) < ASM_TOL and np.array_equal(B, Bp)


def test_quad8_pipeline_matches_oracle(gpu, port):
    sc = scenes.small(nen=8)
    A, B = api.electric_form(sc)
    x, _ = api.solver_gmres_el(A, B, tol=1e-12)
    Ap, Bp = port.assemble(sc)
    xp, _, _ = port.gmres(Ap, Bp, tol=1e-12)
    assert relerr(x, xp) < SOL_TOL
    p0 = sc.particles[0][0]
    pts = np.vstack([sc.nodes[p0:p0 + 30], sc.nodes[:3], np.random.default_rng(8).uniform(-2, 2, (20, 3))])
    assert relerr(api.field(sc, xp, pts), port.field(sc, xp, pts)) < SOL_TOL
    assert relerr(api.potential(sc, xp, pts), port.potential(sc, xp, pts)) < SOL_TOL
    Fce, Xce, Fcm, Xcm = api.force_mst(sc, xp)
    Fp, Xp, Fcp, Xcp = port.force_mst(sc, xp)
    pel = sc.bctype[sc.elems[:, 0] - 1] == 6
    assert relerr(Fce[pel], Fp[pel]) < SOL_TOL and relerr(Xce[pel], Xp[pel]) < 1e-14
    assert np.abs(Fcm - Fcp).max() <= SOL_TOL * np.abs(Fp[pel]).sum()
    assert np.allclose(Xcm, Xcp, rtol=0, atol=1e-14)


def test_quad8_conducting_sphere(gpu):
    sc = scenes.conductor_sphere(8)
    A, B = api.electric_form(sc, full=True)
    x = api.gauss_bksb(A, B)
    pts = np.array([[2.0, 0.0, 0.0], [0.0, 3.0, 0.0], [1.5, 1.5, 1.5], [0.0, 0.0, -4.0]])
    r = np.linalg.norm(pts, axis=1)
    assert np.abs(api.potential(sc, x, pts)[:, 0] * r - 1.0).max() < 2e-3
    E = api.field(sc, x, sc.nodes[::7])[:, 0::2]
    assert np.abs(np.einsum("ij,ij->i", E, sc.nodes[::7]) - 1.0).max() < 0.05   # V / R on the surface


def test_quad8_dielectric_sphere_dipole(gpu):
    ep, em = 10.0, 1.0
    sc = scenes.sphere_between_plates(3, 4, nen=8, plate_side=40.0, plate_z=8.0, medium=(0.0, em),
                                      particle=(0.0, ep), freq=1e6)
    A, B = api.electric_form(sc)
    x, _ = api.solver_gmres_el(A, B, tol=1e-10)
    pts = np.array([[0.0, 0.0, 1.6], [0.0, 0.0, -1.6], [0.0, 0.0, 2.0]])
    r = np.linalg.norm(pts, axis=1)
    phi = api.potential(sc, x, pts)[:, 0]
    (E0, p), *_ = np.linalg.lstsq(np.stack([-pts[:, 2], pts[:, 2] / r ** 3], 1), phi, rcond=None)
    K = (ep - em) / (ep + 2 * em)
    assert abs(p / E0 - K) < 0.02 * K


def test_quad8_is_not_a_session_family(gpu):
    sc = scenes.small(nen=8)
    with pytest.raises(_native.DscError):
        api.Session(sc)
