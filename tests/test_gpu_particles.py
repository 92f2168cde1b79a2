"""Per-particle Maxwell-stress force and torque on a multi-material trap.

The reference sums every type-6 element into one force (src/force.c:516-547);
a particle's own force is that sum over its elements alone, which is what
the reference's forceMST_* returns with vBCType masked to that particle (the
field at its nodes comes from the same solution).  The oracle does exactly
that; the torque (an extension: the reference has none) is checked against
sum (Xce - Xcm) x Fce of the oracle's own per-element output.
"""
import dataclasses

import numpy as np
import pytest

from conftest import relerr
from depsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _masked(sc, k):
    n0, n1, _, _ = sc.particles[k]
    bct = sc.bctype.copy()
    N = sc.N
    for h in (0, N):
        seg = bct[h:h + N]
        other = (seg == 6)
        other[n0:n1] = False
        seg[other] = 0
    return dataclasses.replace(sc, bctype=bct)


@pytest.mark.parametrize("nen", [6, 3])
def test_per_particle_force_and_torque_match_masked_reference(gpu, port, nen):
    sc = scenes.quadrupole_trap(nen=nen, levels=(1, 1, 2, 2), pad_cells=6)
    assert len(sc.particles) == 4 and sc.n_if == 4
    s = api.Session(sc)
    f, _, sig = s.solve([sc.freq], mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    parts = s.particles()[0]
    assert parts.shape == (4, 12)
    A, B = port.assemble(sc)
    xp, _, st = port.gmres(A, B, tol=1e-12)
    assert st == 0
    for k, (n0, n1, e0, e1) in enumerate(sc.particles):
        Fce, Xce, Fcm, Xcm = port.force_mst(_masked(sc, k), xp)
        scale = np.abs(Fce[e0:e1]).sum()
        assert np.abs(parts[k, :3] - Fcm).max() <= 1e-9 * scale, k
        assert np.abs(parts[k, 3:6] - Xcm).max() <= 1e-12, k
        assert np.allclose(parts[k, 6:9], np.abs(Fce[e0:e1]).sum(0), rtol=1e-8), k
        T = np.cross(Xce[e0:e1] - Xcm, Fce[e0:e1]).sum(0)
        rad = np.abs(Xce[e0:e1] - Xcm).max()
        assert np.abs(parts[k, 9:12] - T).max() <= 1e-9 * scale * rad, k
    # the particles' forces add up to the reference's total
    assert np.abs(parts[:, :3].sum(0) - f[0, :3]).max() <= 1e-12 * parts[:, 6:9].sum()
    # The pads' boundary values are complex (phases 90 and 270 deg), where
    # the reference's Jacobi step leaves the imaginary right-hand side
    # unscaled (src/gmres_el.c:87-93): its solution is not that of the
    # assembled system.  The FP64 path with the full scaling is, as the
    # oracle's GMRES without Jacobi scaling confirms; the mixed sweep's
    # per-particle results follow that one.
    s.set_fp64_jacobi(True)
    f2, _, sig2 = s.solve([sc.freq], mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    p2 = s.particles()[0]
    x0, _, st0 = port.gmres(A, B, tol=1e-12, precond=0)
    assert st0 == 0 and relerr(sig2[0], x0) < 1e-9
    assert relerr(sig[0], sig2[0]) > 1e-3   # the two scalings really differ here
    s.solve([sc.freq, 2 * sc.freq], mode=api.MODE_MIXED, tol=1e-10)
    pm = s.particles()
    assert pm.shape == (2, 4, 12)
    for k in range(4):
        sc_k = p2[k, 6:9].sum()
        assert np.abs(pm[0, k, :3] - p2[k, :3]).max() <= 1e-6 * sc_k, k
        rad = np.abs(pm[0, k, 3:6] - p2[k, 3:6]).max() + 1.3
        assert np.abs(pm[0, k, 9:12] - p2[k, 9:12]).max() <= 1e-6 * sc_k * rad, k
