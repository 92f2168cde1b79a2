"""Particle-position sweeps with uneven mesh sizes (dsc_positions_*).

Each position of a sweep is the scene the reference's depSolver-sft run
would solve (nodes pNodes.. shifted by the REPOSITION vector,
src/depSolver-shift.c:212-217): the fixed electrodes' nodes, then the
particle's.  Its forces and nodal solution must be those of a separate
dsc_sweep of that scene (within the tolerance of two independent solves to
tol 1e-11: the conductor-block inverses are shared across positions) and,
at one position, those of the C restatement of the reference's GMRES.
"""
import numpy as np
import pytest

from conftest import relerr
from depsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu

FIXED = dict(plate_side=8.0, plate_z=3.0)


def _position_scene(level, centre, cells=4):
    return scenes.sphere_between_plates(level, cells, center=tuple(centre), **FIXED)


def test_positions_match_separate_sweeps(gpu, port):
    fixed = scenes.plates_only(4, **FIXED)
    ps = api.PositionSweep(fixed)
    levels = [1, 2]
    for lev in levels:
        n, e = scenes.icosphere(lev, 1.0)
        ps.add_particle(n, e, iface=1)
    tm = [1, 0, 1, 0]
    cen = np.array([[0.0, 0.0, 0.4], [0.5, -0.3, -0.2], [-0.4, 0.2, 0.3], [0.3, 0.6, -0.5]])
    freqs = np.logspace(3, 8, 6)
    ps.set_workers(2)
    r = ps.solve(tm, cen, freqs, tol=1e-11, want_sigma=True)
    assert (r["status"] == api.SYS_CONVERGED).all()
    assert 1 <= ps.inversions() <= 2
    for q in range(len(tm)):
        sc = _position_scene(levels[tm[q]], cen[q])
        assert r["sigma"][q].shape == (len(freqs), 2 * sc.N)
        f, _, sig = api.sweep(sc, freqs, mode=api.MODE_MIXED, tol=1e-11)
        for k in range(len(freqs)):
            scale = f[k, 6:9].sum()
            assert np.abs(r["forces"][q, k, :3] - f[k, :3]).max() <= 1e-8 * scale, (q, k)
            assert relerr(r["sigma"][q][k], sig[k]) < 1e-8, (q, k)
        assert np.allclose(r["forces"][q, :, 3:6], f[:, 3:6], rtol=0, atol=1e-13)
        L = api._native.lib()
        st = np.zeros(len(freqs), dtype=np.int32)
        xo = L.dsc_force_crossover(len(freqs), freqs, np.ascontiguousarray(r["forces"][q]), st.ctypes.data)
        assert (np.isnan(xo) and np.isnan(r["crossover_hz"][q])) or xo == r["crossover_hz"][q]
    # one position against the oracle's GMRES (FP64, tol 1e-12) at one frequency
    sc = _position_scene(levels[tm[0]], cen[0]).with_freq(freqs[3])
    A, B = port.assemble(sc)
    xp, _, stp = port.gmres(A, B, tol=1e-12)
    assert stp == 0 and relerr(r["sigma"][0][3], xp) < 1e-5
    Fce, _, Fcm, _ = port.force_mst(sc, xp)
    pel = sc.bctype[sc.elems[:, 0] - 1] == 6
    assert np.abs(r["forces"][0, 3, :3] - Fcm).max() <= 1e-6 * np.abs(Fce[pel]).sum()


def test_positions_one_worker_equals_many(gpu):
    fixed = scenes.plates_only(4, **FIXED)
    ps = api.PositionSweep(fixed)
    for lev in (1, 2):
        ps.add_particle(*scenes.icosphere(lev, 1.0))
    tm = [0, 1, 1, 0, 1]
    cen = np.array([[0.2, 0.1, 0.3 * q - 0.6] for q in range(5)])
    freqs = np.logspace(3, 8, 5)
    ps.set_workers(1)
    a = ps.solve(tm, cen, freqs, tol=1e-10)
    ps.set_workers(4)
    b = ps.solve(tm, cen, freqs, tol=1e-10)
    assert (a["status"] == 0).all() and (b["status"] == 0).all()
    for q in range(5):
        scale = a["forces"][q, :, 6:9].sum(axis=1)
        assert (np.abs(a["forces"][q, :, :3] - b["forces"][q, :, :3]).max(axis=1) <= 1e-8 * scale).all()


def test_positions_report_capped_systems(gpu):
    fixed = scenes.plates_only(4, **FIXED)
    ps = api.PositionSweep(fixed)
    ps.add_particle(*scenes.icosphere(1, 1.0))
    r = ps.solve([0, 0], [[0, 0, 0.3], [0, 0, -0.3]], [1e4, 1e6], tol=1e-11, max_iters=1, partial=True)
    assert (r["status"] == api.SYS_CAPPED).all() and np.isnan(r["forces"]).all()
    assert np.isnan(r["crossover_hz"]).all()
