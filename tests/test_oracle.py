"""Pins the CPU oracle (oracle/port, a C restatement of the reference) to
the reference: committed golden fixtures made by the reference itself, the
reference's 2008 example outputs, and -- where the reference sources exist --
the reference compiled here, bit for bit."""
import os

import numpy as np
import pytest

from conftest import REFERENCE, golden, relerr
from depsolver_gb300 import scenes

TOL = 1e-12  # port vs reference: bit-exact here, FMA contraction may differ on Arm


def _probe_check(A, g, prefix):
    rng = np.random.default_rng(12345)
    r = rng.standard_normal(A.shape[1])
    s = rng.standard_normal(A.shape[0])
    assert relerr(A @ r, g[prefix + "Ar"]) < TOL
    assert relerr(A.T @ s, g[prefix + "ATs"]) < TOL
    assert relerr(A[g[prefix + "rows_idx"]], g[prefix + "rows"]) < TOL


@pytest.mark.parametrize("nen", [6, 3])
def test_port_matches_golden_small(port, nen, tmp_path):
    g = golden(f"small_tria{nen}.npz")
    sc = scenes.small(nen=nen)
    assert (sc.N, sc.E) == (int(g["N"]), int(g["E"]))
    A, B = port.assemble(sc)
    _probe_check(A, g, "compact_")
    assert np.array_equal(B, g["B"])
    log = str(tmp_path / "gmres.log")
    x, it, st = port.gmres(A, B, log_path=log)
    assert st == 0
    assert relerr(x, g["x_gmres"]) < 1e-12
    assert open(log).read() == bytes(g["gmres_log"]).decode()
    xt, _, st = port.gmres(A, B, tol=1e-10)
    assert st == 0 and relerr(xt, g["x_gmres_tight"]) < 1e-12
    Af, Bf = port.assemble(sc, full=True)
    _probe_check(Af, g, "full_")
    assert relerr(port.gauss(Af, Bf), g["x_gauss"]) < 1e-12
    assert relerr(port.field(sc, x, g["pts"]), g["field"]) < TOL
    assert relerr(port.potential(sc, x, g["pts"]), g["potential"]) < TOL
    Fce, Xce, Fcm, Xcm = port.force_mst(sc, x)
    pel = g["pel"]
    assert relerr(Fce[pel], g["Fce"]) < TOL
    assert relerr(Xce[pel], g["Xce"]) < TOL
    assert np.abs(Fcm - g["Fcm"]).max() <= TOL * np.abs(g["Fce"]).sum()
    assert relerr(Xcm, g["Xcm"]) < TOL


def test_port_matches_golden_dep_trap_2(port, tmp_path):
    """The reference's own example deck (tria3, REPOSITION, MST force)."""
    g = golden("dep_trap_2.npz")
    sc = scenes.Scene(int(g["nen"]), g["nodes"], g["elems"], g["bctype"], g["mbc"], g["ifaces"],
                      g["mat"], float(g["freq"])).contiguous()
    A, B = port.assemble(sc, nthreads=4)
    _probe_check(A, g, "compact_")
    log = str(tmp_path / "gmres.log")
    x, it, st = port.gmres(A, B, log_path=log)
    assert st == 0 and it == 37
    assert relerr(x, g["x_gmres"]) < 1e-12
    text = open(log).read()
    assert text == bytes(g["gmres_log"]).decode()
    assert text == bytes(g["golden_gmres_log"]).decode()  # the file shipped in 2008
    Fce, Xce, Fcm, Xcm = port.force_mst(sc, x, nthreads=4)
    assert relerr(Fce[g["pel"]], g["Fce"]) < TOL
    # the 2008 force-mst.dat, printed to 7 significant digits
    lines = bytes(g["golden_force_mst"]).decode().splitlines()
    tot = np.array([float(v) for v in lines[1].split()])
    assert np.allclose(np.r_[Xcm, Fcm], tot, rtol=1e-6, atol=0)
    rows = np.array([[float(v) for v in l.split()] for l in lines[3:] if l.strip()])
    assert np.allclose(np.hstack([Xce[g["pel"]], Fce[g["pel"]]]), rows, rtol=1e-6, atol=1e-30)


def test_port_matches_golden_cfg0(port):
    g = golden("cfg0_tria6.npz")
    sc = scenes.cfg0(nen=6, center=(0.0, 0.0, 1.0))
    A, B = port.assemble(sc, nthreads=8)
    _probe_check(A, g, "compact_")
    x, it, st = port.gmres(A, B, tol=1e-10, nthreads=4)
    assert st == 0 and relerr(x, g["x_gmres_tight"]) < 1e-12


def _rand_element(rng, nen):
    base = rng.standard_normal((3, 3))
    if nen == 3:
        return base
    mids = [(base[0] + base[1]) / 2, (base[1] + base[2]) / 2, (base[2] + base[0]) / 2]
    mids = [m + 0.05 * rng.standard_normal(3) for m in mids]  # curved element
    return np.array([base[0], mids[0], base[1], mids[1], base[2], mids[2]])


@pytest.mark.parametrize("nen", [3, 6])
def test_port_integrals_match_reference(port, ref, nen):
    """Every element integral, every singular node, both H forms."""
    rng = np.random.default_rng(99 + nen)
    for trial in range(3):
        X = _rand_element(rng, nen)
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        xe = rng.standard_normal(3) * 3
        for which, flag in (("G", 0), ("H", 0), ("H", 1)):
            a = port.integral(which, nen, X, xe, flag=flag, normal=n)
            b = ref.integral(which, nen, X, xe, flag=flag, normal=n)
            assert np.array_equal(a, b), (which, flag)
        for s in range(1, nen + 1):
            xs = X[s - 1]
            a = port.integral("SG", nen, X, xs, sin=s)
            b = ref.integral("SG", nen, X, xs, sin=s)
            assert np.array_equal(a, b), ("SG", s)
            for flag in (0, 1):
                a = port.integral("SH", nen, X, xs, flag=flag, sin=s, normal=n)
                b = ref.integral("SH", nen, X, xs, flag=flag, sin=s, normal=n)
                assert np.array_equal(a, b), ("SH", s, flag)


@pytest.mark.parametrize("nen", [6, 3])
def test_port_matches_reference_live(port, ref, nen):
    """A scene not in the fixtures, two interfaces' worth of materials."""
    sc = scenes.small(nen=nen, sphere_level=1, plate_cells=2, center=(0.3, -0.2, 0.5), freq=3.3e5)
    Ap, Bp = port.assemble(sc)
    Ar, Br = ref.assemble(sc)
    assert np.array_equal(Ap, Ar) and np.array_equal(Bp, Br)
    Afp, _ = port.assemble(sc, full=True)
    Afr, Bfr = ref.assemble(sc, full=True)
    assert np.array_equal(Afp, Afr)
    assert np.array_equal(port.gauss(Afr, Bfr), ref.gauss(Afr, Bfr))
    xr, _ = ref.gmres(Ar, Br)
    xp, _, _ = port.gmres(Ar, Br)
    assert np.array_equal(xp, xr)
    for i in (0, sc.N // 2, sc.N - 1):
        assert np.array_equal(port.node_normal(sc, i), ref.node_normal(sc, i))
    Fr = ref.force_mst(sc, xr)
    Fp = port.force_mst(sc, xr)
    assert np.array_equal(Fr[2], Fp[2])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "examples")),
                    reason="reference examples not present")
def test_port_reproduces_capacitor_example(port):
    """examples/capacitor-1/quadratic: tria6 conductors, GMRES, 5202 nodes;
    solution.dat is printed with %e (7 significant digits)."""
    d = os.path.join(REFERENCE, "examples", "capacitor-1", "quadratic")
    sc = scenes.read_bem(d)
    A, B = port.assemble(sc, nthreads=os.cpu_count() or 4)
    x, it, st = port.gmres(A, B, nthreads=4)
    assert st == 0 and it == 28
    gold = np.loadtxt(os.path.join(d, "solution.dat"))
    sol = np.stack([x[: sc.N], x[sc.N:]], 1)
    scale = np.abs(gold[:, 3]).max()
    assert np.abs(sol[:, 0] - gold[:, 3]).max() / scale < 2e-6


def test_scene_sizes():
    """Node counts of the generated meshes (icosphere: 40*4^L + 2 tria6 nodes)."""
    n, e = scenes.icosphere(2)
    assert (n.shape[0], e.shape[0]) == (642, 320)
    n, e = scenes.icosphere(4)
    assert (n.shape[0], e.shape[0]) == (10242, 5120)
    n, e = scenes.plate(20.0, 20.0, 10, 10)
    assert (n.shape[0], e.shape[0]) == (441, 200)
    sc = scenes.cfg1()
    assert (sc.N, sc.E) == (17684, 8720)
    sc = scenes.cfg0()
    assert (sc.N, sc.E) == (1524, 720)
    # outward normals on spheres: every element's normal points away from the centre
    n, e = scenes.icosphere(1, nen=3)
    c = np.cross(n[e[:, 1]] - n[e[:, 0]], n[e[:, 2]] - n[e[:, 0]])
    assert (np.einsum("ij,ij->i", c, n[e].mean(1)) > 0).all()


def test_bem_roundtrip(tmp_path):
    sc = scenes.small(nen=6)
    scenes.write_bem(sc, str(tmp_path))
    sc2 = scenes.read_bem(str(tmp_path))
    assert np.array_equal(sc.nodes, sc2.nodes) and np.array_equal(sc.elems, sc2.elems)
    assert np.array_equal(sc.bctype, sc2.bctype) and np.array_equal(sc.mbc, sc2.mbc)
    assert sc.freq == sc2.freq and np.array_equal(sc.mat, sc2.mat)


def test_port_rejects_undefined_bc_type(port):
    sc = scenes.small(nen=3)
    bt = sc.bctype.copy()
    bt[3] = 2
    bad = scenes.Scene(sc.nen, sc.nodes, sc.elems, bt, sc.mbc, sc.ifaces, sc.mat, sc.freq)
    with pytest.raises(ValueError):
        port.assemble(bad.contiguous())
