"""Parity of the CUDA library (through its C ABI) with the reference.

Checked against the golden fixtures made by the reference itself and, at
full matrices, against the C restatement of the reference (oracle/port).
Bars (FP64 path): assembly <= 1e-12 relative to the matrix's largest entry,
nodal solution <= 1e-10 relative, field/potential/force <= 1e-10.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import golden, relerr
from depsolver_gb300 import _native, api, scenes

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-10
ASM_TOL = 1e-12


def _probe(A, g, prefix, tol=ASM_TOL):
    rng = np.random.default_rng(12345)
    r = rng.standard_normal(A.shape[1])
    s = rng.standard_normal(A.shape[0])
    assert relerr(A @ r, g[prefix + "Ar"]) < tol
    assert relerr(A.T @ s, g[prefix + "ATs"]) < tol
    assert relerr(A[g[prefix + "rows_idx"]], g[prefix + "rows"]) < tol


@pytest.mark.parametrize("nen", [6, 3])
@pytest.mark.parametrize("full", [False, True])
def test_assembly_matches_oracle(gpu, port, nen, full):
    sc = scenes.small(nen=nen)
    A, B = api.electric_form(sc, full=full)
    Ap, Bp = port.assemble(sc, full=full)
    assert relerr(A, Ap) < ASM_TOL
    assert np.array_equal(B, Bp)


@pytest.mark.parametrize("nen", [6, 3])
def test_pipeline_matches_golden_small(gpu, nen, tmp_path):
    g = golden(f"small_tria{nen}.npz")
    sc = scenes.small(nen=nen)
    A, B = api.electric_form(sc)
    _probe(A, g, "compact_")
    log = str(tmp_path / "gmres.log")
    x, it = api.solver_gmres_el(A, B, log_path=log)
    assert relerr(x, g["x_gmres"]) < SOL_TOL
    mine = open(log).read().splitlines()
    gold = bytes(g["gmres_log"]).decode().splitlines()
    assert len(mine) == len(gold)  # same iteration count
    assert mine[-2:] == gold[-2:] and mine[:5] == gold[:5]
    xt, _ = api.solver_gmres_el(A, B, tol=1e-10)
    assert relerr(xt, g["x_gmres_tight"]) < SOL_TOL
    Af, Bf = api.electric_form(sc, full=True)
    _probe(Af, g, "full_")
    assert relerr(api.gauss_bksb(Af, Bf), g["x_gauss"]) < SOL_TOL
    assert relerr(api.field(sc, x, g["pts"]), g["field"]) < SOL_TOL
    assert relerr(api.potential(sc, x, g["pts"]), g["potential"]) < SOL_TOL
    Fce, Xce, Fcm, Xcm = api.force_mst(sc, x)
    assert relerr(Fce[g["pel"]], g["Fce"]) < SOL_TOL
    assert relerr(Xce[g["pel"]], g["Xce"]) < 1e-13
    assert np.abs(Fcm - g["Fcm"]).max() <= SOL_TOL * np.abs(g["Fce"]).sum()
    assert relerr(Xcm, g["Xcm"]) < 1e-13


def test_pipeline_matches_golden_dep_trap_2(gpu):
    """The reference's example deck: tria3, REPOSITION, MST force."""
    g = golden("dep_trap_2.npz")
    sc = scenes.Scene(int(g["nen"]), g["nodes"], g["elems"], g["bctype"], g["mbc"], g["ifaces"],
                      g["mat"], float(g["freq"])).contiguous()
    A, B = api.electric_form(sc)
    _probe(A, g, "compact_")
    x, it = api.solver_gmres_el(A, B)
    assert it == 37
    assert relerr(x, g["x_gmres"]) < SOL_TOL
    Fce, Xce, Fcm, Xcm = api.force_mst(sc, x)
    assert relerr(Fce[g["pel"]], g["Fce"]) < SOL_TOL
    lines = bytes(g["golden_force_mst"]).decode().splitlines()
    tot = np.array([float(v) for v in lines[1].split()])
    assert np.allclose(np.r_[Xcm, Fcm], tot, rtol=1e-6, atol=0)


def test_cfg0_gauss_and_tight_gmres(gpu):
    """Level-2 sphere between 10 x 10-cell plates (1524 nodes): Gauss on the
    3048-unknown real form and GMRES at 1e-10, both against the reference."""
    g = golden("cfg0_tria6.npz")
    sc = scenes.cfg0(nen=6, center=(0.0, 0.0, 1.0))
    A, B = api.electric_form(sc)
    _probe(A, g, "compact_")
    xt, _ = api.solver_gmres_el(A, B, tol=1e-10)
    assert relerr(xt, g["x_gmres_tight"]) < SOL_TOL
    Af, Bf = api.electric_form(sc, full=True)
    xg = api.gauss_bksb(Af, Bf)
    assert relerr(xg, g["x_gauss"]) < SOL_TOL
    _, _, Fcm, _ = api.force_mst(sc, xg)
    assert np.abs(Fcm - g["Fcm_gauss"]).max() <= 1e-9 * np.abs(g["Fce"]).sum()
    _, _, Fcm, _ = api.force_mst(sc, xt)
    assert np.abs(Fcm - g["Fcm_tight"]).max() <= 1e-9 * np.abs(g["Fce"]).sum()


def test_field_off_mesh_and_on_nodes_vs_oracle(gpu, port):
    sc = scenes.small(nen=6)
    A, B = port.assemble(sc)
    x, _, _ = port.gmres(A, B)
    p0 = sc.particles[0][0]
    pts = np.vstack([sc.nodes[p0:p0 + 40], sc.nodes[:3],
                     np.random.default_rng(3).uniform(-2, 2, (30, 3))])
    assert relerr(api.field(sc, x, pts), port.field(sc, x, pts)) < SOL_TOL
    assert relerr(api.potential(sc, x, pts), port.potential(sc, x, pts)) < SOL_TOL


def test_few_point_calls_match_batched_and_follow_the_solution(gpu, port):
    """Calls of at most 64 points (the reference's post-processing asks for
    one point per call) keep the solution's quadrature charges on the device
    and move each call's data in one packed copy: they must agree with one
    batched call, on and off the mesh, and after the solution changes."""
    sc = scenes.small(nen=6)
    A, B = port.assemble(sc)
    x, _, _ = port.gmres(A, B)
    p0 = sc.particles[0][0]
    pts = np.vstack([sc.nodes[p0:p0 + 40], sc.nodes[:3], np.random.default_rng(5).uniform(-2, 2, (30, 3))])
    for xs in (x, 2.0 * x + 1e-3, x):
        for fn in (api.field, api.potential):
            full = fn(sc, xs, pts)   # 73 points: the batched path
            one = np.vstack([fn(sc, xs, p[None]) for p in pts[::7]])
            chunks = np.vstack([fn(sc, xs, pts[i:i + 50]) for i in range(0, len(pts), 50)])
            assert relerr(one, full[::7]) < 1e-13
            assert relerr(chunks, full) < 1e-13
        assert relerr(api.field(sc, xs, pts[:5]), port.field(sc, xs, pts[:5])) < SOL_TOL


@pytest.mark.parametrize("full", [False, True])
def test_assembly_rows_in_place_or_staged(gpu, full):
    """The assembled rows reach the caller's matrix added in place by the
    device (where it writes pageable host memory) or through pinned staging
    and host threads: the same values either way, accumulated into what the
    matrix held."""
    sc = scenes.small(nen=6)
    out = []
    try:
        for mode in (2, 0):
            api.set_host_direct(mode)
            A0 = np.full((2 * sc.N if full else sc.N, 2 * sc.N), 0.25)
            A, B = api.electric_form(sc, full=full, A=A0)
            out.append(A.copy())
    finally:
        api.set_host_direct(1)
    assert np.array_equal(out[0], out[1])


def test_assembly_accumulates_like_reference(gpu, port):
    sc = scenes.small(nen=3)
    A0 = np.full((sc.N, 2 * sc.N), 0.25)
    A, _ = api.electric_form(sc, A=A0.copy())
    Ap, _ = port.assemble(sc)
    assert relerr(A - 0.25, Ap) < ASM_TOL


def test_pure_conductor_scene(gpu, port):
    """No interfaces (nInterfaces = 0), like examples/capacitor-1."""
    n1, e1 = scenes.plate(4.0, 4.0, 3, 3, (0, 0, 1.0))
    n2, e2 = scenes.plate(4.0, 4.0, 3, 3, (0, 0, -1.0))
    sc = scenes._assemble([(n1, e1, "conductor", 1.0), (n2, e2, "conductor", -1.0)], 6,
                          [[0.0, 80.0]], np.zeros((0, 2)), 1e6, "capacitor")
    A, B = api.electric_form(sc)
    Ap, Bp = port.assemble(sc)
    assert relerr(A, Ap) < ASM_TOL
    # At the compiled 1e-6 tolerance this scene converges on a tie: the
    # oracle's residual at step 11 is within 9% of the tolerance and a
    # different summation order stops one step earlier, so compare the
    # tight-tolerance and direct solutions instead.
    x, it = api.solver_gmres_el(A, B, tol=1e-12)
    xp, itp, _ = port.gmres(Ap, Bp, tol=1e-12)
    assert abs(it - itp) <= 1 and relerr(x, xp) < SOL_TOL
    Af, Bf = api.electric_form(sc, full=True)
    assert relerr(api.gauss_bksb(Af, Bf), xp) < 1e-9


def test_errors_are_reported_not_faked(gpu):
    sc = scenes.small(nen=3)
    bt = sc.bctype.copy()
    bt[2] = 3
    bad = scenes.Scene(sc.nen, sc.nodes, sc.elems, bt, sc.mbc, sc.ifaces, sc.mat, sc.freq).contiguous()
    with pytest.raises(_native.DscError) as ei:
        api.electric_form(bad)
    assert ei.value.status == 3
    A, B = api.electric_form(sc)
    with pytest.raises(_native.DscError) as ei:
        api.solver_gmres_el(A, B, max_iters=2)
    assert ei.value.status == 5
    with pytest.raises(_native.DscError) as ei:
        api.gauss_bksb(np.zeros((8, 8)), np.ones(8))
    assert ei.value.status == 4


def _rows(arr):
    """Row-pointer view (double** / unsigned**) of a C-contiguous array."""
    T = C.c_double if arr.dtype == np.float64 else C.c_uint
    ptrs = (C.POINTER(T) * arr.shape[0])()
    base = arr.ctypes.data
    for i in range(arr.shape[0]):
        ptrs[i] = C.cast(base + i * arr.strides[0], C.POINTER(T))
    return ptrs


@pytest.mark.parametrize("nen", [6, 3])
def test_dropin_row_pointer_entry_points(gpu, port, nen, tmp_path):
    """The reference's own signatures: globals, double**, gmres.log in cwd."""
    L = gpu
    sc = scenes.small(nen=nen)
    N, E = sc.N, sc.E
    C.c_uint.in_dll(L, "nNodes").value = N
    C.c_uint.in_dll(L, "nElems").value = E
    C.c_uint.in_dll(L, "nInterfaces").value = sc.n_if
    nodes = np.ascontiguousarray(sc.nodes)
    elems = np.ascontiguousarray(sc.elems, dtype=np.uint32)
    mat = np.ascontiguousarray(sc.mat)
    ifc = np.ascontiguousarray(sc.ifaces, dtype=np.uint32)
    mbc = np.ascontiguousarray(sc.mbc)
    bct = np.ascontiguousarray(sc.bctype, dtype=np.uint32)
    prob = np.array([sc.freq])
    A = np.zeros((N, 2 * N))
    B = np.zeros(2 * N)
    fn = getattr(L, f"electricFormA_tria{nen}")
    fn.restype = C.c_int
    fn(_rows(nodes), _rows(elems), bct.ctypes.data_as(C.c_void_p), _rows(ifc), _rows(mat),
       prob.ctypes.data_as(C.c_void_p), _rows(A), _rows(mbc), B.ctypes.data_as(C.c_void_p))
    Ap, Bp = port.assemble(sc)
    assert relerr(A, Ap) < ASM_TOL and np.array_equal(B, Bp)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        L.solverGMRES_el(C.c_uint(1), C.c_uint(0), _rows(A), B.ctypes.data_as(C.c_void_p))
        log = open("gmres.log").read()
    finally:
        os.chdir(cwd)
    xp, itp, _ = port.gmres(Ap, Bp, log_path=str(tmp_path / "port.log"))
    assert relerr(B, xp) < SOL_TOL
    assert log.splitlines()[-2:] == open(tmp_path / "port.log").read().splitlines()[-2:]
    Af = np.zeros((2 * N, 2 * N))
    Bf = np.zeros(2 * N)
    fn = getattr(L, f"electricFormFullA_tria{nen}")
    fn(_rows(nodes), _rows(elems), bct.ctypes.data_as(C.c_void_p), _rows(ifc), _rows(mat),
       prob.ctypes.data_as(C.c_void_p), _rows(Af), _rows(mbc), Bf.ctypes.data_as(C.c_void_p))
    L.gaussBksb(C.c_uint(2 * N), _rows(Af), Bf.ctypes.data_as(C.c_void_p))
    Afp, Bfp = port.assemble(sc, full=True)
    assert relerr(Bf, port.gauss(Afp, Bfp)) < SOL_TOL
    mE = np.zeros(6)
    Xin = np.ascontiguousarray(sc.nodes[sc.particles[0][0] + 2])
    getattr(L, f"field_tria{nen}")(Xin.ctypes.data_as(C.c_void_p), _rows(nodes), _rows(elems),
                                   xp.ctypes.data_as(C.c_void_p), mE.ctypes.data_as(C.c_void_p))
    assert relerr(mE, port.field(sc, xp, Xin)[0]) < SOL_TOL
    Fce = np.zeros((E, 3))
    Xce = np.zeros((E, 3))
    Fcm = np.zeros(3)
    Xcm = np.zeros(3)
    getattr(L, f"forceMST_tria{nen}")(_rows(nodes), _rows(elems), bct.ctypes.data_as(C.c_void_p),
                                      xp.ctypes.data_as(C.c_void_p), C.c_double(sc.eps_medium),
                                      _rows(Fce), _rows(Xce), Fcm.ctypes.data_as(C.c_void_p),
                                      Xcm.ctypes.data_as(C.c_void_p))
    Fp = port.force_mst(sc, xp)
    pel = sc.bctype[sc.elems[:, 0] - 1] == 6
    assert relerr(Fce[pel], Fp[0][pel]) < SOL_TOL
    assert np.abs(Fcm - Fp[2]).max() <= SOL_TOL * np.abs(Fp[0][pel]).sum()
