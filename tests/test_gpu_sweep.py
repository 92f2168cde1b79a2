"""Frequency sweeps on a device-resident scene (dsc_session_* / dsc_sweep).

The plain FP64 path must reproduce the reference's GMRES (through the
strict compact path and the oracle); the mixed path must reach the FP64
solution: Maxwell-stress force within 1e-6 of the force scale (sum over
particle elements of |Fce|), and the nodal solution within 1e-9 relative
when the matrix's regular pairs are assembled in double-FP32, within 1e-5
(the FP32 entries' ~1e-7 times the conditioning) when they are FP32.
"""
import numpy as np
import pytest

from conftest import relerr
from depsolver_gb300 import api, scenes

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-6   # |Fcm_mixed - Fcm_fp64| / sum|Fce|


@pytest.mark.parametrize("nen", [6, 3])
def test_fp64_session_matches_reference_gmres(gpu, port, nen):
    sc = scenes.small(nen=nen)
    s = api.Session(sc)
    forces, its, sig = s.solve([sc.freq], mode=api.MODE_FP64, tol=1e-6, want_sigma=True)
    Ap, Bp = port.assemble(sc)
    xp, itp, st = port.gmres(Ap, Bp)
    assert st == 0 and its[0] == itp
    assert relerr(sig[0], xp) < 1e-10
    Fce, Xce, Fcm, Xcm = port.force_mst(sc, xp)
    pel = sc.bctype[sc.elems[:, 0] - 1] == 6
    assert np.abs(forces[0, :3] - Fcm).max() <= 1e-9 * np.abs(Fce[pel]).sum()
    assert relerr(forces[0, 3:6], Xcm) < 1e-13
    assert np.allclose(forces[0, 6:9], np.abs(Fce[pel]).sum(0), rtol=1e-9)


@pytest.mark.parametrize("asm,sig_tol", [(api.ASM_DF32, 1e-9), (api.ASM_FP32, 1e-5)])
@pytest.mark.parametrize("nen", [6, 3])
def test_mixed_matches_fp64_across_frequencies(gpu, port, nen, asm, sig_tol):
    sc = scenes.small(nen=nen, sphere_level=2, plate_cells=4)
    freqs = np.logspace(3, 8, 6)
    s = api.Session(sc)
    s.set_mixed_assembly(asm)
    # the mixed solve first: it assembles K with double-FP32 or FP32 regular
    # pairs; the FP64 solve then assembles it again in FP64
    fmx, itmx, smx = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    f64, it64, s64 = s.solve(freqs, mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    for k in range(len(freqs)):
        assert relerr(smx[k], s64[k]) < sig_tol, k
        scale = f64[k, 6:9].sum()
        assert np.abs(fmx[k, :3] - f64[k, :3]).max() <= FORCE_TOL * scale, k
    # the reference's own solution at one frequency, by the oracle
    scf = sc.with_freq(freqs[2])
    Ap, Bp = port.assemble(scf)
    xp, _, st = port.gmres(Ap, Bp, tol=1e-12)
    assert st == 0 and relerr(smx[2], xp) < sig_tol


def test_sweep_equals_session(gpu):
    sc = scenes.small(nen=6)
    freqs = [1e4, 1e6, 5e7]
    f1, _, s1 = api.sweep(sc, freqs, mode=api.MODE_MIXED, tol=1e-11)
    s = api.Session(sc)
    f2, _, s2 = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    assert np.array_equal(s1, s2) and np.array_equal(f1, f2)


def test_session_timing_counts_kernels(gpu):
    sc = scenes.small(nen=6)
    s = api.Session(sc)
    s.set_timing(True)
    s.solve([1e6], mode=api.MODE_FP64, tol=1e-6)
    t = s.timing()
    assert t["asm_regular"][1] >= 1 and t["gemv_K64"][1] >= 5 and t["field"][1] == 1
    assert all(ms >= 0 for ms, _, _ in t.values())
    # algorithmic work: every (row, element) pair once; K read once per product
    assert t["asm_regular"][2] == sc.N * sc.E
    assert t["gemv_K64"][2] == 8.0 * sc.N * sc.N * t["gemv_K64"][1]
    F = 3
    s.solve(np.logspace(4, 7, F), mode=api.MODE_MIXED, tol=1e-10)
    t = s.timing()
    assert t["gemm_K"][1] >= 5 and t["gram_schmidt"][1] >= 5
    assert t["gemm_K"][2] == 12.0 * sc.N * sc.N * F * t["gemm_K"][1]
    # each Gram-Schmidt pass reads at least one basis vector of every
    # active system (16 bytes per row and system)
    assert t["gram_schmidt"][2] >= 16.0 * sc.N * t["gram_schmidt"][1]
    # the first residual's digit products: 8 digits of K against 3, 3, 3,
    # 3, 3, 3, 2, 1 digits of the 2F solution columns
    assert t["asm_regular"][1] == 0 and t["residual_fp64"][2] == sc.N * sc.N * 2 * F * 21


@pytest.mark.parametrize("nen", [6, 3])
def test_double_fp32_assembly_matches_fp64(gpu, port, nen):
    """K with the regular pairs in double-FP32 (the mixed mode's
    double-FP32 assembly; its singular pairs are double-FP32 in every mixed
    assembly) against the FP64 assembly, to 1e-13 of the matrix's scale, and
    the FP64 K against the C restatement of the reference."""
    sc = scenes.small(nen=nen)
    s = api.Session(sc)
    s.set_mixed_assembly(api.ASM_DF32)
    s.assemble(api.MODE_MIXED)
    Kd = s.geometric_matrix(api.MODE_MIXED)
    K64 = s.geometric_matrix(api.MODE_FP64)      # assembles again in FP64
    scale = np.abs(K64).max()
    assert np.abs(Kd - K64).max() <= 1e-13 * scale
    assert not np.array_equal(Kd, K64)            # it is a different computation
    # the FP64 K against the oracle's compact matrix (conductor rows: C int G)
    A, _ = port.assemble(sc)
    N = sc.N
    cond = sc.bctype[:N] != 6
    assert relerr(K64[cond], A[cond][:, :N]) < 1e-12


@pytest.mark.parametrize("nen", [6, 3])
def test_fp32_assembly_matches_fp64(gpu, nen):
    """K with the regular pairs in FP32 (centroid-relative offsets): every
    entry within a few FP32 units of its row's scale of the FP64 one."""
    sc = scenes.small(nen=nen)
    s = api.Session(sc)
    s.set_mixed_assembly(api.ASM_FP32)
    s.assemble(api.MODE_MIXED)
    Kf = s.geometric_matrix(api.MODE_MIXED)
    K64 = s.geometric_matrix(api.MODE_FP64)
    rowmax = np.abs(K64).max(axis=1)               # row i = collocation node
    err = np.abs(Kf - K64).max(axis=1) / rowmax
    assert err.max() <= 2e-6, float(err.max())
    assert np.linalg.norm(Kf - K64) <= 1e-6 * np.linalg.norm(K64)
    assert not np.array_equal(Kf, K64)


def test_conductor_preconditioner_cuts_iterations_not_accuracy(gpu):
    """The conductor-block right preconditioner (one block per plate) leaves
    the solution that of the unpreconditioned system -- both runs within
    1e-9 of the FP64 path -- and needs far fewer inner iterations."""
    sc = scenes.small(nen=6, sphere_level=2, plate_cells=6)
    freqs = np.logspace(3, 8, 4)
    s = api.Session(sc)
    s.set_mixed_assembly(api.ASM_DF32)
    ntop = int((sc.bctype[: sc.N] == 1).sum())
    assert s.preconditioner_blocks() == [ntop // 2, ntop // 2]
    f_on, it_on, s_on = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    s.set_preconditioner(False)
    f_off, it_off, s_off = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    s.set_preconditioner(True)
    f64, _, s64 = s.solve(freqs, mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    for k in range(len(freqs)):
        assert relerr(s_on[k], s64[k]) < 1e-9 and relerr(s_off[k], s64[k]) < 1e-9, k
        scale = f64[k, 6:9].sum()
        assert np.abs(f_on[k, :3] - f64[k, :3]).max() <= FORCE_TOL * scale, k
    assert it_on.max() * 2 <= it_off.min(), (it_on, it_off)
    t = s.timing()
    assert set(["precond_build", "precond_apply"]) <= set(t)


def test_field_tensor_cores_match_fp32_pipes(gpu):
    """The batched field's far pairs on the tensor cores (3xFP16 products of
    the generated kernel, read back into FP32 every 64 quadrature points)
    give the forces of the all-FP32-pipe pass to far below the metric's
    bound, and both stay within it against the FP64 path."""
    sc = scenes.small(nen=6, sphere_level=2, plate_cells=6)
    freqs = np.logspace(3, 8, 8)
    s = api.Session(sc)
    f_tc, _, s_tc = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    s.set_field_tensor(False)
    f_32, _, s_32 = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    f64, _, _ = s.solve(freqs, mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    assert np.array_equal(s_tc, s_32)  # the field does not feed back into the solve
    for k in range(len(freqs)):
        scale = f64[k, 6:9].sum()
        assert np.abs(f_tc[k, :3] - f_32[k, :3]).max() <= 1e-7 * scale, k
        assert np.allclose(f_tc[k, 6:9], f_32[k, 6:9], rtol=1e-5), k
        assert np.abs(f_tc[k, :3] - f64[k, :3]).max() <= FORCE_TOL * scale, k


@pytest.mark.parametrize("mode", [api.MODE_MIXED, api.MODE_FP64])
def test_iteration_cap_reports_capped_systems(gpu, mode):
    """max_iters caps every system's GMRES iterations; systems that stop
    short get the status SYS_CAPPED and NaN results (no fake solution), the
    call reports DSC_ERR_NOCONVERGE, and the next uncapped sweep on the same
    session is that of a fresh session."""
    from depsolver_gb300 import _native
    sc = scenes.small(nen=6)
    freqs = [1e4, 1e6, 5e7]
    s = api.Session(sc)
    with pytest.raises(_native.DscError) as e:
        s.solve(freqs, mode=mode, tol=1e-11, max_iters=1)
    assert e.value.status == api.ERR_NOCONVERGE
    f, its, sig = s.solve(freqs, mode=mode, tol=1e-11, max_iters=1, want_sigma=True, partial=True)
    assert (s.status() == api.SYS_CAPPED).all(), s.status()
    assert np.isnan(f).all() and np.isnan(sig).all()
    assert (its == 1).all(), its
    f2, it2, s2 = s.solve(freqs, mode=mode, tol=1e-11, want_sigma=True)
    assert (s.status() == api.SYS_CONVERGED).all() and (it2 > 1).all()
    f3, it3, s3 = api.Session(sc).solve(freqs, mode=mode, tol=1e-11, want_sigma=True)
    assert np.array_equal(f2, f3) and np.array_equal(s2, s3) and np.array_equal(it2, it3)


def test_iteration_cap_within_a_batch(gpu):
    """Under a cap each system of a batch either converges within it (to the
    uncapped sweep's solution) or stops at the cap with status SYS_CAPPED
    and NaN results; the others of the batch are unaffected."""
    sc = scenes.small(nen=6, sphere_level=2, plate_cells=4)
    freqs = np.logspace(3, 8, 6)
    s = api.Session(sc)
    s.set_preconditioner(False)
    f0, it0, s0 = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    for cap in (int(it0.min()) // 2, int(it0.max()) - 1):
        f1, it1, s1 = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, max_iters=cap, want_sigma=True,
                              partial=True)
        st = s.status()
        ok = st == api.SYS_CONVERGED
        assert ((st == api.SYS_CONVERGED) | (st == api.SYS_CAPPED)).all(), st
        assert (it1 <= cap).all(), (it1, cap)
        assert np.isnan(f1[~ok]).all() and np.isnan(s1[~ok]).all() and not np.isnan(f1[ok]).any()
        for k in np.nonzero(ok)[0]:
            assert relerr(s1[k], s0[k]) < 1e-8, k
        if cap == int(it0.min()) // 2:
            assert (~ok).all(), (st, it0, cap)


def test_sweeps_of_different_sizes_on_one_session(gpu):
    """A session that solved a larger batch solves a smaller one (and the
    remainder batch of a sweep longer than 64) exactly as a fresh session."""
    sc = scenes.small(nen=6, sphere_level=2, plate_cells=4)
    s = api.Session(sc)
    s.solve(np.logspace(3, 8, 6), mode=api.MODE_MIXED, tol=1e-10)
    f1, _, s1 = s.solve([1e6], mode=api.MODE_MIXED, tol=1e-10, want_sigma=True)
    f2, _, s2 = api.Session(sc).solve([1e6], mode=api.MODE_MIXED, tol=1e-10, want_sigma=True)
    assert np.array_equal(f1, f2) and np.array_equal(s1, s2)
    freqs = np.logspace(3, 8, 70)
    f3, _, _ = api.Session(sc).solve(freqs, mode=api.MODE_MIXED, tol=1e-10)
    f4, _, _ = api.Session(sc).solve(freqs[64:], mode=api.MODE_MIXED, tol=1e-10)
    assert np.array_equal(f3[64:], f4)


def test_fp64_gemv_first_residual_matches_digits(gpu):
    """The mixed mode's first residual from an FP64 GEMV over K (the path of
    scenes whose K digits would not fit the device) lands on the same
    solution as the tensor-core digit product."""
    sc = scenes.small(nen=6, sphere_level=2, plate_cells=4)
    freqs = np.logspace(3, 8, 4)
    s = api.Session(sc)
    fd, _, sd = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    s.set_residual(api.RESIDUAL_FP64)
    s.set_timing(True)
    s.timing()
    fg, _, sg = s.solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    t = s.timing()
    assert t["residual_fp64"][1] == 0 and t["gemv_K64"][1] >= 1   # no digit products: the GEMV ran
    for k in range(len(freqs)):
        assert relerr(sg[k], sd[k]) < 1e-9, k
        assert np.abs(fg[k, :3] - fd[k, :3]).max() <= 1e-8 * fd[k, 6:9].sum(), k


def test_comb_trap_mixed_matches_fp64(gpu):
    """A small castellated trap (two interdigitated combs, a chain of
    spheres): many conductor blocks and several particles in one solve."""
    sc = scenes.comb_trap(fingers=3, cells=(2, 8), spheres=3, sphere_level=2, spacing=2.5)
    s = api.Session(sc)
    assert len(s.preconditioner_blocks()) == 6
    fm, _, sm = s.solve([1e6], mode=api.MODE_MIXED, tol=1e-10, want_sigma=True)
    pm = s.particles()[0]
    f64, _, s64 = s.solve([1e6], mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    p64 = s.particles()[0]
    assert pm.shape == (3, 12)
    assert np.abs(fm[0, :3] - f64[0, :3]).max() <= FORCE_TOL * f64[0, 6:9].sum()
    for k in range(3):
        assert np.abs(pm[k, :3] - p64[k, :3]).max() <= FORCE_TOL * p64[k, 6:9].sum(), k


def test_autotuned_splits_keep_the_solution(gpu):
    """The split count the autotuner picks for the tensor-core product only
    changes the rounding of the products, not the solution."""
    sc = scenes.small(nen=6, sphere_level=2, plate_cells=5)
    freqs = np.logspace(3, 8, 5)
    api.set_autotune(False)
    try:
        f0, _, s0 = api.Session(sc).solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    finally:
        api.set_autotune(True)
    f1, _, s1 = api.Session(sc).solve(freqs, mode=api.MODE_MIXED, tol=1e-11, want_sigma=True)
    assert any(r[0] == sc.N and r[1] == 2 * len(freqs) and r[2] >= 1 for r in api.autotune_table())
    for k in range(len(freqs)):
        assert relerr(s1[k], s0[k]) < 1e-9, k
        assert np.abs(f1[k, :3] - f0[k, :3]).max() <= 1e-8 * f0[k, 6:9].sum(), k
