"""The direct solve (gaussBksb, src/gaussBksb.c:39-108) as a block LU on the
tensor cores with FP64 iterative refinement, against the FP64 LU, the
oracle's elimination and the reference's own Gauss fixtures.

The reference eliminates without pivoting; so do both GPU factorisations,
and both stop on a pivot within 1e-9 of zero with the reference's message.
The mixed solve must land on the FP64 answer: within 1e-10 relative of the
reference's Gauss solution (the same bar as the FP64 path)."""
import numpy as np
import pytest

from conftest import golden, relerr
from depsolver_gb300 import _native, api, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nen", [6, 3])
def test_mixed_lu_matches_fp64_lu_and_oracle(gpu, port, nen):
    sc = scenes.small(nen=nen)
    Af, Bf = api.electric_form(sc, full=True)
    x64 = api.gauss_bksb(Af, Bf, mode=api.GAUSS_FP64)
    xm = api.gauss_bksb(Af, Bf, mode=api.GAUSS_MIXED)
    mode, it, rr, fb = api.gauss_info()
    # an FP32-accurate factor needs a few refinements, not tens
    assert mode == api.GAUSS_MIXED and not fb and 1 <= it <= 5, (it, rr, fb)
    assert relerr(xm, x64) < 1e-11
    assert relerr(xm, port.gauss(Af, Bf)) < 1e-11


def test_mixed_lu_at_config0_full_form(gpu):
    """2N = 3048 unknowns (not a multiple of the 128-tile): the reference's
    own Gauss solution from the fixture."""
    g = golden("cfg0_tria6.npz")
    sc = scenes.cfg0(nen=6, center=(0.0, 0.0, 1.0))
    Af, Bf = api.electric_form(sc, full=True)
    xm = api.gauss_bksb(Af, Bf, mode=api.GAUSS_MIXED)
    _, it, rr, fb = api.gauss_info()
    assert not fb and it <= 5, (it, rr)
    assert relerr(xm, g["x_gauss"]) < 1e-10
    assert rr < 1e-12


@pytest.mark.parametrize("n", [1, 127, 128, 129, 300])
def test_mixed_lu_ragged_sizes(gpu, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + n * np.eye(n)   # diagonally dominant: no pivoting needed
    b = rng.standard_normal(n)
    x = api.gauss_bksb(A, b, mode=api.GAUSS_MIXED)
    assert relerr(A @ x, b) < 1e-13
    assert relerr(x, np.linalg.solve(A, b)) < 1e-12


def test_mixed_lu_reports_singular_pivot(gpu):
    A = np.eye(200)
    A[150, 150] = 0.0       # exact zero pivot in the second tile
    with pytest.raises(_native.DscError) as ei:
        api.gauss_bksb(A, np.ones(200), mode=api.GAUSS_MIXED)
    assert ei.value.status == 4 and "row 150" in str(ei.value)
    with pytest.raises(_native.DscError) as ei:
        api.gauss_bksb(A, np.ones(200), mode=api.GAUSS_FP64)
    assert ei.value.status == 4


@pytest.mark.parametrize("n", [129, 1000])
def test_host_matrix_read_in_place_or_staged(gpu, n):
    """The host matrix reaches the device read in place by a kernel (where
    the device reads pageable memory) or staged by host threads: the same
    bytes either way, so the same solutions."""
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + n * np.eye(n)
    b = rng.standard_normal(n)
    A2 = rng.standard_normal((n // 2, n)) * 0.01
    A2[:, : n // 2] += np.eye(n // 2) * 3.0
    b2 = rng.standard_normal(n)
    try:
        out = []
        for mode in (1, 0):
            api.set_host_direct(mode)
            x = api.gauss_bksb(A, b, mode=api.GAUSS_MIXED)
            y, it = api.solver_gmres_el(A2, b2, tol=1e-10)
            out.append((x, y, it))
    finally:
        api.set_host_direct(1)
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]
    assert relerr(A @ out[0][0], b) < 1e-13

