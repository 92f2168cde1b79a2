"""The C ABI: the library loads, exports every function and global that
include/depsolver_cuda.h declares, and has no CPU fallback (without a GPU
every compute entry point fails with a CUDA status)."""
import ctypes as C

import numpy as np
import pytest

from depsolver_gb300 import _native, scenes


def test_exports_every_declared_symbol(native):
    names = _native.declared_symbols()
    assert "electricFormA_tria6" in names and "solverGMRES_el" in names and "dsc_assemble" in names
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing
    for g in _native.declared_globals():
        C.c_uint.in_dll(native, g) if g != "file_log" else C.c_void_p.in_dll(native, g)


def test_header_matches_reference_dropin_set():
    """Every hot-path entry point of the reference has a drop-in."""
    expected = {
        "electricFormA_tria3", "electricFormA_tria6", "electricFormFullA_tria3",
        "electricFormFullA_tria6", "gaussBksb", "solverGMRES_el", "field_tria3", "field_tria6",
        "potential_tria3", "potential_tria6", "forceMST_tria3", "forceMST_tria6",
    }
    assert expected <= set(_native.declared_symbols())


def test_no_cpu_fallback_without_device(native):
    if native.dsc_device_count() > 0:
        pytest.skip("a device is present")
    from depsolver_gb300 import api
    sc = scenes.small(nen=3)
    with pytest.raises(_native.DscError) as ei:
        api.electric_form(sc)
    assert ei.value.status == 1 and "device" in str(ei.value)


def test_force_crossover_host_logic(native):
    """dsc_force_crossover (the position sweep's crossover_hz): first sign
    change of the force along its lowest-frequency direction, interpolated
    linearly in log f; NaN without a sign change or past an unconverged
    system."""
    L = _native.lib()
    f = np.logspace(3, 8, 6)
    F = np.zeros((6, 9))
    p = np.array([3.0, 2.0, 1.0, -1.0, -2.0, -3.0])     # changes sign between f[2] and f[3]
    d = np.array([0.6, 0.0, 0.8])
    F[:, :3] = p[:, None] * d
    x = L.dsc_force_crossover(6, f, F, None)
    assert np.isclose(x, np.exp(0.5 * (np.log(f[2]) + np.log(f[3]))), rtol=1e-14)
    st = np.zeros(6, dtype=np.int32)
    st[1] = 1
    assert np.isnan(L.dsc_force_crossover(6, f, F, st.ctypes.data))
    F[:, :3] = np.abs(p)[:, None] * d
    assert np.isnan(L.dsc_force_crossover(6, f, F, None))
    assert np.isnan(L.dsc_force_crossover(1, f, F, None))


def test_host_direct_modes(native):
    """dsc_set_host_direct takes 0 (staged both ways), 1 (host matrices read
    in place, the default) or 2 (the assembled rows also written in place),
    and rejects anything else without changing the mode."""
    L = _native.lib()
    assert L.dsc_set_host_direct(C.c_int(3)) == 2  # DSC_ERR_ARG
    assert b"mode 3" in L.dsc_last_error()
    for mode in (0, 2, 1):
        assert L.dsc_set_host_direct(C.c_int(mode)) == 0
