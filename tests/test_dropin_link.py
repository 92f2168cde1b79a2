"""The library's link recipe: the reference's own driver objects (without
its assembly, solvers, field, potential and force objects) and
libdepsolver_cuda.so make a depSolver executable whose hot-path calls,
the multipole and ellipsoid force models included, resolve to the library.

Needs the reference sources (built into oracle/_ref/); skipped elsewhere.
Without a GPU the executable must stop at its first library call (matrix
assembly) the reference's way: the message in bem.log and exit status 1.
"""
import os
import shutil
import subprocess

import pytest

from conftest import REFERENCE, ROOT

DROPIN = ["electricFormA_tria3", "electricFormA_tria6", "electricFormFullA_tria3",
          "electricFormFullA_tria6", "gaussBksb", "solverGMRES_el", "field_tria3", "field_tria6",
          "potential_tria3", "potential_tria6", "forceMST_tria3", "forceMST_tria6",
          "forceMultipole_tria3", "forceMultipole_tria6", "forceEllipsoid_tria3", "forceEllipsoid_tria6"]


@pytest.fixture(scope="module")
def exe(native):
    if not os.path.isdir(os.path.join(REFERENCE, "src")):
        pytest.skip("reference sources not present")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin",
                        f"REF={REFERENCE}/src"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return os.path.join(ROOT, "oracle", "_ref", "depSolver-gpu")


def test_hot_path_symbols_come_from_the_library(exe):
    undef = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True,
                           text=True).stdout.split()
    defined = subprocess.run(["nm", "--defined-only", exe], capture_output=True,
                             text=True).stdout.split()
    for name in DROPIN:
        assert name in undef, name          # resolved at run time ...
        assert name not in defined, name    # ... and not by an object of the reference
    for cpu_only in ("intDE_tria6", "intF_tria6", "depolarization"):
        assert cpu_only not in defined, cpu_only   # no reference force code is linked
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "libdepsolver_cuda.so" in ldd


def test_runs_an_example_deck_to_the_first_library_call(exe, native, tmp_path):
    if native.dsc_device_count() > 0:
        pytest.skip("a device is present: the GPU run is covered by the parity tests")
    src = os.path.join(REFERENCE, "examples", "capacitor-1", "quadratic")
    for f in os.listdir(src):
        if f.endswith(".bem"):
            shutil.copy(os.path.join(src, f), tmp_path / f)
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 1
    log = (tmp_path / "bem.log").read_text()
    assert "performing matrix assembly" in log
    assert "no CUDA device available" in log and "PROGRAM TERMINATED" in log
