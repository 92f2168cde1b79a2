import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference tree beside the repository (../reference from its root),
# unless DSC_REFERENCE names it; tests that need it skip where it is absent
REFERENCE = os.environ.get("DSC_REFERENCE", os.path.normpath(os.path.join(ROOT, "..", "reference")))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import Port, build_port
    build_port()
    return Port()


@pytest.fixture(scope="session")
def ref():
    from oracle import oracle as orc
    if orc.build_ref() is None:
        pytest.skip("reference sources not present")
    return orc.Ref()


@pytest.fixture(scope="session")
def native():
    """The CUDA library; built if missing.  Never a fallback."""
    from depsolver_gb300 import _native, build
    if not os.path.exists(_native.LIB_PATH):
        build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def gpu(native):
    if native.dsc_device_count() < 1:
        pytest.skip("no CUDA device")
    return native


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))
