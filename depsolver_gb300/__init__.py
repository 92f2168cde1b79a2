"""GB300-native implementation of depSolver's boundary-element hot path.

The product is ``libdepsolver_cuda.so`` (CUDA for sm_103a, C ABI in
``include/depsolver_cuda.h``); this package builds it, binds it with ctypes
(``_native``), mirrors the reference's interface on NumPy arrays (``api``)
and generates synthetic scenes in the reference's input model (``scenes``).
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "api", "build"]
