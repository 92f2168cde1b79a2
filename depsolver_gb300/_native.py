"""ctypes binding of libdepsolver_cuda.so (the in-tree CUDA library).

There is no fallback: if the shared library is missing or fails to load,
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdepsolver_cuda.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "depsolver_cuda.h")

_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


class DscError(RuntimeError):
    """A dsc_* entry point returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"status {status}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run depsolver_gb300.build.build() first")
        L = C.CDLL(LIB_PATH, mode=C.RTLD_LOCAL)
        L.dsc_last_error.restype = C.c_char_p
        L.dsc_device_count.restype = C.c_int
        L.dsc_assemble.restype = C.c_int
        L.dsc_assemble.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_uint, C.c_uint, _dp, _up, _up,
                                   C.c_void_p, C.c_void_p, C.c_double, _dp, C.c_void_p, C.c_size_t,
                                   _dp]
        L.dsc_gauss.restype = C.c_int
        L.dsc_gauss.argtypes = [C.c_uint, _dp, C.c_size_t, _dp]
        L.dsc_set_gauss_mode.restype = C.c_int
        L.dsc_set_gauss_mode.argtypes = [C.c_int]
        L.dsc_set_host_direct.restype = C.c_int
        L.dsc_set_host_direct.argtypes = [C.c_int]
        L.dsc_gauss_info.restype = C.c_int
        L.dsc_gauss_info.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int),
                                     C.c_void_p]
        L.dsc_gmres.restype = C.c_int
        L.dsc_gmres.argtypes = [C.c_uint, C.c_uint, C.c_double, C.c_uint, _dp, C.c_size_t, _dp,
                                C.c_void_p, C.c_char_p, C.POINTER(C.c_uint)]
        for nm in ("dsc_field_points", "dsc_potential_points"):
            f = getattr(L, nm)
            f.restype = C.c_int
            f.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, C.c_uint, _dp, _dp]
        L.dsc_force_multipole.restype = C.c_int
        L.dsc_force_multipole.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, C.c_uint, _dp, C.c_uint,
                                          C.c_double, _dp, C.c_double, _dp]
        L.dsc_force_ellipsoid.restype = C.c_int
        L.dsc_force_ellipsoid.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, C.c_uint, _dp, C.c_uint,
                                          C.c_void_p, _dp, C.c_double, _dp]
        L.dsc_depolarization.restype = C.c_int
        L.dsc_depolarization.argtypes = [_dp, _dp]
        L.dsc_force_mst.restype = C.c_int
        L.dsc_force_mst.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_double,
                                    C.c_void_p, C.c_void_p, _dp, _dp]
        L.dsc_session_create.restype = C.c_int
        L.dsc_session_create.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_uint,
                                         C.c_void_p, C.c_uint, _dp, C.POINTER(C.c_void_p)]
        L.dsc_session_destroy.restype = None
        L.dsc_session_destroy.argtypes = [C.c_void_p]
        L.dsc_session_assemble.restype = C.c_int
        L.dsc_session_assemble.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_geometric_matrix.restype = C.c_int
        L.dsc_session_geometric_matrix.argtypes = [C.c_void_p, C.c_int, _dp, C.c_size_t]
        L.dsc_session_solve.restype = C.c_int
        L.dsc_session_solve.argtypes = [C.c_void_p, C.c_int, C.c_uint, _dp, C.c_double, C.c_uint,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        L.dsc_tc_gemm.restype = C.c_int
        L.dsc_tc_gemm.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int, C.c_int]
        L.dsc_tc_gemm_noalloc.restype = C.c_int
        L.dsc_tc_gemm_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_size_t,
                                          C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int,
                                          C.c_void_p]
        L.dsc_positions_create.restype = C.c_int
        L.dsc_positions_create.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_uint,
                                           C.c_void_p, C.c_uint, _dp, C.POINTER(C.c_void_p)]
        L.dsc_positions_destroy.restype = None
        L.dsc_positions_destroy.argtypes = [C.c_void_p]
        L.dsc_positions_add_particle.restype = C.c_int
        L.dsc_positions_add_particle.argtypes = [C.c_void_p, C.c_uint, C.c_uint, _dp, _up, C.c_uint]
        for nm in ("dsc_positions_set_workers", "dsc_positions_set_mixed_assembly",
                   "dsc_positions_set_timing"):
            getattr(L, nm).restype = C.c_int
            getattr(L, nm).argtypes = [C.c_void_p, C.c_int]
        L.dsc_positions_timing.restype = C.c_int
        L.dsc_positions_timing.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.dsc_positions_inversions.restype = C.c_int
        L.dsc_positions_inversions.argtypes = [C.c_void_p]
        L.dsc_positions_solve.restype = C.c_int
        L.dsc_positions_solve.argtypes = [C.c_void_p, C.c_uint, _up, _dp, C.c_uint, _dp, C.c_double,
                                          C.c_uint, _dp, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
        L.dsc_force_crossover.restype = C.c_double
        L.dsc_force_crossover.argtypes = [C.c_uint, _dp, _dp, C.c_void_p]
        L.dsc_bem_read.restype = C.c_int
        L.dsc_bem_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        L.dsc_bem_free.restype = None
        L.dsc_bem_free.argtypes = [C.c_void_p]
        L.dsc_bem_info.restype = C.c_int
        L.dsc_bem_info.argtypes = [C.c_void_p] + [C.c_void_p] * 16
        L.dsc_bem_arrays.restype = C.c_int
        L.dsc_bem_arrays.argtypes = [C.c_void_p] + [C.c_void_p] * 8
        L.dsc_node_normals.restype = C.c_int
        L.dsc_node_normals.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp]
        L.dsc_session_stream.restype = C.c_void_p
        L.dsc_session_stream.argtypes = [C.c_void_p]
        L.dsc_kernel_launches.restype = C.c_ulonglong
        L.dsc_kernel_launches.argtypes = []
        L.dsc_session_set_timing.restype = C.c_int
        L.dsc_session_set_timing.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_set_preconditioner.restype = C.c_int
        L.dsc_session_set_fp64_jacobi.restype = C.c_int
        L.dsc_session_set_fp64_jacobi.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_set_residual.restype = C.c_int
        L.dsc_session_set_residual.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_set_field_tensor.restype = C.c_int
        L.dsc_session_set_field_tensor.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_set_mixed_assembly.restype = C.c_int
        L.dsc_session_set_mixed_assembly.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_set_preconditioner.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_particles.restype = C.c_int
        L.dsc_session_particles.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
        L.dsc_set_autotune.restype = C.c_int
        L.dsc_set_autotune.argtypes = [C.c_int]
        L.dsc_autotune_table.restype = C.c_int
        L.dsc_autotune_table.argtypes = [C.c_void_p, C.c_int]
        L.dsc_session_status.restype = C.c_int
        L.dsc_session_status.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
        L.dsc_session_preconditioner_blocks.restype = C.c_int
        L.dsc_session_preconditioner_blocks.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.dsc_session_timing.restype = C.c_int
        L.dsc_session_timing.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.dsc_sweep.restype = C.c_int
        L.dsc_sweep.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_uint,
                                C.c_void_p, C.c_uint, _dp, C.c_int, C.c_uint, _dp, C.c_double,
                                C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise DscError(status, lib().dsc_last_error().decode(errors="replace"))


def declared_symbols() -> list[str]:
    """Function names declared in include/depsolver_cuda.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
    skip = {"if", "defined"}
    return sorted({n for n in names if n not in skip})


def declared_globals() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = []
    for m in re.finditer(r"^extern\s+([^;({\"]*);", text, flags=re.M):
        decl = m.group(1)
        decl = re.sub(r"^(unsigned int|FILE\s*\*|double|int)\s*", "", decl)
        out += [d.strip().lstrip("*") for d in decl.split(",")]
    return out
