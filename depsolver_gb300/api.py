"""Host-side mirror of the reference's hot-path interface, on NumPy arrays.

Each function calls the CUDA library through its C ABI and mirrors one
reference entry point (same meaning of arguments and results):

=========================  ===============================================
``electric_form``          electricFormA_* / electricFormFullA_*
                           (src/assembly_el.c:63-589)
``gauss_bksb``             gaussBksb (src/gaussBksb.c:39)
``solver_gmres_el``        solverGMRES_el (src/gmres_el.c:66)
``field``                  field_* (src/field.c:57-200)
``potential``              potential_* (src/potential.c:55-179)
``force_mst``              forceMST_* (src/force.c:348-552)
=========================  ===============================================

Errors that the reference answers with ``exit(1)`` raise
:class:`depsolver_gb300._native.DscError` here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .scenes import Scene


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _u(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def electric_form(sc: Scene, full: bool = False, A: np.ndarray | None = None):
    """Assembles the compact (N x 2N) or full (2N x 2N) system; returns
    (A, B).  A given A is accumulated into, as the reference does."""
    L = _native.lib()
    N = sc.N
    if A is None:
        A = np.zeros((2 * N if full else N, 2 * N))
    B = np.zeros(2 * N)
    ifc = _u(sc.ifaces)
    mat = _f(sc.mat)
    _native.check(L.dsc_assemble(sc.nen, int(full), N, sc.E, sc.n_if, _f(sc.nodes), _u(sc.elems),
                                 _u(sc.bctype), ifc.ctypes.data if sc.n_if else None,
                                 mat.ctypes.data, sc.freq, _f(sc.mbc), A.ctypes.data, A.shape[1],
                                 B))
    return A, B


def gauss_bksb(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    A = _f(A)
    x = _f(B).copy()
    _native.check(_native.lib().dsc_gauss(A.shape[0], A, A.shape[1], x))
    return x


def solver_gmres_el(A: np.ndarray, B: np.ndarray, preCond: int = 1, tol: float = 1.0e-6,
                    max_iters: int = 600, x0: np.ndarray | None = None,
                    log_path: str | None = None):
    """Returns (x, iterations)."""
    A = _f(A)
    x = _f(B).copy()
    it = C.c_uint(0)
    x0a = _f(x0) if x0 is not None else None
    _native.check(_native.lib().dsc_gmres(A.shape[0], preCond, tol, max_iters, A, A.shape[1], x,
                                          x0a.ctypes.data if x0a is not None else None,
                                          log_path.encode() if log_path else None, C.byref(it)))
    return x, it.value


def field(sc: Scene, vB: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """(npts, 6): Re Ex, Im Ex, Re Ey, Im Ey, Re Ez, Im Ez."""
    pts = _f(np.atleast_2d(pts))
    out = np.zeros((pts.shape[0], 6))
    _native.check(_native.lib().dsc_field_points(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems),
                                                 _f(vB), pts.shape[0], pts, out))
    return out


def potential(sc: Scene, vB: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """(npts, 2): Re, Im."""
    pts = _f(np.atleast_2d(pts))
    out = np.zeros((pts.shape[0], 2))
    _native.check(_native.lib().dsc_potential_points(sc.nen, sc.N, sc.E, _f(sc.nodes),
                                                     _u(sc.elems), _f(vB), pts.shape[0], pts, out))
    return out


def force_mst(sc: Scene, vB: np.ndarray, eps: float | None = None):
    """Returns (Fce, Xce, Fcm, Xcm); Fce/Xce rows of non-particle elements are NaN."""
    eps = sc.eps_medium if eps is None else eps
    Fce = np.full((sc.E, 3), np.nan)
    Xce = np.full((sc.E, 3), np.nan)
    Fcm = np.zeros(3)
    Xcm = np.zeros(3)
    _native.check(_native.lib().dsc_force_mst(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems),
                                              _u(sc.bctype), _f(vB), eps, Fce.ctypes.data,
                                              Xce.ctypes.data, Fcm, Xcm))
    return Fce, Xce, Fcm, Xcm
