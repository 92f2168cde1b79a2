"""ctypes front-ends of the two CPU oracles (test infrastructure only).

``Port`` drives ``oracle/liboracle.so`` (the C restatement, builds anywhere);
``Ref`` drives ``oracle/_ref/libdsref.so`` (the reference's own objects plus
``oracle/ref_harness.c``; built only where the reference tree exists).  Both
take a :class:`depsolver_gb300.scenes.Scene` and NumPy arrays.

The reference's GMRES writes ``gmres.log`` (and its error path ``bem.log``)
in the working directory, so :meth:`Ref.gmres` runs inside a scratch
directory.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdsref.so")
# the reference tree beside the repository (../reference from its root),
# unless DSC_REFERENCE_SRC names its src directory
REF_SRC = os.environ.get("DSC_REFERENCE_SRC",
                         os.path.normpath(os.path.join(HERE, "..", "..", "reference", "src")))

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def build_ref() -> str | None:
    if not os.path.isdir(REF_SRC):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)
    return REF_SO


@contextlib.contextmanager
def _in_dir(d):
    old = os.getcwd()
    os.chdir(d)
    try:
        yield
    finally:
        os.chdir(old)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _u(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


class Port:
    """The C restatement of the reference (oracle/port)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build_port()
        L = C.CDLL(path)
        self.lib = L
        L.orc_assemble.restype = C.c_int
        L.orc_assemble.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_uint, C.c_uint, _dp, _up, _up,
                                   C.c_void_p, C.c_void_p, C.c_double, _dp, C.c_uint, C.c_uint,
                                   C.c_void_p, C.c_size_t, _dp, C.c_int]
        L.orc_gauss.restype = C.c_int
        L.orc_gauss.argtypes = [C.c_uint, _dp, _dp]
        L.orc_gmres.restype = C.c_int
        L.orc_gmres.argtypes = [C.c_uint, C.c_uint, C.c_double, C.c_uint, _dp, _dp, C.c_void_p,
                                C.c_void_p, C.c_int, C.POINTER(C.c_uint)]
        L.orc_field_points.restype = None
        L.orc_field_points.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, C.c_uint, _dp,
                                       _dp, C.c_int]
        L.orc_potential.restype = None
        L.orc_potential.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, _dp, _dp]
        L.orc_forceMST.restype = C.c_int
        L.orc_forceMST.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_double,
                                   _dp, _dp, _dp, _dp, C.c_int]
        L.orc_node_normal.restype = None
        L.orc_node_normal.argtypes = [C.c_int, C.c_uint, _dp, _up, C.c_uint, _dp]
        for nm in ("orc_intG",):
            getattr(L, nm).argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_intH.argtypes = [C.c_int, C.c_uint, _dp, _dp, _dp, _dp]
        L.orc_intSingularG.argtypes = [C.c_int, C.c_uint, _dp, _dp, _dp]
        L.orc_intSingularH.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _dp, _dp, _dp]
        L.orc_interface_coeffs.argtypes = [C.c_uint, C.c_void_p, C.c_void_p, C.c_double, _dp, _dp]
        L.orc_matvec_rows.restype = None
        L.orc_matvec_rows.argtypes = [C.c_uint, C.c_void_p, _dp, _dp, C.c_uint, C.c_uint, C.c_int]
        # the quad8 extension (oracle/port/quad8.c)
        L.orc_q8_assemble.restype = C.c_int
        L.orc_q8_assemble.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_uint, _dp, _up, _up, C.c_void_p,
                                      C.c_void_p, C.c_double, _dp, C.c_void_p, C.c_size_t, _dp]
        L.orc_q8_field.restype = None
        L.orc_q8_field.argtypes = [C.c_uint, C.c_uint, _dp, _up, _dp, _dp, _dp]
        L.orc_q8_potential.restype = None
        L.orc_q8_potential.argtypes = [C.c_uint, C.c_uint, _dp, _up, _dp, _dp, _dp]
        L.orc_q8_forceMST.restype = None
        L.orc_q8_forceMST.argtypes = [C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_double, _dp, _dp, _dp, _dp]
        L.orc_q8_node_normal.restype = None
        L.orc_q8_node_normal.argtypes = [C.c_uint, _dp, _up, C.c_uint, _dp]

    # -- assembly -------------------------------------------------------
    def assemble(self, sc, full: bool = False, rows=None, nthreads: int = 1):
        """Returns (A, B): A is N x 2N (compact) or 2N x 2N (full); with
        `rows` = (r0, r1) only those rows are formed (others stay zero)."""
        N = sc.N
        A = np.zeros((2 * N if full else N, 2 * N))
        B = np.zeros(2 * N)
        r0, r1 = rows if rows is not None else (0, N)
        ifc = _u(sc.ifaces)
        mat = _f(sc.mat)
        if sc.nen == 8:
            rc = self.lib.orc_q8_assemble(int(full), N, sc.E, sc.n_if, _f(sc.nodes), _u(sc.elems),
                                          _u(sc.bctype), ifc.ctypes.data if sc.n_if else None,
                                          mat.ctypes.data, sc.freq, _f(sc.mbc), A.ctypes.data, 2 * N, B)
            if rc:
                raise ValueError("boundary type other than 0, 1, 6 in the scene")
            return A, B
        rc = self.lib.orc_assemble(sc.nen, int(full), N, sc.E, sc.n_if, _f(sc.nodes), _u(sc.elems),
                                   _u(sc.bctype), ifc.ctypes.data if sc.n_if else None,
                                   mat.ctypes.data, sc.freq, _f(sc.mbc), r0, r1,
                                   A.ctypes.data, 2 * N, B, nthreads)
        if rc:
            raise ValueError("boundary type other than 0, 1, 6 in the scene")
        return A, B

    def interface_coeffs(self, sc):
        a = np.zeros(max(sc.n_if, 1))
        b = np.zeros(max(sc.n_if, 1))
        ifc = _u(sc.ifaces)
        mat = _f(sc.mat)
        self.lib.orc_interface_coeffs(sc.n_if, ifc.ctypes.data, mat.ctypes.data, sc.freq, a, b)
        return a[:sc.n_if], b[:sc.n_if]

    # -- solvers --------------------------------------------------------
    def gauss(self, A, b):
        A = _f(A).copy()
        x = _f(b).copy()
        rc = self.lib.orc_gauss(A.shape[0], A, x)
        if rc:
            raise np.linalg.LinAlgError("singular pivot")
        return x

    def gmres(self, A, B, tol=1e-6, max_iters=600, precond=1, x0=None, nthreads=1,
              log_path=None):
        """Returns (x, iters, status); A (N x 2N) and B are not modified."""
        A = _f(A).copy()
        x = _f(B).copy()
        it = C.c_uint(0)
        x0a = _f(x0) if x0 is not None else None
        libc = C.CDLL(None)
        libc.fopen.restype = C.c_void_p
        libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
        libc.fclose.argtypes = [C.c_void_p]
        fp = libc.fopen(log_path.encode(), b"w") if log_path else None
        st = self.lib.orc_gmres(A.shape[0], precond, tol, max_iters, A, x,
                                x0a.ctypes.data if x0a is not None else None, fp, nthreads,
                                C.byref(it))
        if fp:
            libc.fclose(fp)
        return x, it.value, st

    # -- post-processing -------------------------------------------------
    def field(self, sc, vB, pts, nthreads=1):
        pts = _f(np.atleast_2d(pts))
        out = np.zeros((pts.shape[0], 6))
        if sc.nen == 8:
            for i in range(pts.shape[0]):
                r = np.zeros(6)
                self.lib.orc_q8_field(sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB), _f(pts[i]), r)
                out[i] = r
            return out
        self.lib.orc_field_points(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB),
                                  pts.shape[0], pts, out, nthreads)
        return out

    def potential(self, sc, vB, pts):
        pts = _f(np.atleast_2d(pts))
        out = np.zeros((pts.shape[0], 2))
        for i in range(pts.shape[0]):
            r = np.zeros(2)
            if sc.nen == 8:
                self.lib.orc_q8_potential(sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB), _f(pts[i]), r)
                out[i] = r
                continue
            self.lib.orc_potential(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB),
                                   _f(pts[i]), r)
            out[i] = r
        return out

    def force_mst(self, sc, vB, eps=None, nthreads=1):
        eps = sc.eps_medium if eps is None else eps
        Fce = np.zeros((sc.E, 3))
        Xce = np.zeros((sc.E, 3))
        Fcm = np.zeros(3)
        Xcm = np.zeros(3)
        if sc.nen == 8:
            self.lib.orc_q8_forceMST(sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _u(sc.bctype), _f(vB), eps,
                                     Fce, Xce, Fcm, Xcm)
            return Fce, Xce, Fcm, Xcm
        self.lib.orc_forceMST(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _u(sc.bctype),
                              _f(vB), eps, Fce, Xce, Fcm, Xcm, nthreads)
        return Fce, Xce, Fcm, Xcm

    def node_normal(self, sc, node0):
        n = np.zeros(3)
        if sc.nen == 8:
            self.lib.orc_q8_node_normal(sc.E, _f(sc.nodes), _u(sc.elems), node0 + 1, n)
            return n
        self.lib.orc_node_normal(sc.nen, sc.E, _f(sc.nodes), _u(sc.elems), node0 + 1, n)
        return n

    def integral(self, which, nen, X, xe, flag=0, sin=0, normal=(0.0, 0.0, 1.0)):
        X = _f(X)
        out = np.zeros(18)
        xe = _f(xe)
        nrm = _f(normal)
        if which == "G":
            self.lib.orc_intG(nen, X, xe, out)
        elif which == "H":
            self.lib.orc_intH(nen, flag, X, xe, out, nrm)
        elif which == "SG":
            self.lib.orc_intSingularG(nen, sin, X, xe, out)
        else:
            self.lib.orc_intSingularH(nen, flag, sin, X, xe, out, nrm)
        return out[: (3 * nen if flag else nen)]


class Ref:
    """The unmodified reference, through oracle/ref_harness.c."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            if build_ref() is None:
                raise FileNotFoundError("reference sources not available")
        self.workdir = tempfile.mkdtemp(prefix="dsref-")
        with _in_dir(self.workdir):
            L = C.CDLL(path)
        self.lib = L
        L.ref_assemble.restype = C.c_int
        L.ref_assemble.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_uint, C.c_uint, _dp, _up, _up,
                                   C.c_void_p, C.c_void_p, C.c_double, _dp, _dp, _dp]
        L.ref_gauss.argtypes = [C.c_uint, _dp, _dp]
        L.ref_gmres.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _dp]
        L.ref_field.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, _dp, _dp]
        L.ref_potential.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, _dp, _dp]
        L.ref_forceMST.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _up, _dp, C.c_double,
                                   _dp, _dp, _dp, _dp]
        L.ref_int.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_uint, _dp, _dp, _dp, _dp]
        L.ref_node_normal.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, C.c_uint, _dp]
        L.ref_set_sizes.argtypes = [C.c_uint, C.c_uint, C.c_uint]
        L.ref_forceMultipole.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, C.c_uint, C.c_double,
                                         _dp, _dp, C.c_double, _dp]
        L.ref_forceEllipsoid.argtypes = [C.c_int, C.c_uint, C.c_uint, _dp, _up, _dp, C.c_uint, _dp, _dp,
                                         _dp, C.c_double, _dp]

    def assemble(self, sc, full=False):
        N = sc.N
        A = np.zeros((2 * N if full else N, 2 * N))
        B = np.zeros(2 * N)
        ifc = _u(sc.ifaces)
        mat = _f(sc.mat)
        with _in_dir(self.workdir):
            self.lib.ref_assemble(sc.nen, int(full), N, sc.E, sc.n_if, _f(sc.nodes), _u(sc.elems),
                                  _u(sc.bctype), ifc.ctypes.data if sc.n_if else None,
                                  mat.ctypes.data, sc.freq, _f(sc.mbc), A, B)
        return A, B

    def gauss(self, A, b):
        A = _f(A).copy()
        x = _f(b).copy()
        with _in_dir(self.workdir):
            self.lib.ref_gauss(A.shape[0], A, x)
        return x

    def gmres(self, A, B, tight=False, precond=1):
        """Returns (x, gmres.log text).  tight selects the copy built with
        TOLERANCE 1e-10."""
        A = _f(A).copy()
        x = _f(B).copy()
        with _in_dir(self.workdir):
            self.lib.ref_gmres(int(tight), precond, A.shape[0], A, x)
            log = open("gmres.log").read()
        return x, log

    def field(self, sc, vB, pts):
        pts = _f(np.atleast_2d(pts))
        out = np.zeros((pts.shape[0], 6))
        for i in range(pts.shape[0]):
            r = np.zeros(6)
            self.lib.ref_field(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB), _f(pts[i]), r)
            out[i] = r
        return out

    def potential(self, sc, vB, pts):
        pts = _f(np.atleast_2d(pts))
        out = np.zeros((pts.shape[0], 2))
        for i in range(pts.shape[0]):
            r = np.zeros(2)
            self.lib.ref_potential(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB),
                                   _f(pts[i]), r)
            out[i] = r
        return out

    def force_mst(self, sc, vB, eps=None):
        eps = sc.eps_medium if eps is None else eps
        Fce = np.zeros((sc.E, 3))
        Xce = np.zeros((sc.E, 3))
        Fcm = np.zeros(3)
        Xcm = np.zeros(3)
        self.lib.ref_forceMST(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _u(sc.bctype),
                              _f(vB), eps, Fce, Xce, Fcm, Xcm)
        return Fce, Xce, Fcm, Xcm

    def node_normal(self, sc, node0):
        n = np.zeros(3)
        self.lib.ref_node_normal(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), node0 + 1, n)
        return n

    def force_multipole(self, sc, vB, order, R, xeval):
        """forceMultipole_* at xeval (materials 1 and 2 of the scene)."""
        F = np.zeros(3)
        with _in_dir(self.workdir):
            self.lib.ref_forceMultipole(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB), order, R,
                                        _f(xeval), _f(sc.mat[:2]), sc.freq, F)
        return F

    def force_ellipsoid(self, sc, vB, analysis, axis, xeval):
        """forceEllipsoid_* (analysis 10 or 11) at xeval."""
        F = np.zeros(3)
        with _in_dir(self.workdir):
            self.lib.ref_forceEllipsoid(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB), analysis,
                                        _f(axis), _f(xeval), _f(sc.mat[:2]), sc.freq, F)
        return F

    def integral(self, which, nen, X, xe, flag=0, sin=0, normal=(0.0, 0.0, 1.0)):
        code = {"G": 0, "H": 1, "SG": 2, "SH": 3}[which]
        out = np.zeros(18)
        self.lib.ref_int(code, nen, flag, sin, _f(X).ravel(), _f(xe), out, _f(normal))
        return out[: (3 * nen if flag else nen)]
