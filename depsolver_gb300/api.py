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


def row_pointers(arr: np.ndarray):
    """The reference's row-pointer view (double** / unsigned**) of a
    C-contiguous 2-D array, for the drop-in entry points; the array must
    outlive the view."""
    T = C.c_double if arr.dtype == np.float64 else C.c_uint
    ptrs = (C.POINTER(T) * arr.shape[0])()
    base = arr.ctypes.data
    step = arr.strides[0]
    for i in range(arr.shape[0]):
        ptrs[i] = C.cast(base + i * step, C.POINTER(T))
    return ptrs


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


GAUSS_MIXED = 0
GAUSS_FP64 = 1


def gauss_bksb(A: np.ndarray, B: np.ndarray, mode: int | None = None) -> np.ndarray:
    """Direct solve (gaussBksb).  mode: GAUSS_MIXED (tensor-core block LU
    with FP64 refinement, the library's default), GAUSS_FP64, or None (the
    current process-wide mode)."""
    L = _native.lib()
    A = _f(A)
    x = _f(B).copy()
    old = None
    if mode is not None:
        old = L.dsc_gauss_info(None, None, None, None)
        _native.check(L.dsc_set_gauss_mode(int(mode)))
    try:
        _native.check(L.dsc_gauss(A.shape[0], A, A.shape[1], x))
    finally:
        if old is not None:
            L.dsc_set_gauss_mode(old)
    return x


def set_host_direct(mode: int) -> None:
    """Host matrices read in place by the device where it can (mode 1, the
    default), the assembled rows also written in place (2), or every copy
    through pinned staging (0)."""
    _native.check(_native.lib().dsc_set_host_direct(int(mode)))


def gauss_info(times: bool = False):
    """(mode, refinement steps, relative residual, fell back to FP64) of the
    last direct solve; with times, also (factorisation ms, refinement ms)
    of its device work."""
    it = C.c_int(0)
    rr = C.c_double(0.0)
    fb = C.c_int(0)
    ms = np.zeros(2)
    mode = _native.lib().dsc_gauss_info(C.byref(it), C.byref(rr), C.byref(fb), ms.ctypes.data)
    out = (mode, it.value, rr.value, bool(fb.value))
    return out + (float(ms[0]), float(ms[1])) if times else out


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


def force_multipole(sc: Scene, vB: np.ndarray, pts, order: int, R: float) -> np.ndarray:
    """forceMultipole_* at each point (npts x 3): sphere of radius R,
    materials 1 (medium) and 2 (particle) of the scene, its frequency."""
    pts = _f(np.atleast_2d(pts))
    F = np.zeros((pts.shape[0], 3))
    _native.check(_native.lib().dsc_force_multipole(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB),
                                                    pts.shape[0], pts, order, float(R), _f(sc.mat[:2]).ravel(),
                                                    sc.freq, F))
    return F


def force_ellipsoid(sc: Scene, vB: np.ndarray, pts, analysis: int, axis) -> np.ndarray:
    """forceEllipsoid_* (analysis 10 or 11) at each point (npts x 3)."""
    pts = _f(np.atleast_2d(pts))
    F = np.zeros((pts.shape[0], 3))
    ax = _f(axis)
    _native.check(_native.lib().dsc_force_ellipsoid(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _f(vB),
                                                    pts.shape[0], pts, analysis, ax.ctypes.data,
                                                    _f(sc.mat[:2]).ravel(), sc.freq, F))
    return F


def depolarization(axis) -> np.ndarray:
    """Depolarisation factors of an ellipsoid of semi-axes `axis`."""
    Ld = np.zeros(3)
    _native.check(_native.lib().dsc_depolarization(_f(axis), Ld))
    return Ld


# ------------------------------------------------------------------ sweeps

MODE_FP64 = 1
MODE_MIXED = 2
ERR_NOCONVERGE = 5
RESIDUAL_AUTO = 0
RESIDUAL_DIGITS = 1
RESIDUAL_FP64 = 2
# outcome of one system of a sweep (Session.status)
SYS_CONVERGED = 0
SYS_CAPPED = 1
SYS_STAGNATED = 2
# arithmetic of the mixed mode's regular pairs (Session.set_mixed_assembly)
ASM_DF32 = 1
ASM_FP32 = 2
TIMER_NAMES = ("asm_regular", "asm_fixup", "asm_singular", "gemv_K64", "gemm_K", "field", "mst",
               "residual_fp64", "krylov", "gram_schmidt", "convert_K", "precond_build",
               "precond_apply")


def set_autotune(on: bool):
    """Split-count autotuner of the mixed sweep's tensor-core product."""
    _native.check(_native.lib().dsc_set_autotune(int(on)))


def autotune_table():
    """[(N, columns, splits)] of the sizes tuned so far in this process."""
    L = _native.lib()
    n = L.dsc_autotune_table(None, 0)
    rows = np.zeros((max(n, 1), 3), dtype=np.int32)
    L.dsc_autotune_table(rows.ctypes.data, n)
    return [tuple(int(v) for v in r) for r in rows[:n]]


class Session:
    """A geometry kept on the GPU (geometric matrix assembled once) for
    frequency sweeps; wraps dsc_session_* of the C ABI."""

    def __init__(self, sc: Scene):
        L = _native.lib()
        self._L = L
        self.scene = sc
        h = C.c_void_p()
        ifc = _u(sc.ifaces)
        _native.check(L.dsc_session_create(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems),
                                           _u(sc.bctype), _f(sc.mbc), sc.n_if,
                                           ifc.ctypes.data if sc.n_if else None,
                                           sc.mat.shape[0], _f(sc.mat), C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            self._L.dsc_session_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def assemble(self, mode: int = MODE_FP64):
        """Assemble K now: MODE_FP64 in FP64, MODE_MIXED with the regular
        pairs in the arithmetic set_mixed_assembly chose (FP32 by default),
        the singular pairs in double-FP32, and the tensor cores' fp16
        pair."""
        _native.check(self._L.dsc_session_assemble(self._h, mode))

    def geometric_matrix(self, mode: int = MODE_FP64) -> np.ndarray:
        """K (N x N, row i = collocation node, column c = node) as assembled
        for `mode`."""
        N = self.scene.N
        Kt = np.empty((N, N))
        _native.check(self._L.dsc_session_geometric_matrix(self._h, mode, Kt, N))
        return Kt.T

    def stream_handle(self) -> int:
        """cudaStream_t of the session (for torch.cuda.ExternalStream)."""
        return int(self._L.dsc_session_stream(self._h) or 0)

    def set_timing(self, on: bool):
        _native.check(self._L.dsc_session_set_timing(self._h, int(on)))

    def set_mixed_assembly(self, prec: int):
        """Mixed mode's regular pairs: ASM_FP32 (default; ~1e-7 per entry)
        or ASM_DF32 (double-FP32, within ~1e-13 of FP64)."""
        _native.check(self._L.dsc_session_set_mixed_assembly(self._h, int(prec)))

    def set_field_tensor(self, on: bool):
        """Mixed mode: the batched field's far pairs on the tensor cores
        (default on) or on the FP32 pipes."""
        _native.check(self._L.dsc_session_set_field_tensor(self._h, int(on)))

    def set_fp64_jacobi(self, full: bool):
        """FP64 mode: also scale the imaginary right-hand side in the Jacobi
        step (the reference scales only the real half; they differ for
        complex boundary values)."""
        _native.check(self._L.dsc_session_set_fp64_jacobi(self._h, int(full)))

    def set_residual(self, how: int):
        """Mixed mode's first FP64 residual: RESIDUAL_AUTO, RESIDUAL_DIGITS
        (tensor-core digit products) or RESIDUAL_FP64 (FP64 GEMV)."""
        _native.check(self._L.dsc_session_set_residual(self._h, int(how)))

    def set_preconditioner(self, on: bool):
        """Mixed mode: the conductor-block right preconditioner (default on)."""
        _native.check(self._L.dsc_session_set_preconditioner(self._h, int(on)))

    def preconditioner_blocks(self):
        """Row counts of the preconditioner's blocks (one per electrode)."""
        n = self._L.dsc_session_preconditioner_blocks(self._h, None, 0)
        rows = np.zeros(max(n, 1), dtype=np.int32)
        self._L.dsc_session_preconditioner_blocks(self._h, rows.ctypes.data, n)
        return rows[:n].tolist()

    def timing(self):
        """{class: (ms, timed scopes, algorithmic work)} since the last call
        (work units per class in dsc_session_timing's header comment)."""
        ms = np.zeros(len(TIMER_NAMES))
        cnt = np.zeros(len(TIMER_NAMES), dtype=np.int32)
        wk = np.zeros(len(TIMER_NAMES))
        _native.check(self._L.dsc_session_timing(self._h, ms.ctypes.data, cnt.ctypes.data,
                                                 wk.ctypes.data, len(TIMER_NAMES)))
        return {n: (float(ms[k]), int(cnt[k]), float(wk[k])) for k, n in enumerate(TIMER_NAMES)}

    def solve(self, freqs, mode: int = MODE_MIXED, tol: float = 1e-10, max_iters: int = 600,
              want_sigma: bool = False, partial: bool = False):
        """Returns (forces (F x 9): Fcm, Xcm, sum|Fce|; iterations; sigma or None).

        A system that does not converge raises DscError (DSC_ERR_NOCONVERGE)
        unless partial is true; then its forces and sigma are NaN and
        :meth:`status` gives each system's outcome (SYS_*)."""
        fr = _f(np.atleast_1d(freqs))
        F = fr.shape[0]
        forces = np.zeros((F, 9))
        its = np.zeros(F, dtype=np.uint32)
        sig = np.zeros((F, 2 * self.scene.N)) if want_sigma else None
        rc = self._L.dsc_session_solve(self._h, mode, F, fr, tol, max_iters,
                                       sig.ctypes.data if sig is not None else None,
                                       forces.ctypes.data, its.ctypes.data)
        if not (partial and rc == ERR_NOCONVERGE):
            _native.check(rc)
        return forces, its, sig

    def particles(self) -> np.ndarray:
        """Per-particle results of the last solve: (F, P, 12) -- force[3],
        centre[3], sum|Fce|[3], torque[3] about the centre."""
        n = self._L.dsc_session_status(self._h, None, 0)
        P = self._L.dsc_session_particles(self._h, None, 0)
        out = np.zeros((n, P, 12))
        self._L.dsc_session_particles(self._h, out.ctypes.data, n)
        return out

    def status(self) -> np.ndarray:
        """Outcome of each system of the last solve: SYS_CONVERGED,
        SYS_CAPPED (max_iters reached) or SYS_STAGNATED."""
        n = self._L.dsc_session_status(self._h, None, 0)
        st = np.zeros(max(n, 1), dtype=np.int32)
        self._L.dsc_session_status(self._h, st.ctypes.data, n)
        return st[:n]


def sweep(sc: Scene, freqs, mode: int = MODE_MIXED, tol: float = 1e-10, max_iters: int = 600,
          want_sigma: bool = True):
    """One call from host arrays to forces (and sigma): dsc_sweep."""
    L = _native.lib()
    fr = _f(np.atleast_1d(freqs))
    F = fr.shape[0]
    forces = np.zeros((F, 9))
    its = np.zeros(F, dtype=np.uint32)
    sig = np.zeros((F, 2 * sc.N)) if want_sigma else None
    ifc = _u(sc.ifaces)
    _native.check(L.dsc_sweep(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), _u(sc.bctype),
                              _f(sc.mbc), sc.n_if, ifc.ctypes.data if sc.n_if else None,
                              sc.mat.shape[0], _f(sc.mat), mode, F, fr, tol, max_iters,
                              sig.ctypes.data if sig is not None else None, forces.ctypes.data,
                              its.ctypes.data))
    return forces, its, sig


class PositionSweep:
    """Particle-position sweeps (dsc_positions_*): a fixed part of the scene
    (electrodes) and particle meshes of any size, solved at many positions
    and frequencies per call -- the work of many depSolver-sft runs
    (src/depSolver-shift.c:129-133,212-217)."""

    def __init__(self, fixed: Scene):
        L = _native.lib()
        self._L = L
        self.fixed = fixed
        self.sizes = []
        h = C.c_void_p()
        ifc = _u(fixed.ifaces)
        _native.check(L.dsc_positions_create(fixed.nen, fixed.N, fixed.E, _f(fixed.nodes),
                                             _u(fixed.elems), _u(fixed.bctype), _f(fixed.mbc),
                                             fixed.n_if, ifc.ctypes.data if fixed.n_if else None,
                                             fixed.mat.shape[0], _f(fixed.mat), C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            self._L.dsc_positions_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_particle(self, nodes, elems0, iface: int = 1) -> int:
        """A particle mesh: nodes about its own origin, 0-based elements."""
        nodes = _f(nodes)
        el = _u(np.asarray(elems0) + 1)
        r = self._L.dsc_positions_add_particle(self._h, nodes.shape[0], el.shape[0], nodes, el, iface)
        if r < 0:
            _native.check(-r)
        self.sizes.append(nodes.shape[0])
        return r

    def set_workers(self, n: int):
        _native.check(self._L.dsc_positions_set_workers(self._h, int(n)))

    def set_mixed_assembly(self, prec: int):
        _native.check(self._L.dsc_positions_set_mixed_assembly(self._h, int(prec)))

    def set_timing(self, on: bool):
        _native.check(self._L.dsc_positions_set_timing(self._h, int(on)))

    def timing(self):
        ms = np.zeros(len(TIMER_NAMES))
        cnt = np.zeros(len(TIMER_NAMES), dtype=np.int32)
        wk = np.zeros(len(TIMER_NAMES))
        _native.check(self._L.dsc_positions_timing(self._h, ms.ctypes.data, cnt.ctypes.data,
                                                   wk.ctypes.data, len(TIMER_NAMES)))
        return {n: (float(ms[k]), int(cnt[k]), float(wk[k])) for k, n in enumerate(TIMER_NAMES)}

    def inversions(self) -> int:
        return int(self._L.dsc_positions_inversions(self._h))

    def solve(self, particles, centres, freqs, tol: float = 1e-10, max_iters: int = 600,
              want_sigma: bool = False, partial: bool = False):
        """Returns a dict: forces (P x F x 9), iters (P x F), status (P x F),
        crossover_hz (P), sigma (list of F x 2N_q arrays, or None)."""
        tp = _u(np.atleast_1d(particles))
        ce = _f(np.asarray(centres, dtype=np.float64).reshape(-1, 3))
        fr = _f(np.atleast_1d(freqs))
        P, F = tp.shape[0], fr.shape[0]
        forces = np.zeros((P, F, 9))
        its = np.zeros((P, F), dtype=np.uint32)
        st = np.zeros((P, F), dtype=np.int32)
        xo = np.zeros(P)
        Ns = [self.fixed.N + self.sizes[t] for t in tp]
        sig = np.zeros(sum(2 * n * F for n in Ns)) if want_sigma else None
        rc = self._L.dsc_positions_solve(self._h, P, tp, ce, F, fr, tol, max_iters, forces,
                                         its.ctypes.data, st.ctypes.data, xo.ctypes.data,
                                         sig.ctypes.data if sig is not None else None)
        if not (partial and rc == ERR_NOCONVERGE):
            _native.check(rc)
        sigmas = None
        if sig is not None:
            sigmas, o = [], 0
            for n in Ns:
                sigmas.append(sig[o:o + 2 * n * F].reshape(F, 2 * n))
                o += 2 * n * F
        return {"forces": forces, "iters": its, "status": st, "crossover_hz": xo, "sigma": sigmas}


def read_bem(directory: str) -> dict:
    """The reference's input deck through the library's reader
    (dsc_bem_read): a dict of the scene arrays (as Scene holds them) and
    the deck's analysis settings."""
    L = _native.lib()
    h = C.c_void_p()
    _native.check(L.dsc_bem_read(directory.encode(), C.byref(h)))
    try:
        nen, an, gm, rp = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        N, E, nm, ni, pc, nin, nint, nfp, pn = (C.c_uint() for _ in range(9))
        fr = C.c_double()
        dr = np.zeros(3)
        ax = np.zeros(3)
        refs = [nen, N, E, nm, ni, fr, an, gm, pc, nin, nint, nfp, rp, pn]
        _native.check(L.dsc_bem_info(h, *[C.addressof(r) for r in refs], dr.ctypes.data, ax.ctypes.data))
        out = {"nen": nen.value, "nodes": np.zeros((N.value, 3)),
               "elems": np.zeros((E.value, nen.value), dtype=np.uint32),
               "bctype": np.zeros(2 * N.value, dtype=np.uint32), "mbc": np.zeros((2 * N.value, 3)),
               "mat": np.zeros((nm.value, 2)), "ifaces": np.zeros((ni.value, 2), dtype=np.uint32),
               "internal": np.zeros((nint.value, 3)), "force_points": np.zeros((nfp.value, 3)),
               "freq": fr.value, "analysis": an.value, "gmres": bool(gm.value), "precond": pc.value,
               "ninit": nin.value, "reposition": bool(rp.value), "pnodes": pn.value, "dr": dr,
               "axis": ax}
        _native.check(L.dsc_bem_arrays(h, *[out[k].ctypes.data for k in
                                            ("nodes", "elems", "bctype", "mbc", "mat", "ifaces",
                                             "internal", "force_points")]))
        return out
    finally:
        L.dsc_bem_free(h)


def node_normals(sc: Scene) -> np.ndarray:
    """Averaged unit normal at every node (N x 3): dsc_node_normals."""
    out = np.zeros((sc.N, 3))
    _native.check(_native.lib().dsc_node_normals(sc.nen, sc.N, sc.E, _f(sc.nodes), _u(sc.elems), out))
    return out
