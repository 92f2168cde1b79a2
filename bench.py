"""Benchmark: DEP solves/s on the 12k-node scene (level-4 sphere between
30 x 30-cell plates, tria6, N = 17684, E = 8720).

A step is one batch: assemble the geometric matrix of the scene (regular
pairs in FP32 from centroid-relative offsets: the far-field assembly in
FP32; singular pairs in double-FP32, about 1e-13 of FP64) and
solve a 64-frequency sweep (1 kHz .. 100 MHz, log-spaced) to a relative
residual of 1e-10 with the mixed-precision batched path, then the
Maxwell-stress DEP force of every system.  value = systems solved per
second (inputs resident in GPU memory).  e2e = the same through the C ABI
from host arrays (dsc_sweep: mesh in, nodal solution and forces out).

Also measured and reported: the plain FP64 GPU path (the reference's GMRES
in FP64, one frequency per solve, assembly included), the force error of
the mixed path against an FP64 solve, and a CPU baseline (the C
restatement of the reference, all host cores).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DEP solves/s at 12k nodes: mixed-prec+batched vs FP64 GPU, force err ≤1e-6"
UNIT = "solves/s"
NFREQ = 64
TOL = 1e-10
FREQS = np.logspace(3.0, 8.0, NFREQ)


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


# ------------------------------------------------------------------ roofline
# Per kernel class: the bound, the unit, the scale from the library's work
# count to that unit, the peak and where the peak comes from.  The
# tensor-core product (3xFP16, kind::f16 at the bf16 rate) is HBM-bound: its
# work counter (flops of the three products) converts to the algorithmic
# bytes of a product -- the fp16 pair of K (4 N^2), the operand pairs and the
# FP32 result (8 F N each) -- and its tensor-pipe fraction is reported
# beside.  The mixed mode's regular-pair assembly runs in FP32 on the FP32
# pipes (packed FP32x2): it is reported as (row, element) pairs per second with no
# single-number peak (its FP32-pipe utilisation is in
# profiles/asm_regular_mid.md).


def gemm_bytes_per_flop(N, F=None):
    F = F or NFREQ
    return (4.0 * N * N + 16.0 * F * N) / (12.0 * F * N * N)


def roofline(timing, N, E):
    P = peaks()
    hbm = P.get("hbm_gbs")
    bf16 = P.get("bf16_tflops")
    src = "MEASURED_PEAKS.json" if P else "fallback"
    if not hbm:
        hbm, bf16 = 6800.0, 1900.0
    models = {
        "gemm_K": ("hbm", "GB/s", gemm_bytes_per_flop(N) * 1e-9, hbm,
                   f"{src} hbm_gbs, of measured"),
        "gram_schmidt": ("hbm", "GB/s", 1e-9, hbm, f"{src} hbm_gbs, of measured"),
        "gemv_K64": ("hbm", "GB/s", 1e-9, hbm, f"{src} hbm_gbs, of measured"),
        "asm_regular": ("fp32-pipe", "Gpairs/s", 1e-9, None,
                        "no single-number peak: FP32 and integer issue on the FP32 pipes"),
    }
    out = {}
    for k, (bound, unit, scale, peak, psrc) in models.items():
        ms, cnt, wk = timing.get(k, (0.0, 0, 0.0))
        if cnt and ms > 0 and wk > 0:
            ach = wk * scale / (ms / 1e3)
            out[k] = {"kernel": k, "bound": bound, "achieved": ach, "peak": peak, "unit": unit,
                      "frac": ach / peak if peak else None, "traffic": TRAFFIC.get(k),
                      "peak_source": psrc,
                      "ms": ms, "scopes": cnt}
            if k == "gemm_K":
                tf = wk * 1e-12 / (ms / 1e3)
                out[k]["tensor"] = {"achieved_tflops": tf, "peak_tflops": bf16,
                                    "frac": tf / bf16 if bf16 else None,
                                    "peak_source": f"{src} bf16_tflops (fp16 issues at the same rate)"}
    main = [k for k in out if out[k]["bound"] in ("hbm", "tensor")]
    dom = max(main, key=lambda k: out[k]["ms"]) if main else None
    return (out[dom] if dom else None), out


# DRAM bytes per timed scope of a class, from one ncu capture of the same
# workload (dram__bytes_read.sum + dram__bytes_write.sum); None where not
# captured.  The summaries behind these numbers are under profiles/.
TRAFFIC = {
    # k_tc_gemm3<3> at N = 17684, Nc = 128: 1.28 GB read + 93.4 MB written
    # (profiles/tc_gemm3_f16_cfg1.md)
    "gemm_K": 1373360000,
}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline
def cpu_baseline(sc, nthreads: int, sample_div: int = 8, full_first: bool = True):
    """The C restatement of the reference (oracle/port) on the host cores.

    One full solve of one frequency (assembly, GMRES at the reference's
    compiled tolerance 1e-6, MST force) gives the reference's iteration
    count; the timed sample is 1/sample_div of the assembly rows, the same
    rows' share of every GMRES matrix-vector product (times that count) and
    1/sample_div of the particle-node fields, scaled to one full solve;
    Gram-Schmidt and the MST integral are timed in full."""
    from oracle.oracle import Port
    P = Port()
    N = sc.N
    info = {}
    if full_first:
        t0 = time.perf_counter()
        A, B = P.assemble(sc, nthreads=nthreads)
        t1 = time.perf_counter()
        x, it, st = P.gmres(A, B, nthreads=nthreads)
        t2 = time.perf_counter()
        F = P.force_mst(sc, x, nthreads=nthreads)
        t3 = time.perf_counter()
        info = {"full_solve_s": t3 - t0, "assembly_s": t1 - t0, "gmres_s": t2 - t1,
                "force_s": t3 - t2, "gmres_iters": int(it), "Fcm": F[2].tolist()}
        del A
    it = info.get("gmres_iters", 40)
    # sampled step: one contiguous chunk of rows per thread, evenly spread,
    # 1/sample_div of all rows, assembled concurrently (ctypes releases the
    # GIL, each call single-threaded)
    per = max(1, N // sample_div // nthreads)
    starts = np.linspace(0, N - per, nthreads).astype(int)
    Ab = np.zeros((nthreads * per, 2 * N))
    Bbs = [np.zeros(2 * N) for _ in range(nthreads)]
    nodes = np.ascontiguousarray(sc.nodes)
    elems = np.ascontiguousarray(sc.elems, np.uint32)
    bct = np.ascontiguousarray(sc.bctype, np.uint32)
    ifc = np.ascontiguousarray(sc.ifaces, np.uint32)
    mat = np.ascontiguousarray(sc.mat)
    mbc = np.ascontiguousarray(sc.mbc)

    def asm(t):
        s0 = int(starts[t])
        # rows s0..s0+per land at Ab[t*per ...]: row i at base + i * 2N
        base = Ab.ctypes.data + (t * per - s0) * 2 * N * 8
        P.lib.orc_assemble(sc.nen, 0, N, sc.E, sc.n_if, nodes, elems, bct, ifc.ctypes.data,
                           mat.ctypes.data, sc.freq, mbc, s0, s0 + per, base, 2 * N, Bbs[t], 1)

    ths = [threading.Thread(target=asm, args=(t,)) for t in range(nthreads)]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    t_asm = time.perf_counter() - t0
    blocks = [None] * nthreads
    xv = np.random.default_rng(0).standard_normal(2 * N)
    y = np.zeros(2 * N)
    t0 = time.perf_counter()
    P.lib.orc_matvec_rows(N, Ab.ctypes.data, xv, y, 0, nthreads * per, nthreads)
    t_mv = time.perf_counter() - t0
    chunk = per
    # Gram-Schmidt of an iteration with half the final Krylov dimension, in full
    V = np.random.default_rng(1).standard_normal((max(1, it // 2), 2 * N))
    t0 = time.perf_counter()
    w = xv.copy()
    for v in V:
        w -= (v @ w) * v
    t_mgs = time.perf_counter() - t0
    p0, p1 = sc.particles[0][0], sc.particles[-1][1]
    pts = sc.nodes[p0:p1][:: sample_div]
    sol = np.zeros(2 * N)
    sol[:N] = 1.0
    t0 = time.perf_counter()
    P.field(sc, sol, pts, nthreads=nthreads)
    t_field = time.perf_counter() - t0
    est = sample_div * (t_asm + it * t_mv + t_field) + it * t_mgs
    sample = (f"one full solve of one frequency (assembly, GMRES to 1e-6 in {it} iterations, "
              f"force) then a timed 1/{sample_div} sample: {len(blocks) * chunk} of {N} assembly rows, "
              f"their share of {it} matrix-vector products, {len(pts)} of {p1 - p0} particle-node "
              f"fields, scaled x{sample_div}; Gram-Schmidt timed in full")
    return {"value": 1.0 / est, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": sample, "est_solve_s": est, "parts_s": {"assembly": sample_div * t_asm,
            "gmres": it * (sample_div * t_mv + t_mgs), "field": sample_div * t_field},
            "full": info}


# ------------------------------------------------------------------ position sweep
NPOS = 128


def position_bench(args, with_cpu: bool):
    """The batched frequency and position sweep on the config-0 plates: 128
    seeded sphere centres (levels 2, 3, 4 drawn per position: N = 1524, 3444
    or 11124) x the 64 frequencies, every system to 1e-10, in one
    dsc_positions_solve call.  Timed by the host clock around the call with
    the device synchronised on both sides (the positions' kernels run on
    several streams); the systems' inputs are host arrays by construction
    (each position's mesh is built and uploaded inside the call), so the
    number is end to end."""
    import torch

    from depsolver_gb300 import api, scenes
    fixed = scenes.plates_only(10)
    lev, cen = scenes.cfg3_positions(NPOS)
    ps = api.PositionSweep(fixed)
    ps.set_workers(args.pos_workers)
    tid = {}
    for lv in (2, 3, 4):
        tid[lv] = ps.add_particle(*scenes.icosphere(lv, 1.0))
    tm = np.array([tid[int(v)] for v in lev], dtype=np.uint32)
    Ns = {lv: fixed.N + scenes.icosphere(lv, 1.0)[0].shape[0] for lv in (2, 3, 4)}
    # warm-up: a few positions of every size (grows the device memory pool)
    warm = [int(np.nonzero(lev == lv)[0][0]) for lv in (4, 3, 2)] * 2
    for _ in range(max(1, args.warmup - 2)):
        ps.solve(tm[warm], cen[warm], FREQS, tol=TOL)
    ps.set_timing(True)
    ps.timing()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = ps.solve(tm, cen, FREQS, tol=TOL)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    timing = ps.timing()
    nsys = NPOS * NFREQ
    value = nsys / wall
    # roofline of the dominant class: the library counts the flops of every
    # product (12 F N^2); a product moves 4 N^2 + 16 F N bytes, i.e.
    # 1/(3F) + 4/(3N) bytes per flop -- nearly independent of N, so the
    # positions' mean converts the summed flops to bytes
    P = peaks()
    hbm = P.get("hbm_gbs") or 6800.0
    src = "MEASURED_PEAKS.json hbm_gbs, of measured" if P else "fallback"
    ms, cnt, wk = timing["gemm_K"]
    byts = 0.0
    for lv, n in Ns.items():
        k = int((lev == lv).sum())
        byts += k * (4.0 * n * n + 16.0 * NFREQ * n) / (12.0 * NFREQ * n * n)
    bpf = byts / NPOS
    roof = None
    if cnt and ms > 0:
        ach = wk * bpf * 1e-9 / (ms / 1e3)
        roof = {"kernel": "gemm_K", "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "traffic": None, "peak_source": src, "ms": ms, "scopes": cnt,
                "note": "kernels of several positions overlap on the GPU: per-kernel times include "
                        "the sharing, so the fraction is a lower bound"}
    # accuracy: one position of every size against FP64 solves of the same
    # scene at 8 of the frequencies
    chk = np.linspace(0, NFREQ - 1, 8).astype(int)
    ferr, serr = [], []
    for lv in (2, 3, 4):
        q = int(np.nonzero(lev == lv)[0][0])
        sc = scenes.sphere_between_plates(lv, 10, center=tuple(cen[q]))
        s = api.Session(sc)
        f64, _, _ = s.solve(FREQS[chk], mode=api.MODE_FP64, tol=1e-12)
        s.close()
        for j, k in enumerate(chk):
            ferr.append(float(np.abs(r["forces"][q, k, :3] - f64[j, :3]).max() / f64[j, 6:9].sum()))
    xo = r["crossover_hz"]
    fin = np.isfinite(xo)
    out = {"workload": "cfg3: 128 seeded sphere centres (uniform in [-4,4]^2 x [-3,3]) between the "
                       "config-0 plates, sphere levels 2/3/4 drawn per position, x 64 frequencies "
                       "1 kHz..100 MHz, tol 1e-10",
           "value": value, "unit": UNIT, "systems": nsys, "wall_s": wall,
           "positions_per_level": {str(lv): int((lev == lv).sum()) for lv in (2, 3, 4)},
           "N_per_level": {str(lv): n for lv, n in Ns.items()},
           "workers": args.pos_workers, "conductor_inversions": ps.inversions(),
           "e2e": {"value": value, "unit": UNIT, "note": "the call takes host arrays; same number"},
           "roofline": roof,
           "force_err_vs_fp64_max": max(ferr), "force_err_checked": len(ferr),
           "inner_iterations_mean": float(r["iters"].mean()),
           "crossover": {"positions_with_sign_change": int(fin.sum()),
                         "median_hz": float(np.median(xo[fin])) if fin.any() else None,
                         "per_position_hz": [None if not np.isfinite(v) else float(v) for v in xo]},
           "kernels_ms": {k: v[0] for k, v in timing.items()}}
    if with_cpu:
        # the C restatement on the host cores, one position of each size
        # (a full solve at 1e-6 then a 1/8 row sample), weighted by the
        # positions per size
        est = 0.0
        for lv in (2, 3, 4):
            q = int(np.nonzero(lev == lv)[0][0])
            sc = scenes.sphere_between_plates(lv, 10, center=tuple(cen[q]))
            cb = cpu_baseline(sc, os.cpu_count() or 1)
            est += int((lev == lv).sum()) * cb["est_solve_s"]
        est /= NPOS
        out["cpu_baseline"] = {"value": 1.0 / est, "unit": UNIT, "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": "one position of each sphere level, one "
                               "frequency each (full solve at the reference's 1e-6, then a 1/8 row "
                               "sample scaled x8), weighted by the positions per level"}
    ps.close()
    return out


# ------------------------------------------------------------------ direct solve
def gauss_bench(with_cpu: bool):
    """gaussBksb through the C ABI (dsc_gauss: host matrix in, solution out)
    on the full 2N x 2N real form of two scenes: config 0 (2N = 3048) and the
    size of the reference's capacitor-1/quadratic Gauss run (two 25 x 25-cell
    plates, 2N = 10404; 371 s on one x86 core in the survey's re-run).  The
    tensor-core block LU with FP64 refinement against the FP64 LU; the
    factorisation's rate is (2/3) n^3 flops over its CUDA-event time."""
    from depsolver_gb300 import api, scenes
    P = peaks()
    bf16 = P.get("bf16_tflops") or 1900.0
    out = {}
    for name, sc in (("cfg0", scenes.cfg0(center=(0.0, 0.0, 1.0))), ("capacitor25", scenes.capacitor(25))):
        Af, Bf = api.electric_form(sc, full=True)
        n = Af.shape[0]
        api.gauss_bksb(Af, Bf, mode=api.GAUSS_MIXED)        # warm-up
        best, xm, inf = None, None, None
        for _ in range(3):
            t0 = time.perf_counter()
            xm = api.gauss_bksb(Af, Bf, mode=api.GAUSS_MIXED)
            dt = time.perf_counter() - t0
            if best is None or dt < best:
                best, inf = dt, api.gauss_info(times=True)
        t0 = time.perf_counter()
        x64 = api.gauss_bksb(Af, Bf, mode=api.GAUSS_FP64)
        t64 = time.perf_counter() - t0
        flops = 2.0 / 3.0 * n ** 3
        tf = flops / (inf[4] * 1e-3) * 1e-12 if inf[4] > 0 else None
        out[name] = {"unknowns": n, "e2e_s": best, "factor_ms": inf[4], "refine_ms": inf[5],
                     "refinements": inf[1], "rel_residual": inf[2], "fell_back_to_fp64": inf[3],
                     "fp64_lu_e2e_s": t64, "sol_rel_diff_vs_fp64_lu": float(np.abs(xm - x64).max() / np.abs(x64).max()),
                     "factor_tflops": tf, "factor_frac_of_bf16_peak": tf / bf16 if tf else None,
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops, of measured" if P else "fallback",
                     "speedup_vs_fp64_lu": t64 / best}
        if with_cpu and name == "cfg0":
            from oracle.oracle import Port
            t0 = time.perf_counter()
            Port().gauss(Af, Bf)
            tc = time.perf_counter() - t0
            out[name]["cpu_port_gauss_s"] = tc
            out[name]["cpu_cores"] = 1
        del Af
    out["cpu_note"] = ("cfg0: the C restatement's elimination (the reference's loop order) on one host "
                       "core; capacitor25: the survey's x86 re-run of the reference took 371 s")
    return out


# ------------------------------------------------------------------ multi-material trap
def trap_bench():
    """Config 2: four 4 x 4 pads (16 x 16 cells, phases 0/90/180/270 deg, 1 V,
    100 kHz) and four spheres of their own materials (levels 3/3/4/4):
    the mixed solve at 100 kHz against the FP64 path, with the force and
    torque of every particle."""
    import torch

    from depsolver_gb300 import api, scenes
    sc = scenes.quadrupole_trap()
    s = api.Session(sc)
    fm, itm, _ = s.solve([sc.freq], mode=api.MODE_MIXED, tol=TOL)   # assembles
    pm = s.particles()[0]
    t = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.assemble(api.MODE_MIXED)
        s.solve([sc.freq], mode=api.MODE_MIXED, tol=TOL)
        torch.cuda.synchronize()
        t.append(time.perf_counter() - t0)
    # the FP64 check with the imaginary right-hand side scaled too: the
    # pads' boundary values are complex, where the reference's Jacobi step
    # (which scales only the real half) solves a different system
    s.set_fp64_jacobi(True)
    f64, it64, _ = s.solve([sc.freq], mode=api.MODE_FP64, tol=1e-12)
    p64 = s.particles()[0]
    s.close()
    parts = []
    for k in range(pm.shape[0]):
        scale = p64[k, 6:9].sum()
        parts.append({"force": pm[k, :3].tolist(), "torque": pm[k, 9:12].tolist(), "centre": pm[k, 3:6].tolist(),
                      "force_err_vs_fp64": float(np.abs(pm[k, :3] - p64[k, :3]).max() / scale),
                      "torque_err_vs_fp64": float(np.abs(pm[k, 9:12] - p64[k, 9:12]).max() / scale)})
    return {"workload": "cfg2: quadrupole trap, 4 pads + 4 spheres (levels 3/3/4/4, own eps_r and sigma), "
                        "100 kHz, tol 1e-10", "N": sc.N, "E": sc.E,
            "s_per_solve": min(t), "inner_iterations": int(itm[0]), "fp64_gmres_iters": int(it64[0]),
            "particles": parts}


# ------------------------------------------------------------------ large scene
def large_bench():
    """Config 4: the castellated trap (two interdigitated combs of 10
    fingers, 8 x 32 cells each, and a chain of 8 level-4 spheres: N = 104036,
    E = 51200) at 1 MHz.  K in FP64 (87 GB) and its fp16 pair (43 GB) on the
    device; K's digits (173 GB) do not fit, so the first residual is an FP64
    GEMV.  Reported: the mixed solve (assembly included), the K product's
    HBM rate, the assembly's (row, element) pairs/s and the force error
    against the FP64 GMRES of the same scene."""
    import torch

    from depsolver_gb300 import api, scenes
    free, total = torch.cuda.mem_get_info()
    if total < 200e9:
        return {"unavailable": f"needs about 135 GB of device memory; the device has {total / 1e9:.0f} GB"}
    sc = scenes.comb_trap()
    s = api.Session(sc)
    try:
        s.set_timing(True)
        s.solve([1e6], mode=api.MODE_MIXED, tol=TOL)     # first solve: assembly, conversion, inverses
        s.timing()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.assemble(api.MODE_MIXED)
        fm, itm, _ = s.solve([1e6], mode=api.MODE_MIXED, tol=TOL)
        torch.cuda.synchronize()
        t_mixed = time.perf_counter() - t0
        timing = s.timing()
        free2, _ = torch.cuda.mem_get_info()
        pm = s.particles()[0]
        t0 = time.perf_counter()
        f64, it64, _ = s.solve([1e6], mode=api.MODE_FP64, tol=TOL)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        p64 = s.particles()[0]
    except Exception as e:  # an allocation the device refused, reported as such
        s.close()
        return {"unavailable": str(e)[:300]}
    s.close()
    P = peaks()
    hbm = P.get("hbm_gbs") or 6800.0
    N = sc.N
    ms, cnt, wk = timing["gemm_K"]
    bpf = (4.0 * N * N + 16.0 * N) / (12.0 * N * N)   # one system: 2 columns
    gemm = {"achieved": wk * bpf * 1e-9 / (ms / 1e3), "unit": "GB/s", "peak": hbm,
            "frac": wk * bpf * 1e-9 / (ms / 1e3) / hbm, "ms": ms, "launches": cnt} if cnt else None
    ams, acnt, awk = timing["asm_regular"]
    gms, gcnt, gwk = timing["gemv_K64"]
    pe = [float(np.abs(pm[k, :3] - p64[k, :3]).max() / p64[k, 6:9].sum()) for k in range(pm.shape[0])]
    return {"workload": "cfg4: castellated trap, 2 x 10 interdigitated fingers (2 x 8, 8 x 32 cells, "
                        "+-1 V) + chain of 8 level-4 spheres (r = 1), 1 MHz, tol 1e-10",
            "N": N, "E": sc.E, "device_memory_used_gb": (total - free2) / 1e9,
            "mixed_s": t_mixed, "inner_iterations": int(itm[0]), "fp64_gmres_s": t64,
            "fp64_gmres_iters": int(it64[0]),
            "force_err_vs_fp64": float(np.abs(fm[0, :3] - f64[0, :3]).max() / f64[0, 6:9].sum()),
            "particle_force_err_vs_fp64_max": max(pe),
            "k_product_hbm": gemm,
            "fp64_residual_gemv": {"achieved": gwk * 1e-9 / (gms / 1e3), "unit": "GB/s", "peak": hbm,
                                   "frac": gwk * 1e-9 / (gms / 1e3) / hbm} if gcnt else None,
            "assembly_pairs_per_s": awk / (ams / 1e3) if acnt else None,
            "kernels_ms": {k: v[0] for k, v in timing.items()}}


# ------------------------------------------------------------------ drop-in sequence
def dropin_bench():
    """The reference's own call sequence through the drop-in entry points on
    host row-pointer buffers (src/depSolver.c:284-310, src/postProcess.c:
    398-445): electricFormA_tria6 -> solverGMRES_el(1, 0) (tolerance 1e-6,
    gmres.log written) -> forceMST_tria6, then field_tria6 at 2646 internal
    points one call each (the point count of the dep-trap-1 example)."""
    import ctypes as C
    import tempfile

    from depsolver_gb300 import _native, api, scenes
    L = _native.lib()
    out = {}
    for name, sc in (("cfg0", scenes.cfg0(center=(0.0, 0.0, 1.0))), ("cfg1", scenes.cfg1())):
        N, E = sc.N, sc.E
        C.c_uint.in_dll(L, "nNodes").value = N
        C.c_uint.in_dll(L, "nElems").value = E
        C.c_uint.in_dll(L, "nInterfaces").value = sc.n_if
        nodes = np.ascontiguousarray(sc.nodes)
        elems = np.ascontiguousarray(sc.elems, dtype=np.uint32)
        mat = np.ascontiguousarray(sc.mat)
        ifc = np.ascontiguousarray(sc.ifaces, dtype=np.uint32)
        mbc = np.ascontiguousarray(sc.mbc)
        bct = np.ascontiguousarray(sc.bctype, dtype=np.uint32)
        prob = np.array([sc.freq])
        A = np.zeros((N, 2 * N))
        B = np.zeros(2 * N)
        rn, re_, rA = api.row_pointers(nodes), api.row_pointers(elems), api.row_pointers(A)
        L.electricFormA_tria6.restype = C.c_int
        t0 = time.perf_counter()
        L.electricFormA_tria6(rn, re_, bct.ctypes.data_as(C.c_void_p), api.row_pointers(ifc),
                              api.row_pointers(mat), prob.ctypes.data_as(C.c_void_p), rA,
                              api.row_pointers(mbc), B.ctypes.data_as(C.c_void_p))
        t1 = time.perf_counter()
        asm_first = t1 - t0
        # the same call again: the rows' pages now exist (the first call
        # pays the host's first touch of the caller's fresh allocation)
        L.electricFormA_tria6(rn, re_, bct.ctypes.data_as(C.c_void_p), api.row_pointers(ifc),
                              api.row_pointers(mat), prob.ctypes.data_as(C.c_void_p), rA,
                              api.row_pointers(mbc), B.ctypes.data_as(C.c_void_p))
        asm_again = time.perf_counter() - t1
        t1 = time.perf_counter()
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)
            try:
                L.solverGMRES_el(C.c_uint(1), C.c_uint(0), rA, B.ctypes.data_as(C.c_void_p))
                t2 = time.perf_counter()
                its = sum(1 for ln in open("gmres.log") if ln[:8].strip().isdigit())
            finally:
                os.chdir(cwd)
        del A, rA
        Fce = np.zeros((E, 3))
        Xce = np.zeros((E, 3))
        Fcm = np.zeros(3)
        Xcm = np.zeros(3)
        t2b = time.perf_counter()
        L.forceMST_tria6(rn, re_, bct.ctypes.data_as(C.c_void_p), B.ctypes.data_as(C.c_void_p),
                         C.c_double(sc.eps_medium), api.row_pointers(Fce), api.row_pointers(Xce),
                         Fcm.ctypes.data_as(C.c_void_p), Xcm.ctypes.data_as(C.c_void_p))
        t3 = time.perf_counter()
        xs, zs = np.linspace(-4.0, 4.0, 63), np.linspace(-3.0, 3.0, 42)
        pts = np.ascontiguousarray([[x, 0.3, z] for z in zs for x in xs])
        mE = np.zeros(6)
        t4 = time.perf_counter()
        for p in pts:
            L.field_tria6(p.ctypes.data_as(C.c_void_p), rn, re_, B.ctypes.data_as(C.c_void_p),
                          mE.ctypes.data_as(C.c_void_p))
        t5 = time.perf_counter()
        out[name] = {"N": N, "E": E, "assembly_s": asm_first, "assembly_again_s": asm_again,
                     "assembly_bytes": 8.0 * N * 2 * N, "gmres_s": t2 - t1, "gmres_iters": its,
                     "force_s": t3 - t2b, "field_points": len(pts), "field_s": t5 - t4,
                     "field_us_per_point": (t5 - t4) / len(pts) * 1e6,
                     "total_s": asm_first + (t2 - t1) + (t3 - t2b) + (t5 - t4)}
        # the C restatement at the same points: batched on every host core,
        # and one point per call on one core as the reference's post-
        # processing runs (a sample of the points at the larger scene)
        from oracle.oracle import Port
        nt = os.cpu_count() or 1
        if name == "cfg0":
            t6 = time.perf_counter()
            Port().field(sc, B, pts, nthreads=nt)
            out[name]["cpu_port_field_s"] = time.perf_counter() - t6
            out[name]["cpu_port_threads"] = nt
        sample = pts[:: (1 if name == "cfg0" else 40)]
        port = Port()
        t7 = time.perf_counter()
        for p in sample:
            port.field(sc, B, p[None], nthreads=1)
        out[name]["cpu_port_1core_us_per_point"] = (time.perf_counter() - t7) / len(sample) * 1e6
        out[name]["cpu_port_1core_points"] = len(sample)
    return out


# ------------------------------------------------------------------ ours
def max_over_ranks(ms: float, world: int, device: str) -> float:
    """The slowest rank's time (every rank gets it): replicas share no data,
    so the job ends when the last replica does."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def replica_throughput(ms: float, world: int, steps: int) -> float:
    """Whole-job systems per second: every replica solves `steps` sweeps of
    NFREQ systems in the slowest rank's `ms`."""
    return world * steps * NFREQ / (ms / 1e3)


def run_ours(args, rank, world):
    import torch

    from depsolver_gb300 import _native, api, scenes

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    L = _native.lib()
    # the 12k-node scene of the metric; --scene mid (level-3 sphere between
    # 25 x 25-cell plates, N = 7764) only for profiler captures of one step
    scene_of = {"cfg1": scenes.cfg1, "mid": lambda: scenes.sphere_between_plates(3, 25, name="mid"),
                "cfg0": lambda: scenes.cfg0(center=(0.0, 0.0, 1.0)), "capacitor25": lambda: scenes.capacitor(25)}
    sc = scene_of[args.scene]()
    N, E = sc.N, sc.E
    s = api.Session(sc)
    s.set_mixed_assembly(api.ASM_FP32 if args.mixed_assembly == "fp32" else api.ASM_DF32)
    stream = torch.cuda.ExternalStream(s.stream_handle())
    if args.only_step:
        # one warm-up and one timed step only (for profiler launch lists);
        # --step-mode fp64: the plain FP64 path's step (FP64 assembly, the
        # reference's GMRES at 1 MHz, force) instead; gauss: the direct
        # solve of the scene's full 2N form (block LU + refinement);
        # positions: 12 positions of the position sweep (levels 2/3/4)
        s.close()
        if args.step_mode == "gauss":
            Af, Bf = api.electric_form(sc, full=True)
            for _ in range(2):
                api.gauss_bksb(Af, Bf, mode=api.GAUSS_MIXED)
        elif args.step_mode == "positions":
            ps = api.PositionSweep(scenes.plates_only(10))
            lev, cen = scenes.cfg3_positions(12)
            tid = {lv: ps.add_particle(*scenes.icosphere(lv, 1.0)) for lv in (2, 3, 4)}
            tm = np.array([tid[int(v)] for v in lev], dtype=np.uint32)
            for _ in range(2):
                ps.solve(tm, cen, FREQS, tol=TOL)
            ps.close()
        else:
            s = api.Session(sc)
            s.set_mixed_assembly(api.ASM_FP32 if args.mixed_assembly == "fp32" else api.ASM_DF32)
            for _ in range(2):
                if args.step_mode == "fp64":
                    s.assemble(api.MODE_FP64)
                    s.solve([1e6], mode=api.MODE_FP64, tol=TOL)
                else:
                    s.assemble(api.MODE_MIXED)
                    s.solve(FREQS, mode=api.MODE_MIXED, tol=TOL)
        torch.cuda.synchronize()
        print(json.dumps({"only_step": True, "launches": int(L.dsc_kernel_launches())}))
        return

    # accuracy: the mixed sweep against FP64 solves (tol 1e-12) at every one
    # of the 64 frequencies (outside the timed region)
    fm, _, sm = s.solve(FREQS, mode=api.MODE_MIXED, tol=TOL, want_sigma=True)
    f64, it64, s64 = s.solve(FREQS, mode=api.MODE_FP64, tol=1e-12, want_sigma=True)
    ferrs = np.abs(fm[:, :3] - f64[:, :3]).max(axis=1) / f64[:, 6:9].sum(axis=1)
    serrs = np.abs(sm - s64).max(axis=1) / np.abs(s64).max(axis=1)
    del sm, s64

    # plain FP64 GPU path: assembly + the reference's GMRES (tol 1e-10) + force
    fp64_t = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.assemble()
        _, itf, _ = s.solve([1e6], mode=api.MODE_FP64, tol=TOL)
        torch.cuda.synchronize()
        fp64_t.append(time.perf_counter() - t0)
    fp64_s = min(fp64_t)

    # the speed-up split into its parts (each a step of assembly + solve,
    # best of 3 after one warm-up): precision (mixed, one frequency per step,
    # complex Jacobi scaling only, against the FP64 path's Jacobi GMRES),
    # the conductor-block preconditioner (one frequency per step), batching
    # (64 frequencies per step)
    def per_solve(freqs, pre):
        s.set_preconditioner(pre)
        best = None
        for r in range(4):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.assemble(api.MODE_MIXED)
            s.solve(freqs, mode=api.MODE_MIXED, tol=TOL)
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / len(freqs)
            if r:
                best = dt if best is None else min(best, dt)
        s.set_preconditioner(True)
        return best
    one = [1e6]
    abl = {"fp64_jacobi_1freq": fp64_s, "mixed_jacobi_1freq": per_solve(one, False),
           "mixed_precond_1freq": per_solve(one, True), "mixed_jacobi_64freq": per_solve(FREQS, False),
           "mixed_precond_64freq": per_solve(FREQS, True)}
    ablation = {"s_per_solve": abl,
                "precision": abl["fp64_jacobi_1freq"] / abl["mixed_jacobi_1freq"],
                "preconditioner": abl["mixed_jacobi_1freq"] / abl["mixed_precond_1freq"],
                "batching": abl["mixed_precond_1freq"] / abl["mixed_precond_64freq"],
                "def": "each factor a ratio of seconds per solve (assembly included, 1 MHz for one frequency): "
                       "precision = FP64 Jacobi GMRES / mixed without the preconditioner; preconditioner = "
                       "mixed without / with it; batching = one frequency per step / 64 per step"}

    # headline: warm-up, then K timed steps (assembly + 64-system sweep)
    for _ in range(args.warmup):
        s.assemble(api.MODE_MIXED)
        s.solve(FREQS, mode=api.MODE_MIXED, tol=TOL)
    s.set_timing(True)
    s.timing()  # reset
    clocks = ClockSampler(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = L.dsc_kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        s.assemble(api.MODE_MIXED)
        _, its, _ = s.solve(FREQS, mode=api.MODE_MIXED, tol=TOL)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = int(L.dsc_kernel_launches() - l0)
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), world, "cuda")
    timing = s.timing()
    total_ms = sum(v[0] for v in timing.values())
    value = replica_throughput(ms, world, args.steps)

    s.close()  # its device memory goes back to the pool the sweeps draw from

    # e2e through the C ABI from host arrays: dsc_sweep (session created,
    # mesh uploaded, assembled, solved, nodal solution and forces read back);
    # one untimed call first, which grows the device memory pool to a
    # sweep's size (later calls reuse those blocks)
    e2e_steps = max(1, min(args.steps, 3))
    api.sweep(sc, FREQS, mode=api.MODE_MIXED, tol=TOL, want_sigma=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        fe, _, se = api.sweep(sc, FREQS, mode=api.MODE_MIXED, tol=TOL, want_sigma=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = (sc.nodes.nbytes + sc.elems.astype(np.uint32).nbytes + sc.bctype.astype(np.uint32).nbytes
           + sc.mbc.nbytes + sc.mat.nbytes + sc.ifaces.astype(np.uint32).nbytes + FREQS.nbytes)
    d2h = se.nbytes + fe.nbytes

    if rank != 0:
        return
    pos = position_bench(args, with_cpu=not args.no_cpu) if not args.no_positions else None
    gauss = gauss_bench(with_cpu=not args.no_cpu) if not args.no_extras else None
    trap = trap_bench() if not args.no_extras else None
    large = large_bench() if not args.no_extras else None
    dropin = dropin_bench() if not args.no_extras else None
    # roofline of the dominant kernel class over the timed region: achieved
    # = algorithmic work (counted by the library per class) / CUDA-event time
    # of the class on the session's stream
    roof, roof_all = roofline(timing, N, E)
    cpu = cpu_baseline(sc, os.cpu_count() or 1) if not args.no_cpu else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-matvec/f64-residual",
        "data": "synthetic (seeded scene generator, reference input model)",
        "config": {"workload": "cfg1: level-4 tria6 sphere (r=1, eps_r 2.5, sigma 1e-3) between "
                               "30x30-cell tria6 plates at z=+-5, +-1 V; medium eps_r 78, sigma 1e-4",
                   "N": N, "E": E, "freqs_per_step": NFREQ, "freq_range_hz": [1e3, 1e8],
                   "tol": TOL, "step": f"assemble K ({args.mixed_assembly.upper()} regular / double-FP32 singular pairs) + 64-system mixed sweep + MST forces",
                   "l2": "inputs larger than L2 (K 2.5 GB FP64 + its 1.25 GB fp16 pair + 5 GB digits)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": NFREQ / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "calls_timed": e2e_steps, "untimed_calls_before": 1},
        "roofline": roof,
        "cpu_baseline": cpu,
        "fp64_path": {"value": 1.0 / fp64_s, "unit": UNIT, "ms_per_solve": fp64_s * 1e3,
                      "gmres_iters": int(itf[0])},
        "speedup_vs_fp64_path": value / world / (1.0 / fp64_s),
        "speedup_parts": ablation,
        "position_sweep": pos,
        "gauss": gauss,
        "trap": trap,
        "large": large,
        "dropin": dropin,
        "inner_iterations": {"mean": float(np.mean(its)), "max": int(np.max(its)),
                             "products_per_step": timing["gemm_K"][1] // max(1, args.steps)},
        "accuracy": {"force_err_vs_fp64": float(ferrs.max()),
                     "force_err_median": float(np.median(ferrs)),
                     "sigma_rel_err_vs_fp64": float(serrs.max()),
                     "sigma_rel_err_median": float(np.median(serrs)),
                     "frequencies_checked": int(len(ferrs)),
                     "force_err_def": "over all 64 frequencies: |Fcm_mixed - Fcm_fp64|_max / sum|Fce| "
                                      "(FP64 path at tol 1e-12); sigma: max |diff| / max |sigma_fp64|"},
        "kernels_ms": {k: {"ms": v[0], "scopes": v[1], "share": v[0] / total_ms if total_ms else 0}
                       for k, v in timing.items()},
        "roofline_classes": roof_all,
        "autotuned_splits": [{"N": r[0], "columns": r[1], "splits": r[2]} for r in api.autotune_table()],
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ reference
def run_reference(args, rank, world):
    if rank != 0:
        return
    from depsolver_gb300 import scenes
    sc = scenes.cfg1()
    threads = os.cpu_count() or 1
    # warm-up: one full solve (the reference's iteration count), then samples
    first = cpu_baseline(sc, threads, full_first=True)
    for _ in range(max(0, args.warmup - 1)):
        cpu_baseline(sc, threads, full_first=False)
    ests = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = cpu_baseline(sc, threads, full_first=False)
        ests.append(r["est_solve_s"])
    wall = time.perf_counter() - t0
    it = first["full"]["gmres_iters"]
    est = statistics.median(ests)
    value = 1.0 / est
    cb = dict(first)
    cb["value"] = value
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded scene generator, reference input model)",
           "config": {"workload": "cfg1 (as the GPU arm), one frequency per solve, "
                                  f"reference GMRES tolerance 1e-6 ({it} iterations)",
                      "N": sc.N, "E": sc.E, "threads": threads},
           "cpu_baseline": cb,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-positions", action="store_true", help="skip the position sweep (cfg3)")
    ap.add_argument("--no-extras", action="store_true", help="skip the direct-solve and trap sections")
    ap.add_argument("--pos-workers", type=int, default=4, help="host workers (streams) of the position sweep")
    ap.add_argument("--scene", choices=["cfg1", "mid", "cfg0", "capacitor25"], default="cfg1",
                    help="mid, cfg0, capacitor25: other scenes for ncu captures (with --only-step)")
    ap.add_argument("--mixed-assembly", choices=["fp32", "df32"], default="fp32",
                    help="arithmetic of the mixed mode's regular pairs (FP32 far field, or double-FP32)")
    ap.add_argument("--step-mode", choices=["mixed", "fp64", "gauss", "positions"], default="mixed",
                    help="with --only-step: profile the mixed sweep, the plain FP64 path, the direct "
                         "solve of the scene's full form, or a 12-position sample of the position sweep")
    ap.add_argument("--only-step", action="store_true",
                    help="run one warm-up and one step and nothing else (profiling)")
    args = ap.parse_args()
    if args.scene != "cfg1" and not args.only_step:
        ap.error("--scene mid is for profiler captures: use it with --only-step")
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
