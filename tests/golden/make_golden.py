"""Generates the golden fixtures in this directory from the reference itself.

Run where the reference sources exist (it builds oracle/_ref/libdsref.so
from them):

    python tests/golden/make_golden.py [--reference DIR]

DIR defaults to the reference tree beside the repository (../reference from
the repository's root).

Fixtures (NumPy .npz, all FP64 bit patterns straight from the reference's
own functions through oracle/ref_harness.c):

* small_tria6.npz / small_tria3.npz -- scenes.small(nen): probes of the
  compact and full matrices (A @ r, A^T @ s for seeded r, s and a few whole
  rows), the GMRES solution at the compiled tolerance 1e-6 and its
  gmres.log, the tol-1e-10 GMRES and Gauss solutions, field and potential
  at six points, the MST force.
* cfg0_tria6.npz -- the level-2 sphere between 10 x 10-cell plates
  (1524 nodes): Gauss (3048 unknowns) and GMRES at 1e-10 solutions, MST
  force from each.
* multipole.npz -- forceMultipole_* (orders 1-5) and forceEllipsoid_*
  (analyses 10 and 11) of both small scenes at three points, from their
  Gauss solutions.
* dep_trap_2.npz -- the reference's own example deck examples/dep-trap-2
  (956 nodes, 1676 tria3, nodes 537.. shifted by (1.25e-5, 0, 0) as its
  REPOSITION section asks), with the reference's solution, gmres.log and
  MST force; also the 2008 golden force-mst.dat and gmres.log texts shipped
  with the example.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from depsolver_gb300 import scenes  # noqa: E402

PROBE_SEED = 12345
PROBE_ROWS = 8


def probes(A: np.ndarray, seed: int = PROBE_SEED):
    rng = np.random.default_rng(seed)
    r = rng.standard_normal(A.shape[1])
    s = rng.standard_normal(A.shape[0])
    rows = np.linspace(0, A.shape[0] - 1, PROBE_ROWS).astype(np.int64)
    return {"Ar": A @ r, "ATs": A.T @ s, "rows_idx": rows, "rows": A[rows]}


def eval_points(sc):
    p0 = sc.particles[0][0]
    pts = [sc.nodes[p0], sc.nodes[p0 + 1], sc.nodes[p0 + 7]]  # on the particle (singular)
    pts += [[0.1, 0.2, -1.5], [0.7, -0.3, 2.2], [-2.0, 1.0, 0.0]]
    return np.asarray(pts, dtype=np.float64)


def scene_fixture(ref, sc, path, with_full=True):
    out = {"name": sc.name, "N": sc.N, "E": sc.E}
    A, B = ref.assemble(sc)
    for k, v in probes(A).items():
        out["compact_" + k] = v
    out["B"] = B
    x, log = ref.gmres(A, B)
    out["x_gmres"] = x
    out["gmres_log"] = np.frombuffer(log.encode(), dtype=np.uint8)
    xt, logt = ref.gmres(A, B, tight=True)
    out["x_gmres_tight"] = xt
    out["gmres_tight_log"] = np.frombuffer(logt.encode(), dtype=np.uint8)
    if with_full:
        Af, Bf = ref.assemble(sc, full=True)
        for k, v in probes(Af).items():
            out["full_" + k] = v
        out["x_gauss"] = ref.gauss(Af, Bf)
        Fce, Xce, Fcm, Xcm = ref.force_mst(sc, out["x_gauss"])
        out["Fcm_gauss"] = Fcm
    pts = eval_points(sc)
    out["pts"] = pts
    out["field"] = ref.field(sc, x, pts)
    out["potential"] = ref.potential(sc, x, pts)
    Fce, Xce, Fcm, Xcm = ref.force_mst(sc, x)
    mask = sc.bctype[sc.elems[:, 0] - 1] == 6
    out["pel"] = np.nonzero(mask)[0]
    out["Fce"] = Fce[mask]
    out["Xce"] = Xce[mask]
    out["Fcm"] = Fcm
    out["Xcm"] = Xcm
    Fce, Xce, Fcm, Xcm = ref.force_mst(sc, xt)
    out["Fcm_tight"] = Fcm
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def dep_trap_2(ref, examples, path):
    d = os.path.join(examples, "dep-trap-2")
    sc = scenes.shifted(scenes.read_bem(d), 536, (1.25e-5, 0.0, 0.0))
    A, B = ref.assemble(sc)
    x, log = ref.gmres(A, B)
    Fce, Xce, Fcm, Xcm = ref.force_mst(sc, x)
    mask = sc.bctype[sc.elems[:, 0] - 1] == 6
    out = dict(nen=sc.nen, nodes=sc.nodes, elems=sc.elems, bctype=sc.bctype, mbc=sc.mbc,
               ifaces=sc.ifaces, mat=sc.mat, freq=sc.freq, x_gmres=x,
               gmres_log=np.frombuffer(log.encode(), np.uint8), pel=np.nonzero(mask)[0],
               Fce=Fce[mask], Xce=Xce[mask], Fcm=Fcm, Xcm=Xcm,
               golden_force_mst=np.frombuffer(open(os.path.join(d, "force-mst.dat"), "rb").read(), np.uint8),
               golden_gmres_log=np.frombuffer(open(os.path.join(d, "gmres.log"), "rb").read(), np.uint8))
    for k, v in probes(A).items():
        out["compact_" + k] = v
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


MP_POINTS = np.array([[0.0, 0.0, 0.4], [0.05, -0.1, 0.3], [0.5, 0.5, -1.8]])
MP_AXIS = np.array([1.0, 0.9, 0.8])


def multipole_fixture(ref, path):
    """forceMultipole_* (orders 1-5) and forceEllipsoid_* (analyses 10, 11)
    of the reference at three points (the small scene's sphere centre, a
    point inside the sphere and one in the medium), from the reference's
    own Gauss solution of each small scene (radius 1; semi-axes MP_AXIS)."""
    out = {"points": MP_POINTS, "axis": MP_AXIS, "R": np.float64(1.0)}
    for nen in (6, 3):
        sc = scenes.small(nen=nen)
        g = np.load(os.path.join(HERE, f"small_tria{nen}.npz"))
        x = g["x_gauss"]
        out[f"x_{nen}"] = x
        out[f"multipole_{nen}"] = np.array([[ref.force_multipole(sc, x, o, 1.0, p) for o in range(1, 6)]
                                            for p in MP_POINTS])
        out[f"ellipsoid_{nen}"] = np.array([[ref.force_ellipsoid(sc, x, a, MP_AXIS, p) for a in (10, 11)]
                                            for p in MP_POINTS])
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference",
                    default=os.path.normpath(os.path.join(HERE, "..", "..", "..", "reference")))
    ap.add_argument("--only", nargs="*", default=None,
                    help="fixtures to write (small, cfg0, dep_trap_2, multipole; default: all)")
    args = ap.parse_args()
    want = set(args.only) if args.only else {"small", "cfg0", "dep_trap_2", "multipole"}
    os.environ["DSC_REFERENCE_SRC"] = os.path.join(args.reference, "src")
    from oracle import oracle as orc
    orc.REF_SRC = os.environ["DSC_REFERENCE_SRC"]
    if orc.build_ref() is None:
        sys.exit("reference sources not found")
    ref = orc.Ref()
    if "small" in want:
        for nen in (6, 3):
            scene_fixture(ref, scenes.small(nen=nen), os.path.join(HERE, f"small_tria{nen}.npz"))
    if "cfg0" in want:
        scene_fixture(ref, scenes.cfg0(nen=6, center=(0.0, 0.0, 1.0)), os.path.join(HERE, "cfg0_tria6.npz"))
    if "dep_trap_2" in want:
        dep_trap_2(ref, os.path.join(args.reference, "examples"), os.path.join(HERE, "dep_trap_2.npz"))
    if "multipole" in want:
        multipole_fixture(ref, os.path.join(HERE, "multipole.npz"))


if __name__ == "__main__":
    main()
