"""Synthetic BEM scenes in the reference's input model.

A scene carries exactly what depSolver reads from ``input.bem`` and its mesh
files (reference ``src/depSolver.c:98-237``):

* ``nodes``   N x 3 float64 coordinates (SI units, as the reference);
* ``elems``   E x nen uint32, **1-based** node ids, node order
  corner, mid, corner, mid, corner, mid for tria6 (``src/shapeFunctions.c:68``);
* ``bctype``  2N uint32 boundary types: 1 = conductor (potential given),
  0 = dielectric interface, 6 = interface whose Maxwell-stress force is wanted;
  rows N..2N-1 describe the imaginary equations;
* ``mbc``     2N x 3 float64: value, interface id (1-based) for interface rows;
* ``ifaces``  nIf x 2 material ids (1-based); ``mat`` nMat x 2 (sigma S/m, eps_r);
  material 1 is the medium (the force uses its permittivity,
  ``src/postProcess.c:432``);
* ``freq``    Hz.

Geometry builders: level-L icosahedral spheres (tria6: 40*4^L + 2 nodes,
20*4^L elements; tria3: 10*4^L + 2 nodes) with mid-side nodes on the sphere,
and flat square electrodes whose n x n quad cells are each split into two
triangles (tria6: (2n+1)^2 nodes).  Element normals point out of spheres, so
an interface (medium=1, particle=k) has its normal pointing into material 1
as the reference's interface coefficients expect (``src/assembly_el.c:223-239``).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

EPS0 = 8.854187817e-12


@dataclasses.dataclass
class Scene:
    nen: int
    nodes: np.ndarray
    elems: np.ndarray
    bctype: np.ndarray
    mbc: np.ndarray
    ifaces: np.ndarray
    mat: np.ndarray
    freq: float
    name: str = "scene"
    # [start, end) node ranges and element ranges of each particle (type 6)
    particles: List[Tuple[int, int, int, int]] = dataclasses.field(default_factory=list)

    @property
    def N(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def E(self) -> int:
        return int(self.elems.shape[0])

    @property
    def n_if(self) -> int:
        return int(self.ifaces.shape[0])

    @property
    def eps_medium(self) -> float:
        return float(self.mat[0, 1] * EPS0)

    def with_freq(self, f: float) -> "Scene":
        return dataclasses.replace(self, freq=float(f))

    def contiguous(self) -> "Scene":
        return dataclasses.replace(
            self,
            nodes=np.ascontiguousarray(self.nodes, dtype=np.float64),
            elems=np.ascontiguousarray(self.elems, dtype=np.uint32),
            bctype=np.ascontiguousarray(self.bctype, dtype=np.uint32),
            mbc=np.ascontiguousarray(self.mbc, dtype=np.float64),
            ifaces=np.ascontiguousarray(self.ifaces.reshape(-1, 2), dtype=np.uint32),
            mat=np.ascontiguousarray(self.mat, dtype=np.float64),
        )


# ---------------------------------------------------------------- geometry


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def _subdivide(v: np.ndarray, f: np.ndarray):
    verts = [tuple(x) for x in v]
    cache = {}

    def mid(a, b):
        key = (a, b) if a < b else (b, a)
        if key in cache:
            return cache[key]
        m = (np.asarray(verts[a]) + np.asarray(verts[b])) * 0.5
        m /= np.linalg.norm(m)
        verts.append(tuple(m))
        cache[key] = len(verts) - 1
        return cache[key]

    nf = []
    for a, b, c in f:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
    return np.asarray(verts), np.asarray(nf, dtype=np.int64)


def _orient_outward(v: np.ndarray, f: np.ndarray) -> np.ndarray:
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, a + b + c) < 0
    f = f.copy()
    f[flip] = f[flip][:, [0, 2, 1]]
    return f


def _drop_unused(nodes: np.ndarray, elems: np.ndarray):
    """Nodes that no element names removed (quad8 grids have no node at a
    cell's centre), the rest renumbered in their order."""
    used = np.zeros(nodes.shape[0], bool)
    used[elems.ravel()] = True
    new = np.cumsum(used) - 1
    return nodes[used], new[elems].astype(np.int64)


def cubed_sphere(cells: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Sphere of quad8 elements: each face of the cube [-1, 1]^3 cut into
    cells x cells quads, every node (corners and mid-sides) projected onto
    the sphere, nodes shared across faces merged, elements oriented with
    their normal outward.  Returns (nodes, 0-based elems)."""
    g = 2 * cells + 1
    t = np.linspace(-1.0, 1.0, g)
    faces = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            U, V = np.meshgrid(t, t, indexing="xy")
            P = np.zeros((g, g, 3))
            a, b = [d for d in range(3) if d != axis]
            P[..., axis] = sign
            P[..., a] = U
            P[..., b] = V
            faces.append(P)
    key_id, nodes = {}, []

    def node(p):
        q = p / np.linalg.norm(p)
        k = tuple(np.round(p, 12))
        if k not in key_id:
            key_id[k] = len(nodes)
            nodes.append(q)
        return key_id[k]

    el = []
    for P in faces:
        ids = [[node(P[j, i]) for i in range(g)] for j in range(g)]
        for j in range(cells):
            for i in range(cells):
                I, J = 2 * i, 2 * j
                e = [ids[J][I], ids[J][I + 2], ids[J + 2][I + 2], ids[J + 2][I],
                     ids[J][I + 1], ids[J + 1][I + 2], ids[J + 2][I + 1], ids[J + 1][I]]
                el.append(e)
    nodes = np.asarray(nodes)
    elems = np.asarray(el, dtype=np.int64)
    # outward: the corners' diagonal cross product along the centroid
    c0, c1, c2, c3 = (nodes[elems[:, k]] for k in range(4))
    n = np.cross(c2 - c0, c3 - c1)
    flip = np.einsum("ij,ij->i", n, c0 + c1 + c2 + c3) < 0
    elems[flip] = elems[flip][:, [0, 3, 2, 1, 7, 6, 5, 4]]
    nodes, elems = _drop_unused(nodes, elems)
    return nodes * radius + np.asarray(center, dtype=np.float64), elems


def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0), nen: int = 6):
    """Unit icosphere subdivided `level` times, as (nodes, 0-based elems).

    tria6 mid-side nodes are projected onto the sphere, so the quadratic
    elements follow the curved surface."""
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    f = _orient_outward(v, f)
    if nen == 3:
        nodes = v
        elems = f
    else:
        edge_id = {}
        mids = []
        nv = v.shape[0]

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in edge_id:
                m = (v[a] + v[b]) * 0.5
                mids.append(m / np.linalg.norm(m))
                edge_id[key] = nv + len(mids) - 1
            return edge_id[key]

        el = []
        for a, b, c in f:
            el.append([a, mid(a, b), b, mid(b, c), c, mid(c, a)])
        nodes = np.vstack([v, np.asarray(mids)])
        elems = np.asarray(el, dtype=np.int64)
    nodes = nodes * radius + np.asarray(center, dtype=np.float64)
    return nodes, elems


def plate(side_x: float, side_y: float, ncell_x: int, ncell_y: int, center=(0.0, 0.0, 0.0),
          nen: int = 6):
    """Flat rectangle in the plane z = center[2], meshed as ncell_x x ncell_y
    quads, each split into two triangles along its (0,0)-(1,1) diagonal, or
    kept as one quad8 (nen = 8: corners counter-clockwise, then the
    mid-sides of edges 1-2, 2-3, 3-4, 4-1).  Returns (nodes, 0-based elems);
    normals point along +z."""
    cx, cy, cz = center
    if nen == 3:
        gx, gy = ncell_x + 1, ncell_y + 1
    else:
        gx, gy = 2 * ncell_x + 1, 2 * ncell_y + 1
    xs = np.linspace(cx - side_x / 2, cx + side_x / 2, gx)
    ys = np.linspace(cy - side_y / 2, cy + side_y / 2, gy)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    nodes = np.stack([X.ravel(), Y.ravel(), np.full(X.size, cz)], axis=1)

    def idx(i, j):
        return j * gx + i

    el = []
    for j in range(ncell_y):
        for i in range(ncell_x):
            if nen == 3:
                p00, p10, p11, p01 = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
                el.append([p00, p10, p11])
                el.append([p00, p11, p01])
            elif nen == 8:
                I, J = 2 * i, 2 * j
                el.append([idx(I, J), idx(I + 2, J), idx(I + 2, J + 2), idx(I, J + 2),
                           idx(I + 1, J), idx(I + 2, J + 1), idx(I + 1, J + 2), idx(I, J + 1)])
            else:
                I, J = 2 * i, 2 * j
                p00, p10, p11, p01 = idx(I, J), idx(I + 2, J), idx(I + 2, J + 2), idx(I, J + 2)
                cc = idx(I + 1, J + 1)
                el.append([p00, idx(I + 1, J), p10, idx(I + 2, J + 1), p11, cc])
                el.append([p00, cc, p11, idx(I + 1, J + 2), p01, idx(I, J + 1)])
    elems = np.asarray(el, dtype=np.int64)
    if nen == 8:
        nodes, elems = _drop_unused(nodes, elems)
    return nodes, elems


# ---------------------------------------------------------------- scenes


def _assemble(parts, nen, mat, ifaces, freq, name) -> Scene:
    """parts: list of (nodes, elems0, kind, payload) where kind is
    'conductor' (payload = complex potential) or 'particle'
    (payload = 1-based interface id, with force)."""
    nodes_all, elems_all, bct, mbc_re, mbc_im = [], [], [], [], []
    particles = []
    off = 0
    eoff = 0
    for nodes, elems0, kind, payload in parts:
        n = nodes.shape[0]
        nodes_all.append(nodes)
        elems_all.append(elems0 + off + 1)
        if kind == "conductor":
            v = complex(payload)
            bct.append(np.ones(n, np.uint32))
            mbc_re.append(np.tile([v.real, 0.0, 0.0], (n, 1)))
            mbc_im.append(np.tile([v.imag, 0.0, 0.0], (n, 1)))
        else:
            bct.append(np.full(n, 6, np.uint32))
            mbc_re.append(np.tile([0.0, float(payload), 0.0], (n, 1)))
            mbc_im.append(np.tile([0.0, float(payload), 0.0], (n, 1)))
            particles.append((off, off + n, eoff, eoff + elems0.shape[0]))
        off += n
        eoff += elems0.shape[0]
    nodes = np.vstack(nodes_all)
    elems = np.vstack(elems_all).astype(np.uint32)
    bt = np.concatenate(bct)
    bctype = np.concatenate([bt, bt]).astype(np.uint32)
    mbc = np.vstack([np.vstack(mbc_re), np.vstack(mbc_im)])
    return Scene(nen, nodes, elems, bctype, mbc,
                 np.asarray(ifaces, np.uint32).reshape(-1, 2),
                 np.asarray(mat, np.float64).reshape(-1, 2), float(freq), name,
                 particles).contiguous()


def sphere_between_plates(sphere_level: int, plate_cells: int, *, nen: int = 6,
                          radius: float = 1.0, center=(0.0, 0.0, 0.0),
                          plate_side: float = 20.0, plate_z: float = 5.0,
                          volts: float = 1.0, freq: float = 1.0e6,
                          medium=(1.0e-4, 78.0), particle=(1.0e-3, 2.5),
                          name: Optional[str] = None) -> Scene:
    """One dielectric sphere between two square plate electrodes at
    z = +-plate_z held at +-volts.  Material 1 = medium, 2 = sphere;
    interface 1 = (1, 2); sphere nodes carry boundary type 6.  nen = 8: quad8
    plates and a cubed sphere of 2^sphere_level cells per face edge."""
    if nen == 8:
        s_nodes, s_el = cubed_sphere(2 ** sphere_level, radius, center)
    else:
        s_nodes, s_el = icosphere(sphere_level, radius, center, nen)
    top_n, top_e = plate(plate_side, plate_side, plate_cells, plate_cells, (0, 0, plate_z), nen)
    bot_n, bot_e = plate(plate_side, plate_side, plate_cells, plate_cells, (0, 0, -plate_z), nen)
    parts = [(top_n, top_e, "conductor", volts), (bot_n, bot_e, "conductor", -volts),
             (s_nodes, s_el, "particle", 1)]
    mat = [list(medium), list(particle)]
    return _assemble(parts, nen, mat, [[1, 2]], freq,
                     name or f"sphere-L{sphere_level}-plates-{plate_cells}x{plate_cells}-tria{nen}")


def conductor_sphere(cells: int = 4, *, nen: int = 8, radius: float = 1.0, volts: float = 1.0,
                     eps_r: float = 1.0, freq: float = 1.0e6) -> Scene:
    """One sphere held at `volts` alone in one medium (a real system whose
    potential outside is volts * radius / r and whose field on the surface
    is volts / radius along the normal): a quad8 cubed sphere of `cells`
    cells per face edge, or (nen = 3, 6) an icosphere of level `cells`."""
    if nen == 8:
        n, e = cubed_sphere(cells, radius)
    else:
        n, e = icosphere(cells, radius, nen=nen)
    return _assemble([(n, e, "conductor", volts)], nen, [[0.0, eps_r]], np.zeros((0, 2)), freq,
                     f"conductor-sphere-{cells}-n{nen}")


def cfg0(nen: int = 6, center=(0.0, 0.0, 0.0)) -> Scene:
    """Level-2 sphere (r = 1, eps_r 2.5, sigma 1e-3) between 20 x 20 plates
    of 10 x 10 cells at z = +-5, +-1 V, 1 MHz; medium eps_r 78, sigma 1e-4.
    tria6: 642 + 2 x 441 = 1524 nodes, 320 + 400 elements."""
    return sphere_between_plates(2, 10, nen=nen, center=center, name="cfg0-sphereL2-plates10")


def cfg1(nen: int = 6, center=(0.0, 0.0, 0.0)) -> Scene:
    """Level-4 sphere between 30 x 30-cell plates: 10242 + 2 x 3721 =
    17684 nodes, 5120 + 3600 = 8720 tria6 elements."""
    return sphere_between_plates(4, 30, nen=nen, center=center, name="cfg1-sphereL4-plates30")


def small(nen: int = 6, sphere_level: int = 1, plate_cells: int = 3,
          center=(0.0, 0.0, 0.4), freq: float = 1.0e6) -> Scene:
    """A few-hundred-node scene for parity tests (off-centre sphere so that
    the net force is not zero by symmetry)."""
    return sphere_between_plates(sphere_level, plate_cells, nen=nen, center=center,
                                 plate_side=8.0, plate_z=3.0, freq=freq,
                                 name=f"small-L{sphere_level}-p{plate_cells}-tria{nen}")


def quadrupole_trap(nen: int = 6, seed: int = 7, levels=(3, 3, 4, 4),
                    radii=(0.5, 0.8, 1.0, 1.3), pad_cells: int = 16,
                    freq: float = 1.0e5) -> Scene:
    """Four 4 x 4 pads on z = 0 at (+-3, +-3) with phases 0/90/180/270 deg
    at 1 V, and four spheres of the given radii at seeded non-overlapping
    positions in [-2,2]^2 x [1,3]; each sphere has its own material
    (eps_r ~ U[2,10], sigma log-uniform in [1e-6, 1e-2]) and interface."""
    rng = np.random.default_rng(seed)
    parts = []
    phases = [0.0, 90.0, 180.0, 270.0]
    for (sx, sy), ph in zip([(3, 3), (-3, 3), (-3, -3), (3, -3)], phases):
        n, e = plate(4.0, 4.0, pad_cells, pad_cells, (sx, sy, 0.0), nen)
        parts.append((n, e, "conductor", complex(math.cos(math.radians(ph)),
                                                 math.sin(math.radians(ph)))))
    centers = []
    for r in radii:
        for _ in range(10000):
            c = np.array([rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(1, 3)])
            if c[2] - r <= 0.05:
                continue
            if all(np.linalg.norm(c - c2) > r + r2 + 0.05 for c2, r2 in centers):
                break
        centers.append((c, r))
    mat = [[1.0e-4, 78.0]]
    ifaces = []
    for k, ((c, r), lev) in enumerate(zip(centers, levels)):
        eps_r = rng.uniform(2.0, 10.0)
        sig = 10.0 ** rng.uniform(-6.0, -2.0)
        mat.append([sig, eps_r])
        ifaces.append([1, k + 2])
        n, e = icosphere(lev, r, c, nen)
        parts.append((n, e, "particle", k + 1))
    return _assemble(parts, nen, mat, ifaces, freq, f"quadrupole-trap-tria{nen}")


def capacitor(cells: int = 25, *, nen: int = 6, side: float = 20.0, gap: float = 2.0,
              volts: float = 1.0, eps_r: float = 80.0, freq: float = 1.0e6) -> Scene:
    """Two parallel square plates (side x side, cells x cells quads split into
    triangles) at z = +-gap/2 held at +-volts in one medium: conductors only,
    a real system.  cells = 25, tria6: 2 x 2601 = 5202 nodes and 2500
    elements, the size of the reference's capacitor-1/quadratic example."""
    top_n, top_e = plate(side, side, cells, cells, (0, 0, gap / 2), nen)
    bot_n, bot_e = plate(side, side, cells, cells, (0, 0, -gap / 2), nen)
    parts = [(top_n, top_e, "conductor", volts), (bot_n, bot_e, "conductor", -volts)]
    return _assemble(parts, nen, [[0.0, eps_r]], np.zeros((0, 2)), freq, f"capacitor-{cells}x{cells}-tria{nen}")


def comb_trap(nen: int = 6, fingers: int = 10, finger=(2.0, 8.0), cells=(8, 32), pitch: float = 3.0,
              overlap: float = 6.0, spheres: int = 8, sphere_level: int = 4, radius: float = 1.0,
              spacing: float = 2.5, height: float = 2.0, volts: float = 1.0, freq: float = 1.0e6,
              medium=(1.0e-4, 78.0), particle=(1.0e-3, 2.5)) -> Scene:
    """Castellated trap: two interdigitated combs of `fingers` fingers each,
    alternating in x at `pitch` in the plane z = 0 (each finger w x l,
    cells[0] x cells[1] quads split into triangles; comb A's fingers, at
    +volts, span y in [overlap/2 - l, overlap/2], comb B's, at -volts,
    [-overlap/2, l - overlap/2]), and a chain of `spheres` spheres along x
    at height z = height, all of one particle material on interface 1.
    Defaults: 20 fingers of 8 x 32 cells (1105 tria6 nodes each) and 8
    level-4 spheres: N = 104036, E = 51200."""
    w, l = finger
    parts = []
    n_f = 2 * fingers
    x0 = -(n_f - 1) * pitch / 2.0
    for q in range(n_f):
        a = q % 2 == 0
        yc = (overlap / 2.0 - l / 2.0) if a else (l / 2.0 - overlap / 2.0)
        n, e = plate(w, l, cells[0], cells[1], (x0 + q * pitch, yc, 0.0), nen)
        parts.append((n, e, "conductor", volts if a else -volts))
    xs = -(spheres - 1) * spacing / 2.0
    for k in range(spheres):
        n, e = icosphere(sphere_level, radius, (xs + k * spacing, 0.0, height), nen)
        parts.append((n, e, "particle", 1))
    return _assemble(parts, nen, [list(medium), list(particle)], [[1, 2]], freq,
                     f"comb-trap-{fingers}x2-spheres{spheres}-L{sphere_level}-tria{nen}")


def plates_only(plate_cells: int = 10, *, nen: int = 6, plate_side: float = 20.0,
                plate_z: float = 5.0, volts: float = 1.0, freq: float = 1.0e6,
                medium=(1.0e-4, 78.0), particle=(1.0e-3, 2.5)) -> Scene:
    """The fixed part of a position sweep: the two plate electrodes of
    :func:`sphere_between_plates` (materials and interface 1 = medium /
    particle as there), without the sphere."""
    top_n, top_e = plate(plate_side, plate_side, plate_cells, plate_cells, (0, 0, plate_z), nen)
    bot_n, bot_e = plate(plate_side, plate_side, plate_cells, plate_cells, (0, 0, -plate_z), nen)
    parts = [(top_n, top_e, "conductor", volts), (bot_n, bot_e, "conductor", -volts)]
    return _assemble(parts, nen, [list(medium), list(particle)], [[1, 2]], freq,
                     f"plates-{plate_cells}x{plate_cells}-tria{nen}")


def cfg3_positions(n: int = 128, seed: int = 3, levels=(2, 3, 4), radius: float = 1.0,
                   box=((-4.0, 4.0), (-4.0, 4.0), (-3.0, 3.0)), plate_z: float = 5.0):
    """Seeded sphere positions of the batched position sweep on the config-0
    plates: centres uniform in the box, each sphere's mesh level drawn
    uniformly from `levels`; centres whose sphere would reach a plate are
    drawn again.  Returns (levels (n,), centres (n, 3))."""
    rng = np.random.default_rng(seed)
    lev = np.empty(n, dtype=np.int64)
    cen = np.empty((n, 3))
    for q in range(n):
        while True:
            c = np.array([rng.uniform(*box[0]), rng.uniform(*box[1]), rng.uniform(*box[2])])
            if abs(c[2]) + radius < plate_z - 0.05:
                break
        cen[q] = c
        lev[q] = rng.choice(np.asarray(levels))
    return lev, cen


def shifted(scene: Scene, first_node: int, delta) -> Scene:
    """Rigid shift of nodes first_node.. (0-based) by delta, as the
    reference's position-sweep driver does (src/depSolver-shift.c:212-217)."""
    nodes = scene.nodes.copy()
    nodes[first_node:] += np.asarray(delta, dtype=np.float64)
    return dataclasses.replace(scene, nodes=nodes)


# ---------------------------------------------------------------- .bem I/O


def write_bem(scene: Scene, directory: str, solver: str = "gmres 1 0", analysis: int = 3):
    """Writes input.bem, nodes.bem, elems.bem and bcs.bem in the reference's
    formats (src/depSolver.c:98-237)."""
    import os
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "nodes.bem"), "w") as f:
        for i, x in enumerate(scene.nodes):
            f.write(f"{i + 1}\t{x[0]:.17e}\t{x[1]:.17e}\t{x[2]:.17e}\n")
    with open(os.path.join(directory, "elems.bem"), "w") as f:
        for i, e in enumerate(scene.elems):
            f.write(f"{i + 1}\t" + "\t".join(str(int(v)) for v in e) + "\n")
    with open(os.path.join(directory, "bcs.bem"), "w") as f:
        for j in range(2 * scene.N):
            t = int(scene.bctype[j])
            if t in (0, 6):
                f.write(f"{j + 1}\t{t}\t{scene.mbc[j, 0]:.17e}\t{int(scene.mbc[j, 1])}\n")
            else:
                f.write(f"{j + 1}\t{t}\t{scene.mbc[j, 0]:.17e}\n")
    etype = {3: "tria3", 6: "tria6", 8: "quad8"}[scene.nen]
    with open(os.path.join(directory, "input.bem"), "w") as f:
        f.write(f"NODES\n{scene.N}\nnodes.bem\n\nELEMS\n{scene.E}\n{etype}\nelems.bem\n\n")
        f.write(f"MATERIALS\n{scene.mat.shape[0]}\n")
        for k, (s, e) in enumerate(scene.mat):
            f.write(f"{k + 1}\t{s:.17e}\t{e:.17e}\n")
        f.write(f"\nINTERFACES\n{scene.n_if}\n")
        for k, (a, b) in enumerate(scene.ifaces):
            f.write(f"{k + 1}\t{a}\t{b}\n")
        f.write(f"\nPROBLEMS\n{scene.freq:.17e}\nbcs.bem\n\nANALYSIS\n{solver}\n{analysis}\n\n")
        f.write("INTERNALPOINTS\n0\n\nCOLUMNS\n0\n")


def _strip_comments(text: str) -> str:
    return "\n".join(line.split("//")[0] for line in text.splitlines())


def read_bem(directory: str) -> Scene:
    """Reads a reference input deck (NODES, ELEMS, MATERIALS, INTERFACES,
    PROBLEM(S) sections; src/depSolver.c:98-237, `//` comments stripped as
    comFilter does, src/preProcess.c:48-81)."""
    import os
    toks = _strip_comments(open(os.path.join(directory, "input.bem")).read()).split()
    it = iter(toks)
    next(it); n_nodes = int(next(it)); node_file = next(it)
    next(it); n_el = int(next(it)); etype = next(it).lower(); elem_file = next(it)
    next(it); n_mat = int(next(it))
    mat = []
    for _ in range(n_mat):
        next(it); mat.append([float(next(it)), float(next(it))])
    next(it); n_if = int(next(it))
    ifaces = []
    for _ in range(n_if):
        next(it); ifaces.append([int(next(it)), int(next(it))])
    next(it); freq = float(next(it)); bc_file = next(it)
    nen = 6 if etype.startswith("tria6") else 8 if etype.startswith("quad8") else 3

    def table(fname):
        return _strip_comments(open(os.path.join(directory, fname)).read()).split()

    t = table(node_file)
    nodes = np.array([float(x) for x in t], dtype=np.float64).reshape(n_nodes, 4)[:, 1:]
    t = table(elem_file)
    elems = np.array([int(x) for x in t], dtype=np.int64).reshape(n_el, nen + 1)[:, 1:]
    t = iter(table(bc_file))
    bctype = np.zeros(2 * n_nodes, np.uint32)
    mbc = np.zeros((2 * n_nodes, 3))
    for j in range(2 * n_nodes):
        next(t)
        s = next(t)
        typ = int(s[1:]) + 5 if s[0] in "cC" else int(s)
        bctype[j] = typ
        if 2 < typ < 6:
            mbc[j] = [float(next(t)), float(next(t)), float(next(t))]
        elif typ in (0, 6):
            mbc[j, :2] = [float(next(t)), float(next(t))]
        else:
            mbc[j, 0] = float(next(t))
    return Scene(nen, nodes, elems.astype(np.uint32), bctype, mbc,
                 np.asarray(ifaces, np.uint32).reshape(-1, 2), np.asarray(mat), freq,
                 os.path.basename(os.path.normpath(directory))).contiguous()
