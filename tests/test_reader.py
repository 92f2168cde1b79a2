"""The input-deck reader and the node normals as library calls (host code,
no GPU): dsc_bem_read against decks written from the scene generator and
against the reference's own example decks (where the reference tree is
present), dsc_node_normals against the oracle's getNormal restatement
(src/normals.c:120-319) and, where present, the reference's own."""
import os

import numpy as np
import pytest

from conftest import REFERENCE
from depsolver_gb300 import api, scenes


@pytest.mark.parametrize("nen", [6, 3])
def test_reader_round_trip(native, tmp_path, nen):
    sc = scenes.small(nen=nen)
    scenes.write_bem(sc, str(tmp_path), solver="gmres 1 0", analysis=3)
    d = api.read_bem(str(tmp_path))
    assert d["nen"] == nen and d["analysis"] == 3 and d["gmres"] and d["precond"] == 1
    assert np.array_equal(d["nodes"], sc.nodes) and np.array_equal(d["elems"], sc.elems)
    assert np.array_equal(d["bctype"], sc.bctype) and np.array_equal(d["mbc"][:, :2], sc.mbc[:, :2])
    assert np.array_equal(d["mat"], sc.mat) and np.array_equal(d["ifaces"], sc.ifaces)
    assert d["freq"] == sc.freq and not d["reposition"]


def test_reader_comments_reposition_and_points(native, tmp_path):
    """'//' comments, a REPOSITION section (nodes pNodes.. shifted as
    depSolver-sft does), C<k> boundary types and an internal-point file."""
    sc = scenes.small(nen=6)
    scenes.write_bem(sc, str(tmp_path))
    text = open(tmp_path / "input.bem").read()
    p0 = sc.particles[0][0]
    text = text.replace("bcs.bem\n\nANALYSIS", f"bcs.bem   // the boundary conditions\n\n"
                                                f"REPOSITION\n{p0}\n0.1 -0.2 0.25\n\nANALYSIS")
    text = text.replace("INTERNALPOINTS\n0", "INTERNALPOINTS\n3 STD\ninternal.bem")
    open(tmp_path / "input.bem", "w").write("// a deck\n" + text)
    open(tmp_path / "internal.bem", "w").write("1 0.0 0.0 0.5\n2 1.0 1.0 1.0 // mid\n3 -1 2 3\n")
    bcs = open(tmp_path / "bcs.bem").read().splitlines()
    first = bcs[0].split()
    assert first[1] == "1"
    bcs[0] = "\t".join([first[0], "C-4"] + first[2:])   # C<k> = k + 5: C-4 is type 1
    open(tmp_path / "bcs.bem", "w").write("\n".join(bcs) + "\n")
    d = api.read_bem(str(tmp_path))
    shifted = scenes.shifted(sc, p0, (0.1, -0.2, 0.25))
    assert d["reposition"] and d["pnodes"] == p0 and np.allclose(d["dr"], [0.1, -0.2, 0.25])
    assert np.array_equal(d["nodes"], shifted.nodes)
    assert np.array_equal(d["bctype"], sc.bctype)
    assert np.array_equal(d["internal"], [[0, 0, 0.5], [1, 1, 1], [-1, 2, 3]])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "examples")),
                    reason="reference examples not present")
@pytest.mark.parametrize("deck", ["capacitor-1/quadratic", "capacitor-2/linear", "dep-trap-1/std",
                                  "dep-trap-2"])
def test_reader_reads_reference_examples(native, deck):
    """The reference's own example decks: the library's reader gives what
    the scene reader of the tests gives, internal points included."""
    dr = os.path.join(REFERENCE, "examples", deck)
    d = api.read_bem(dr)
    sc = scenes.read_bem(dr)
    assert np.array_equal(d["nodes"], sc.nodes) or d["reposition"]
    assert np.array_equal(d["elems"], sc.elems) and np.array_equal(d["bctype"], sc.bctype)
    assert np.array_equal(d["mbc"], sc.mbc) and d["freq"] == sc.freq
    if deck == "dep-trap-1/std":
        assert d["internal"].shape == (2646, 3)
    if deck == "dep-trap-2":
        assert d["reposition"]
        assert np.array_equal(d["nodes"], scenes.shifted(sc, int(d["pnodes"]), d["dr"]).nodes)


@pytest.mark.parametrize("nen", [6, 3])
def test_node_normals_match_oracle(native, port, nen):
    sc = scenes.small(nen=nen)
    n = api.node_normals(sc)
    ref = np.array([port.node_normal(sc, i) for i in range(sc.N)])
    assert np.abs(n - ref).max() < 1e-14


def test_node_normals_match_reference(native, ref):
    sc = scenes.small(nen=6)
    n = api.node_normals(sc)
    for i in range(0, sc.N, 7):
        assert np.abs(n[i] - ref.node_normal(sc, i)).max() < 1e-14, i
