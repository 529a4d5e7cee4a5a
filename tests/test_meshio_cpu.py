"""TetGen mesh ingestion (MeshVol::loadTet / loadTetEdge, src/mesh.cpp:231-373)
against the texts and asserted values of the reference's test/mesh-test.cpp
(TetgenTest, TetgenEdgeTest), extracted into tests/golden/tetgen_golden.json."""
import json
import os
import re

import numpy as np

from simit_gb300 import meshgen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden():
    with open(os.path.join(GOLDEN, "tetgen_golden.json")) as f:
        return json.load(f)


def _check(asserts, arrays):
    for a in asserts:
        m = re.match(r"m\.(\w+)\[(\d+)\]\[(\d+)\]", a["expr"])
        name, i, j = m.group(1), int(m.group(2)), int(m.group(3))
        assert arrays[name][i, j] == a["expected"], a


def test_tetgen_node_ele_golden():
    g = _golden()["TetgenTest"]
    x = meshgen.parse_tetgen_nodes(g["texts"]["inputNode"])
    e = meshgen.parse_tetgen_elements(g["texts"]["inputEle"])
    assert x.shape == (20, 3) and e.shape == (24, 4)
    assert len(g["asserts"]) == 5
    _check(g["asserts"], {"v": x, "e": e})


def test_tetgen_edge_golden():
    g = _golden()["TetgenEdgeTest"]
    ed = meshgen.parse_tetgen_edges(g["texts"]["inputEdge"])
    assert ed.shape == (24, 2)
    assert len(g["asserts"]) == 3
    _check(g["asserts"], {"edges": ed})


def test_tetgen_reader_rules(tmp_path):
    """Comment and short lines are skipped, the boundary-marker column is
    ignored, a last line without a newline is not read (the reference stops
    at end-of-stream), and missing records stay zero."""
    text = "3 1\n# comment\n\n0  4 7 -1\n  \n1  2 9 0\n2  5 6 -1"
    ed = meshgen.parse_tetgen_edges(text)
    assert ed.tolist() == [[4, 7], [2, 9], [0, 0]]
    ed = meshgen.parse_tetgen_edges(text + "\n")
    assert ed.tolist() == [[4, 7], [2, 9], [5, 6]]
    p = tmp_path / "m.edge"
    p.write_text(text + "\n")
    assert meshgen.load_tetgen_edges(str(p)).tolist() == [4, 7, 2, 9, 5, 6]


def test_bar2k_fixture_counts():
    x, tets = meshgen.load_tetgen(os.path.join(GOLDEN, "bar2k.node"),
                                  os.path.join(GOLDEN, "bar2k.ele"))
    assert x.shape == (439 * 3,) and tets.shape == (1151 * 4,)
    assert tets.min() == 0 and tets.max() == 438
    assert np.all(np.isfinite(x))
