"""The oracle's pattern and slot map on the apps' TetGen meshes (bunny.1 and
dragon40k, tets and the bunny's .edge springs) equal the reference's own
PathIndexBuilder and `loc` (digests recorded from oracle/_ref)."""
import numpy as np
import pytest

from tests import scenarios


@pytest.mark.parametrize("name,xkey,epkey,card", [
    ("bunny_tets", "bunny_x", "bunny_tets", 4),
    ("bunny_edges", "bunny_x", "bunny_edges", 2),
    ("dragon_tets", "dragon_x", "dragon_tets", 4),
])
def test_oracle_pattern_matches_reference_builder(oracle, name, xkey, epkey, card):
    meshes, dig = scenarios.tetmeshes()
    g = dig[name]
    x, ep = meshes[xkey], meshes[epkey]
    n = len(x) // 3
    assert (n, len(ep) // card) == (g["n"], g["nE"])
    rp, ci = oracle.pattern(n, ep, card)
    assert len(ci) == g["nnzb"]
    assert scenarios.sha(rp) == g["rowptr_sha256"]
    assert scenarios.sha(ci) == g["colidx_sha256"]
    sl = oracle.slots(ep, card, rp, ci)
    assert scenarios.sha(sl) == g["slots_sha256"]


def test_bunny_edges_are_the_tet_edges():
    """bunny.1.edge lists every edge of bunny.1.ele once, so both edge sets
    give one pattern (the reference's builder agrees)."""
    meshes, dig = scenarios.tetmeshes()
    t = meshes["bunny_tets"].reshape(-1, 4)
    pairs = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)])
    pairs = np.unique(np.sort(pairs, 1), axis=0)
    e = np.unique(np.sort(meshes["bunny_edges"].reshape(-1, 2), 1), axis=0)
    assert np.array_equal(pairs, e)
    assert dig["bunny_edges"]["colidx_sha256"] == dig["bunny_tets"]["colidx_sha256"]
