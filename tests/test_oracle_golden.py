"""Pin the oracle: reference golden values and the reference's own pattern code.

CPU only (no GPU marker).  Tolerance 1e-13 absolute, as SIMIT_ASSERT_FLOAT_EQ
in FP64 (test/simit-test.h:36-48).
"""
import json
import os

import numpy as np
import pytest

from simit_gb300 import meshgen
from tests import scenarios

GOLD_TOL = 1e-13


def test_isprings_golden(oracle):
    s = scenarios.isprings_chain()
    x, v = s["x"].copy(), s["v"].copy()
    rp, ci = oracle.pattern(s["n"], s["ep"], 2)
    for _ in range(s["steps"]):
        oracle.springs_step(s["form"], x, v, s["m"], s["fixed"], s["ep"], s["k"], s["l0"],
                            s["h"], s["viscous"], s["grav"], rp, ci, s["tol2"], s["maxiters"])
    for g in scenarios.golden("isprings"):
        got = scenarios.golden_lookup(g, {"x": x, "v": v})
        assert abs(got - g["expected"]) <= GOLD_TOL, (g, got)


def test_cg_golden(oracle):
    s = scenarios.cg_chain()
    rp, ci = oracle.pattern(s["n"], s["ep"], 2)
    A = oracle.scalar_springs_assemble(s["n"], s["ep"], s["a"], s["diag"], s["scale"], rp, ci)
    c, it = oracle.cg_norm(s["n"], 1, rp, ci, A, s["b"], s["tol"], s["maxiters"])
    for g in scenarios.golden("cg"):
        got = scenarios.golden_lookup(g, {"c": c})
        assert abs(got - g["expected"]) <= GOLD_TOL, (g, got)


def test_femtet_golden(oracle):
    s = scenarios.femtet_bar2k()
    assert s["n"] == 439 and len(s["tets"]) // 4 == 1151
    x, v = s["x"].copy(), s["v"].copy()
    B, W, m = oracle.tet_precompute(x, s["tets"], s["rho"])
    rp, ci = oracle.pattern(s["n"], s["tets"], 4)
    for _ in range(s["steps"]):
        oracle.tet_step(1, x, v, s["c"], s["tets"], B, W, s["u"], s["l"], s["h"], s["rho"],
                        s["grav"], rp, ci, s["tol2"], s["maxiters"])
    for g in scenarios.golden("femTet"):
        got = scenarios.golden_lookup(g, {"x": x})
        assert abs(got - g["expected"]) <= GOLD_TOL, (g, got)


def test_pattern_golden_fixtures(oracle):
    """Pattern + slot map equal the reference's PathIndexBuilder / loc output
    committed in tests/golden/pattern_golden.json."""
    with open(os.path.join(scenarios.GOLDEN, "pattern_golden.json")) as f:
        cases = json.load(f)
    for name, c in cases.items():
        ep = np.array(c["endpoints"], np.int32)
        rp, ci = oracle.pattern(c["n"], ep, c["card"])
        assert rp.tolist() == c["rowptr"], name
        assert ci.tolist() == c["colidx"], name
        assert oracle.slots(ep, c["card"], rp, ci).tolist() == c["slots"], name


def test_pattern_reference_test_vectors(oracle):
    """VERIFY_INDEX lists of test/path_indices-test.cpp: exist_and (vev on a
    3-point chain, :155-174) and alias (two opposite edges, :309-332)."""
    ep, n = meshgen.box_springs(3, 1, 1)
    rp, ci = oracle.pattern(n, ep, 2)
    rows = [ci[rp[i]:rp[i + 1]].tolist() for i in range(n)]
    assert rows == [[0, 1], [0, 1, 2], [1, 2]]
    rp, ci = oracle.pattern(2, np.array([0, 1, 1, 0], np.int32), 2)
    assert [ci[rp[i]:rp[i + 1]].tolist() for i in range(2)] == [[0, 1], [0, 1]]
    # a vertex with no edge gets an empty row (src/path_indices.cpp:359-429)
    rp, ci = oracle.pattern(4, np.array([0, 1], np.int32), 2)
    assert rp.tolist() == [0, 2, 4, 4, 4]


@pytest.mark.parametrize("card,n,nE,seed", [(2, 50, 120, 1), (3, 64, 90, 2), (4, 80, 150, 3),
                                            (4, 30, 200, 4), (1, 10, 7, 5)])
def test_pattern_matches_reference_builder(oracle, card, n, nE, seed):
    """Random edge sets (duplicate endpoints inside an element included)
    against the reference's own builder compiled from its sources."""
    if not os.path.exists(oracle.REF_LIB):
        pytest.skip("reference pattern builder not built here (no reference sources)")
    ep = meshgen.rng(seed).integers(0, n, size=nE * card).astype(np.int32)
    rp, ci = oracle.pattern(n, ep, card)
    r2, c2 = oracle.ref_pattern(n, ep, card)
    assert np.array_equal(rp, r2) and np.array_equal(ci, c2)
    assert np.array_equal(oracle.slots(ep, card, rp, ci), oracle.ref_slots(ep, card, rp, ci))


def test_tet_grid_counts(oracle):
    """5-tet lattice sizes; 16^3 nnzb 58,769 as computed for the 16^3 config."""
    m = meshgen.tet_grid(16)
    assert (m["n"], len(m["tets"]) // 4) == (4913, 20480)
    rp, ci = oracle.pattern(m["n"], m["tets"], 4)
    assert len(ci) == 58769
    B, W, _ = oracle.tet_precompute(m["x"], m["tets"], 1e3)
    assert W.min() > 0 and abs(W.sum() - 1.0) < 1e-12


def test_tet_grid_48_pattern_matches_reference_builder(oracle):
    """The 48^3 lattice (552,960 tets, 117,649 vertices): nnzb 1,486,513, and
    the oracle's pattern equal to the reference's PathIndexBuilder's."""
    m = meshgen.tet_grid(48)
    assert (m["n"], len(m["tets"]) // 4) == (117649, 552960)
    assert meshgen.tet_grid_counts(48) == (552960, 117649)
    rp, ci = oracle.pattern(m["n"], m["tets"], 4)
    assert len(ci) == 1486513
    ref = oracle.ref_pattern(m["n"], m["tets"], 4)
    if ref is None:
        pytest.skip("reference pattern builder not built here")
    assert np.array_equal(rp, ref[0]) and np.array_equal(ci, ref[1])


def test_element_block_assembly_golden(oracle):
    """Oracle `map ... reduce +` of caller-evaluated element blocks, then the
    blocked SpMV, against the golden values of the reference's gemv_blocked*
    (test/system-gemv-tests.cpp) and matrix_vv (test/assembly-tests.cpp)."""
    from tests import scenarios
    for name, n, ep, bs, eb, x in scenarios.element_block_scenarios():
        rp, ci = oracle.pattern(n, ep, 2)
        vals = oracle.assemble_blocks(ep, 2, bs, eb, rp, ci)
        y = oracle.spmv(n, bs, rp, ci, vals, x)
        want = [g["expected"] for g in scenarios.golden(name)]
        assert list(y) == want, (name, list(y), want)


def test_add_diag_semantics(oracle):
    """The oracle's `MDK = MD + K` (apps/springs/isprings.sim:74) on a hand
    case: rows {0: cols 0, 1}, {1: col 1}; diagonal slots get D + s*K, the
    others 0 + s*K (a -0 becomes +0), ident*I when no array is given."""
    rp = np.array([0, 2, 3], np.uint32)
    ci = np.array([0, 1, 1], np.uint32)
    K = np.array([1.0, -0.0, 3.0])
    out = oracle.add_diag(2, 1, rp, ci, K, diag=np.array([10.0, 20.0]))
    assert out.tolist() == [11.0, 0.0, 23.0] and not np.signbit(out[1])
    out = oracle.add_diag(2, 1, rp, ci, K, ident=2.0, scale=-0.5)
    assert out.tolist() == [1.5, 0.0, 0.5]
    # 3x3 blocks: the identity lands on each diagonal block's diagonal only
    K3 = np.zeros(27)
    out = oracle.add_diag(2, 3, rp, ci, K3, ident=1.0)
    blocks = out.reshape(3, 3, 3)
    assert np.array_equal(blocks[0], np.eye(3)) and np.array_equal(blocks[2], np.eye(3))
    assert not blocks[1].any()
    # the springs oracle's fused MD + K is this expression of its own parts
    L = meshgen.springs_lattice(4, 4, 4, 0.1, 0.01, seed=2)
    n, ep = L["n"], L["ep"]
    rp, ci = oracle.pattern(n, ep, 2)
    g = meshgen.rng(3)
    v, m = g.uniform(-0.1, 0.1, n * 3), g.uniform(0.5, 2.0, n)
    k, l0 = np.full(len(L["l0"]), 1e4), L["l0"] * 1.05
    fixed, grav = np.zeros(n, np.uint8), np.array([0, 0, -9.81])
    fused, _ = oracle.springs_assemble(0, L["x"], v, m, fixed, ep, k, l0, 1e-3, 0.5, grav, rp, ci)
    K, _ = oracle.springs_assemble(0, L["x"], v, np.zeros(n), fixed, ep, k, l0, 1e-3, 0.0, grav,
                                   rp, ci)
    MD = ((m + 1e-3 * 0.5)[:, None, None] * np.eye(3)[None]).reshape(-1)
    assert np.array_equal(oracle.add_diag(n, 3, rp, ci, K, diag=MD), fused)


@pytest.mark.parametrize("case", range(6))
def test_incidence_matrices_golden(oracle, case):
    """Link::ev / Link::ve patterns and the `map` into them (the oracle's
    restatement) reproduce test/assembly-tests.cpp's matrix_ve, matrix_ev
    and heterogeneous results (A * field)."""
    kind, n, sel, npos, eb, vec, expected, name = scenarios.incidence_scenarios()[case]
    rp, ci = oracle.incidence_pattern(kind, n, sel, npos)
    vals = oracle.assemble_incidence(kind, sel, npos, 1, eb, rp, ci)
    rows = len(rp) - 1
    y = oracle.spmv(rows, 1, rp, ci, vals, vec)
    assert y.tolist() == [float(v) for v in expected], name


@pytest.mark.parametrize("case", range(2))
def test_rect_matrix_golden(oracle, case):
    """∃e.(v0-e ∧ e-v1) between two vertex sets (the oracle's restatement)
    reproduces test/assembly-tests.cpp's matrix_vv_heterogeneous results."""
    nr, nc, sr, npr, sc, npc, eb, vec, expected, name = scenarios.rect_scenarios()[case]
    rp, ci = oracle.rect_pattern(nr, sr, npr, sc, npc)
    vals = oracle.assemble_rect(sr, npr, sc, npc, 1, eb, rp, ci)
    y = oracle.spmv(nr, 1, rp, ci, vals, vec)
    assert y.tolist() == [float(v) for v in expected], name


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_incidence_and_rect_patterns_match_reference_builder(oracle, seed):
    """The oracle's Link::ev / Link::ve / two-set And restatements against
    the reference's own PathIndexBuilder (compiled from its sources), bit for
    bit, on heterogeneous edge sets (V1, V1, V0, V1, V1) with repeats and on
    a homogeneous one."""
    if not os.path.exists(oracle.REF_LIB):
        pytest.skip("reference pattern builder not built here")
    g = meshgen.rng(90 + seed)
    for set_of, n0, n1, nE in (([1, 1, 0, 1, 1], 6, 20, 40), ([0, 0, 0], 25, 1, 60)):
        card = len(set_of)
        ep = np.stack([g.integers(0, n1 if s else n0, size=nE) for s in set_of], 1)
        ep[::5, 1] = ep[::5, 0]  # repeated endpoints
        for x in sorted(set(set_of)):
            pos = [k for k in range(card) if set_of[k] == x]
            sel = ep[:, pos]
            nx = n1 if x else n0
            for kind in (0, 1):
                ref = oracle.ref_incidence(kind, n0, n1, set_of, ep, xr=x, xc=x)
                got = oracle.incidence_pattern(kind, nx, sel, len(pos))
                assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
        if 0 in set_of and 1 in set_of:
            for xr, xc in ((0, 1), (1, 0)):
                pr = [k for k in range(card) if set_of[k] == xr]
                pc = [k for k in range(card) if set_of[k] == xc]
                ref = oracle.ref_incidence(2, n0, n1, set_of, ep, xr=xr, xc=xc)
                got = oracle.rect_pattern(n1 if xr else n0, ep[:, pr], len(pr), ep[:, pc],
                                          len(pc))
                assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])


def test_incidence_slots_match_reference_loc(oracle):
    """The slot every element write lands in under the oracle's incidence
    assembly is the one the reference runtime's own `loc` returns
    (src/runtime.cpp:19-23: the first matching column of the row), for EV
    and VE patterns with repeated endpoints."""
    import ctypes
    if not os.path.exists(oracle.REF_LIB):
        pytest.skip("reference pattern builder not built here")
    L = ctypes.CDLL(oracle.REF_LIB)
    L.loc.restype = ctypes.c_int
    L.loc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    g = meshgen.rng(55)
    n, nE, npos = 30, 80, 3
    sel = g.integers(0, n, size=(nE, npos))
    sel[::4, 2] = sel[::4, 0]
    for kind in (0, 1):
        rp, ci = oracle.incidence_pattern(kind, n, sel, npos)
        rpi, cii = rp.astype(np.int32), ci.astype(np.int32)
        # unit blocks mark which slot each (element, listing) write lands in
        for e in range(nE):
            for k in range(npos):
                eb = np.zeros((nE, npos))
                eb[e, k] = 1.0
                vals = oracle.assemble_incidence(kind, sel, npos, 1, eb, rp, ci)
                r, c = (e, int(sel[e, k])) if kind == 0 else (int(sel[e, k]), e)
                q = L.loc(r, c, rpi.ctypes.data, cii.ctypes.data)
                assert int(np.flatnonzero(vals)[0]) == q
