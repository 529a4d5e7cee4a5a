"""Inputs of the reference's own program tests, rebuilt as arrays.

Each builder mirrors the set construction of one reference test so that the
oracle and the GPU path can replay it and compare with its golden values.
"""
import hashlib
import json
import os
import re

import numpy as np

from simit_gb300 import meshgen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_map():
    with open(os.path.join(GOLDEN, "reference_golden.json")) as f:
        return json.load(f)


def golden(name):
    with open(os.path.join(GOLDEN, "reference_golden.json")) as f:
        return json.load(f)[name]


def golden_lookup(entry, fields):
    """Value the golden entry's expression refers to, e.g. 'v(p1)(2)',
    '(simit_float)c.get(p0)' or 'x.get(vertRefs[100])(0)'."""
    e = entry["expr"].replace("(simit_float)", "")
    m = re.match(r"(\w+)\(p(\d+)\)\((\d)\)$", e)
    if m:
        return fields[m.group(1)][int(m.group(2)) * 3 + int(m.group(3))]
    m = re.match(r"(\w+)\.get\(p(\d+)\)$", e)
    if m:
        return fields[m.group(1)][int(m.group(2))]
    m = re.match(r"(\w+)\.get\(vertRefs\[(\d+)\]\)\((\d)\)$", e)
    if m:
        return fields[m.group(1)][int(m.group(2)) * 3 + int(m.group(3))]
    # `TensorRef x1 = x.get(p1); x1(0)`: the points numbered from 1
    m = re.match(r"([a-z])(\d+)\((\d)\)$", e)
    if m:
        return fields[m.group(1)][(int(m.group(2)) - 1) * 3 + int(m.group(3))]
    raise ValueError(e)


def esprings_cube():
    """test/program-esprings-test.cpp:10-150 (TEST(Program, esprings)): the
    8 corners of the unit cube at rest, its 12 edges as springs (mass
    0.0282735, rest length 0.9), 10 runs of test/input/program/esprings.sim
    main: explicit springs, stiffness 3, gravity -9.81 z, h = 0.01."""
    x = np.array([[i & 1, (i >> 1) & 1, (i >> 2) & 1] for i in range(8)], np.float64)
    ends = [(0, 1), (2, 3), (4, 5), (6, 7), (0, 2), (1, 3), (4, 6), (5, 7),
            (0, 4), (1, 5), (2, 6), (3, 7)]
    return {"n": 8, "x": x.reshape(-1), "v": np.zeros(24),
            "ep": np.array(ends, np.int32).reshape(-1), "m": np.full(12, 0.0282735),
            "l0": np.full(12, 0.9), "h": 0.01, "steps": 10}


def esprings_step(s, x, v, fg, M, fs):
    """esprings.sim main after its three maps (numpy or torch arrays):
    p = M .* v + h (fs + fg);  v = p ./ M;  x = x + h v."""
    p = (M * v) + (s["h"] * (fs + fg))
    v = p / M
    return x + (s["h"] * v), v


def isprings_chain():
    """test/program-isprings.cpp:91-146 (TEST(Program, isprings)): 3-point
    vertical chain, p0 fixed (z < 0.4), 10 runs of
    test/input/program/isprings.sim main (h=1e-2, viscous=1e-1, grav -9.81 z,
    CG tol 1e-5 on r'r, 25 iterations)."""
    l0_, stiffness, density, radius, PI_ = 1.0, 100.0, 1000.0, 0.01, 3.14159265358979
    x = np.array([0, 0, 0, 0, 0, 1, 0, 0, 2], np.float64)
    v = np.zeros(9)
    m = np.full(3, PI_ * radius * radius * l0_ * density)
    fixed = np.array([1, 0, 0], np.uint8)
    ep = np.array([0, 1, 1, 2], np.int32)
    return {"n": 3, "x": x, "v": v, "m": m, "fixed": fixed, "ep": ep,
            "k": np.full(2, stiffness), "l0": np.full(2, l0_), "h": 1e-2, "viscous": 1e-1,
            "grav": np.array([0, 0, -9.81]), "tol2": 1e-5, "maxiters": 25, "steps": 10,
            "form": 1}


def cg_chain():
    """test/program-cg-test.cpp:10-44 with test/input/program/cg.sim: 3
    points, b = (1,2,3), springs a = (4,5), A = I - 0.01*K, CG from 0 with
    tol 1e-6 on ||r|| and 5 iterations."""
    return {"n": 3, "ep": np.array([0, 1, 1, 2], np.int32), "a": np.array([4.0, 5.0]),
            "b": np.array([1.0, 2.0, 3.0]), "diag": 1.0, "scale": -0.01, "tol": 1e-6,
            "maxiters": 5}


def femtet_bar2k():
    """test/program-fem-test.cpp:14-106 with test/input/program/femTet.sim:
    bar2k mesh (439 vertices, 1151 tets), E=5e3, nu=0.45, u = 0.5*E/nu,
    l = E*nu/((1+nu)*(1-2nu)), v0 = (0.1, 0, 0.1), vertices with y < 1e-4
    constrained (c=1, v=0); initializeTet then 10 runs of main (h=0.01, CG
    tol 1e-6 on r'r, 100 iterations)."""
    x, tets = meshgen.load_tetgen(os.path.join(GOLDEN, "bar2k.node"),
                                  os.path.join(GOLDEN, "bar2k.ele"))
    n = len(x) // 3
    nT = len(tets) // 4
    E, nu = 5e3, 0.45
    uval = 0.5 * E / nu
    lval = E * nu / ((1 + nu) * (1 - 2 * nu))
    v = np.tile(np.array([0.1, 0.0, 0.1]), n)
    c = np.zeros(n, np.int32)
    ymask = x.reshape(-1, 3)[:, 1] < 0.0001
    c[ymask] = 1
    v.reshape(-1, 3)[ymask] = 0.0
    return {"n": n, "x": x, "v": v, "c": c, "tets": tets, "u": np.full(nT, uval),
            "l": np.full(nT, lval), "h": 0.01, "rho": 1000.0,
            "grav": np.array([0.0, -10.0, 0.0]), "tol2": 1e-6, "maxiters": 100, "steps": 10}


def element_block_scenarios():
    """The small `map f to E reduce +` programs of the reference's gemv and
    assembly tests, with f evaluated here: (name, n, endpoints, bs, element
    blocks [nE, 2, 2, bs, bs], vector x, expected-order labels).  The
    product A x is compared with the golden values in test order
    (c(p0)(0), c(p0)(1), c(p1)(0), ...)."""
    out = []
    b = np.array([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]])
    ep = np.array([0, 1, 1, 2], np.int32)
    a = np.array([[[1.0, 2.0], [3.0, 4.0]], [[5.0, 6.0], [7.0, 8.0]]])
    # test/input/system/gemv_blocked.sim: all four blocks are s.a
    eb = np.zeros((2, 2, 2, 2, 2))
    for s in range(2):
        eb[s, :, :] = a[s]
    out.append(("gemv_blocked", 3, ep, 2, eb, b.reshape(-1)))
    # gemv_blocked_nw.sim: only M(p(0), p(0)) = s.a
    eb = np.zeros((2, 2, 2, 2, 2))
    for s in range(2):
        eb[s, 0, 0] = a[s]
    out.append(("gemv_blocked_nw", 3, ep, 2, eb, b.reshape(-1)))
    # gemv_blocked_computed.sim: all four blocks are p(0).x * p(1).x' (x = b)
    eb = np.zeros((2, 2, 2, 2, 2))
    for s in range(2):
        eb[s, :, :] = np.outer(b[ep[2 * s]], b[ep[2 * s + 1]])
    out.append(("gemv_blocked_computed", 3, ep, 2, eb, b.reshape(-1)))
    # test/input/assembly/matrix_vv.sim: all four (scalar) blocks are 1, a = 1
    eb = np.ones((2, 2, 2, 1, 1))
    out.append(("matrix_vv", 3, ep, 1, eb, np.ones(3)))
    return out


def tet_edges(tets):
    """Unique undirected edges (i < j, sorted) of a tet mesh's elements."""
    t = np.asarray(tets, np.int64).reshape(-1, 4)
    pairs = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)], 0)
    pairs.sort(axis=1)
    return np.unique(pairs, axis=0).astype(np.int32)


def write_tetgen_edges(path, edges):
    """A TetGen .edge file: header "count 1", then "index v0 v1 marker"."""
    with open(path, "w") as f:
        f.write("%d  1\n" % len(edges))
        for i, (a, b) in enumerate(edges):
            f.write("%5d %6d %6d  -1\n" % (i, a, b))
        f.write("# written by tests/scenarios.py\n")


def springs_from_tetgen(node_path, edge_path):
    """apps/springs/springs.cpp:15-90 on TetGen files: positions normalised to
    [0, 1] per axis, points below z = 0.1 fixed, one spring per .edge record
    with k = 1e4, l0 its rest length and half its mass (pi r^2 l0 * 1e3,
    r = 0.01) on each endpoint; apps/springs/isprings.sim constants (h = 1e-2,
    viscous = 2, gravity -9.81 y, CG while r'r > 1e-12, at most 50 steps)."""
    x = meshgen.parse_tetgen_nodes(open(node_path).read())
    ep = meshgen.load_tetgen_edges(edge_path)
    return springs_from_arrays(x, ep)


def springs_from_arrays(x, ep):
    """springs_from_tetgen on positions [n*3] and edge endpoints [nE*2]
    already read from TetGen files."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    ep = np.asarray(ep, np.int32).reshape(-1, 2)
    mn, mx = x.min(0), x.max(0)
    x = (x - mn) / (mx - mn)
    d = x[ep[:, 1]] - x[ep[:, 0]]
    l0 = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    mass = (3.14159265358979 * 0.01 * 0.01 * l0) * 1e3
    m = np.zeros(len(x))
    for (a, b), ms in zip(ep, mass):  # element order, as the reference's loop
        m[a] += 0.5 * ms
        m[b] += 0.5 * ms
    return {"n": len(x), "x": x.reshape(-1), "v": np.zeros(x.size), "m": m,
            "fixed": (x[:, 2] < 0.1).astype(np.uint8), "ep": ep.reshape(-1).astype(np.int32),
            "k": np.full(len(ep), 1e4), "l0": l0, "h": 1e-2, "viscous": 2.0,
            "grav": np.array([0.0, -9.81, 0.0]), "tol2": 1e-12, "maxiters": 50, "form": 0}


def tetmeshes():
    """The apps' TetGen meshes (bunny.1, dragon40k) as read from their
    .node/.ele/.edge files, and the digests of the reference
    PathIndexBuilder's pattern and `loc` slot map for each edge set."""
    z = np.load(os.path.join(GOLDEN, "tetmeshes.npz"))
    meshes = {k: z[k] for k in z.files}
    with open(os.path.join(GOLDEN, "tetmeshes_golden.json")) as f:
        digests = json.load(f)
    return meshes, digests


def sha(a, dtype=np.uint32):
    """SHA-256 of an integer array as little-endian `dtype` bytes (the digest
    tests/golden/make_golden.py records)."""
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.dtype(dtype).newbyteorder("<"))
                          .tobytes()).hexdigest()


def incidence_scenarios():
    """The four incidence-matrix programs of test/assembly-tests.cpp as
    (kind, n, sel, npos, element blocks, vector, expected result, name):
    matrix_ve / matrix_ev (test/input/assembly/matrix_{ve,ev}.sim: every
    write is 1; c = A * E.a and E.a = A * V.c) and their heterogeneous forms
    (an edge set over (V1, V1, V0, V1, V1): the V0 matrix takes endpoint 2,
    the V1 matrix endpoints 0, 1, 3, 4 with writes 1, 2, 3, 4)."""
    g = {k: v for k, v in _golden_map().items() if k.startswith("incidence_")}
    out = []
    ep2 = np.array([[0, 1], [1, 2]])
    exp = [a["expected"] for a in g["incidence_matrix_ve"]["asserts"]]
    out.append((1, 3, ep2, 2, np.ones((2, 2)), np.array([1.0, 2.0]), exp, "matrix_ve"))
    exp = [a["expected"] for a in g["incidence_matrix_ev"]["asserts"]]
    out.append((0, 3, ep2, 2, np.ones((2, 2)), np.array([1.0, 2.0, 3.0]), exp, "matrix_ev"))
    het = np.array([[0, 1, 0, 3, 4], [1, 2, 1, 4, 5], [3, 4, 2, 6, 7], [4, 5, 3, 7, 8]])
    v0, v1 = het[:, [2]], het[:, [0, 1, 3, 4]]
    w1 = np.tile(np.array([1.0, 2.0, 3.0, 4.0]), (4, 1))
    gv = g["incidence_matrix_ve_heterogeneous"]["vectors"]
    ea = np.array([1.0, 2.0, 3.0, 4.0])
    out.append((1, 4, v0, 1, np.ones((4, 1)), ea, gv["b0_loop"], "matrix_ve_heterogeneous V0"))
    out.append((1, 9, v1, 4, w1, ea, gv["b1Expected"], "matrix_ve_heterogeneous V1"))
    ga = [a["expected"] for a in g["incidence_matrix_ev_heterogeneous"]["asserts"]]
    out.append((0, 4, v0, 1, np.ones((4, 1)), np.arange(1.0, 5.0), ga[:4],
                "matrix_ev_heterogeneous V0"))
    out.append((0, 9, v1, 4, w1, np.arange(1.0, 10.0), ga[4:], "matrix_ev_heterogeneous V1"))
    return out


def rect_scenarios():
    """matrix_vv_heterogeneous of test/assembly-tests.cpp
    (test/input/assembly/matrix_vv_heterogeneous.sim): over
    Set E(V1,V1,V0,V1,V1), A01 = matrix[V0,V1] with Ae(v0, vk) = k and
    A10 = matrix[V1,V0] with Ae(vk, v0) = k (k = 1..4); V0.b = A01 * V1.a and
    V1.b = A10 * V0.a with a = i + 1.  Items: (nr, nc, sel_r, npos_r, sel_c,
    npos_c, blocks [nE, npos_r, npos_c], vector, expected, name)."""
    g = _golden_map()["incidence_matrix_vv_heterogeneous"]["vectors"]
    het = np.array([[0, 1, 0, 3, 4], [1, 2, 1, 4, 5], [3, 4, 2, 6, 7], [4, 5, 3, 7, 8]])
    v0, v1 = het[:, [2]], het[:, [0, 1, 3, 4]]
    w = np.array([1.0, 2.0, 3.0, 4.0])
    return [(4, 9, v0, 1, v1, 4, np.tile(w, (4, 1)).reshape(4, 1, 4), np.arange(1.0, 10.0),
             g["b0Expected"], "A01 * V1.a"),
            (9, 4, v1, 4, v0, 1, np.tile(w, (4, 1)).reshape(4, 4, 1), np.arange(1.0, 5.0),
             g["b1Expected"], "A10 * V0.a")]
