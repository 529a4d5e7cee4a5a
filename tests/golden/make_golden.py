"""Regenerate the golden fixtures in this directory from the reference tree.

Run with the reference checkout as the first argument (or SIMIT_REFERENCE,
or a checkout beside this repository); the machines that run the tests need
not have it, so the outputs are committed.  `make_golden.py [REF] lattice`
rewrites only lattice_golden.json.



  reference_golden.json   golden values asserted by the reference's tests,
                          extracted from their sources (file:line recorded),
                          including the incidence-matrix assembly tests
  bar2k.node, bar2k.ele   the TetGen fixture test/program-fem-test.cpp loads
  cube.node, cube.ele     the 8-vertex TetGen fixture test/reorder-tests.cpp's
                          reorderCube loads
  tetgen_golden.json      the TetGen .node/.ele/.edge texts of
                          test/mesh-test.cpp (TetgenTest, TetgenEdgeTest)
                          with the values those tests assert
  pattern_golden.json     pattern + slot map of small meshes produced by the
                          reference's own PathIndexBuilder / `loc`
                          (oracle/_ref/libref_pattern.so)
  tetmeshes.npz           the apps' TetGen meshes (apps/data/tet-bunny/bunny.1
                          .node/.ele/.edge, apps/data/tet-dragon/dragon40k
                          .node/.ele) as read by MeshVol::loadTet /
                          loadTetEdge's rules (simit_gb300.meshgen)
  tetmeshes_golden.json   per mesh: sizes and SHA-256 digests of the
                          reference PathIndexBuilder's rowptr / colidx and of
                          the `loc` slot map, for the tets and for the springs
                          over the bunny's edges
  lattice_golden.json     the same digests for the benchmark configurations'
                          five-tet lattices: 64^3 (lattice order), 128^3
                          (lattice order) and 128^3 in the workload's Morton
                          order
"""
import hashlib
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
# the reference checkout: the first argument, else SIMIT_REFERENCE, else a
# checkout beside this repository
REF = (sys.argv[1] if len(sys.argv) > 1 and os.path.isdir(sys.argv[1])
       else os.environ.get("SIMIT_REFERENCE", os.path.join(os.path.dirname(REPO), "reference")))


def sha(a, dtype):
    """SHA-256 of an integer array as little-endian `dtype` bytes."""
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.dtype(dtype).newbyteorder("<"))
                          .tobytes()).hexdigest()


def extract_asserts(path, test_name):
    """SIMIT_ASSERT_FLOAT_EQ(expected, expr) lines inside TEST(..., test_name)."""
    lines = open(path).read().split("\n")
    out, inside = [], False
    for i, ln in enumerate(lines, 1):
        m = re.match(r"TEST\((\w+),\s*(\w+)\)", ln)
        if m:
            inside = m.group(2) == test_name
            continue
        if inside:
            a = re.search(r"SIMIT_ASSERT_FLOAT_EQ\(\s*([-0-9.eE+]+)\s*,\s*(.*)\);", ln)
            if a:
                out.append({"expected": float(a.group(1)), "expr": a.group(2).strip(),
                            "source": "%s:%d" % (os.path.relpath(path, REF), i)})
    return out


def extract_assert_eq(path, test_name):
    """ASSERT_EQ(expected, expr) lines inside TEST(..., test_name)."""
    lines = open(path).read().split("\n")
    out, inside = [], False
    for i, ln in enumerate(lines, 1):
        m = re.match(r"TEST\((\w+),\s*(\w+)\)", ln)
        if m:
            inside = m.group(2) == test_name
            continue
        if inside:
            a = re.search(r"ASSERT_EQ\(\s*([-0-9.eE+]+)\s*,\s*(.*)\);", ln)
            if a:
                out.append({"expected": float(a.group(1)), "expr": a.group(2).strip(),
                            "source": "%s:%d" % (os.path.relpath(path, REF), i)})
    return out


def extract_raw_strings(path, test_name):
    """The R"(...)" string constants inside TEST(..., test_name), by name."""
    src = open(path).read()
    m = re.search(r"TEST\(\w+,\s*%s\)\s*\{" % test_name, src)
    body = src[m.end():]
    nxt = re.search(r"\nTEST\(", body)
    body = body[:nxt.start()] if nxt else body
    return {k: v for k, v in re.findall(r"string\s+(\w+)\s*=\s*R\"\((.*?)\)\";", body, re.S)}


def extract_incidence_asserts(path, test_name):
    """Expected ints of TEST(..., test_name) in test/assembly-tests.cpp, in
    either ASSERT_EQ order, plus `const std::vector<int> name = {...}`."""
    src = open(path).read()
    m = re.search(r"TEST\(\w+,\s*%s\)\s*\{" % test_name, src)
    start = src[:m.start()].count("\n") + 1
    body = src[m.end():]
    nxt = re.search(r"\nTEST\(", body)
    body = body[:nxt.start()] if nxt else body
    out = {"source": "%s:%d" % (os.path.relpath(path, REF), start), "asserts": [], "vectors": {}}
    arg = r"((?:[^(),]|\((?:[^()]|\([^()]*\))*\))+)"
    for a, b in re.findall(r"ASSERT_EQ\(\s*" + arg + r"\s*,\s*" + arg + r"\s*\);", body):
        a, b = a.strip(), b.strip()
        if re.fullmatch(r"-?\d+", a):
            out["asserts"].append({"expected": int(a), "expr": b})
        elif re.fullmatch(r"-?\d+", b):
            out["asserts"].append({"expected": int(b), "expr": a})
    # for (int i = 0; i < N; ++i) { ASSERT_EQ(i + 1, (int)f(v[i])); }
    for cnt, fld in re.findall(r"for \(int i = 0; i < (\d+); \+\+i\) \{\s*"
                               r"ASSERT_EQ\(i \+ 1, \(int\)(\w+)\(\w+\[i\]\)\);", body):
        out["vectors"][fld + "_loop"] = [i + 1 for i in range(int(cnt))]
    for name, vals in re.findall(r"std::vector<int>\s+(\w+)\s*=\s*\{([^}]*)\}", body):
        out["vectors"][name] = [int(t) for t in vals.split(",")]
    return out


def main():
    test = os.path.join(REF, "test")
    if not os.path.isdir(test):
        sys.exit("reference test sources not found at %s" % test)
    golden = {
        "isprings": extract_asserts(os.path.join(test, "program-isprings.cpp"), "isprings"),
        "cg": extract_asserts(os.path.join(test, "program-cg-test.cpp"), "cg"),
        "femTet": extract_asserts(os.path.join(test, "program-fem-test.cpp"), "femTet"),
        "esprings": extract_asserts(os.path.join(test, "program-esprings-test.cpp"),
                                    "esprings"),
        # assembly + SpMV of small element functions (test/input/system/*.sim,
        # test/input/assembly/matrix_vv.sim)
        "gemv_blocked": extract_assert_eq(os.path.join(test, "system-gemv-tests.cpp"),
                                          "gemv_blocked"),
        "gemv_blocked_nw": extract_assert_eq(os.path.join(test, "system-gemv-tests.cpp"),
                                             "gemv_blocked_nw"),
        "gemv_blocked_computed": extract_assert_eq(os.path.join(test, "system-gemv-tests.cpp"),
                                                   "gemv_blocked_computed"),
        "matrix_vv": extract_assert_eq(os.path.join(test, "assembly-tests.cpp"), "matrix_vv"),
    }
    for name in ("matrix_ve", "matrix_ev", "matrix_ve_heterogeneous", "matrix_ev_heterogeneous",
                 "matrix_vv_heterogeneous"):
        golden["incidence_" + name] = extract_incidence_asserts(
            os.path.join(test, "assembly-tests.cpp"), name)
    with open(os.path.join(HERE, "reference_golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    mesh_test = os.path.join(test, "mesh-test.cpp")
    tetgen = {}
    for name in ("TetgenTest", "TetgenEdgeTest"):
        tetgen[name] = {"texts": extract_raw_strings(mesh_test, name),
                        "asserts": extract_assert_eq(mesh_test, name)}
    with open(os.path.join(HERE, "tetgen_golden.json"), "w") as f:
        json.dump(tetgen, f, indent=1)
    for mesh in ("bar2k", "cube"):
        for ext in ("node", "ele"):
            shutil.copy(os.path.join(test, "input", "program", "fem", mesh + "." + ext),
                        os.path.join(HERE, mesh + "." + ext))

    sys.path.insert(0, REPO)
    from oracle import oracle
    oracle.build_ref()
    from simit_gb300 import meshgen
    cases = {}
    ep, n = meshgen.box_springs(4, 3, 2)
    cases["box_springs_4x3x2"] = (n, ep, 2)
    mesh = meshgen.tet_grid(3, 2, 2)
    cases["tet_grid_3x2x2"] = (mesh["n"], mesh["tets"], 4)
    rng = np.random.default_rng(7)
    cases["random_tris_40"] = (40, rng.integers(0, 40, size=3 * 60).astype(np.int32), 3)
    out = {}
    for name, (n, ep, card) in cases.items():
        rp, ci = oracle.ref_pattern(n, ep, card)
        sl = oracle.ref_slots(ep, card, rp, ci)
        out[name] = {"n": int(n), "card": card, "endpoints": np.asarray(ep).tolist(),
                     "rowptr": rp.tolist(), "colidx": ci.tolist(), "slots": sl.tolist()}
    with open(os.path.join(HERE, "pattern_golden.json"), "w") as f:
        json.dump(out, f)

    data = os.path.join(REF, "apps", "data")
    arrays, digests = {}, {}
    bx, bt = meshgen.load_tetgen(os.path.join(data, "tet-bunny", "bunny.1.node"),
                                 os.path.join(data, "tet-bunny", "bunny.1.ele"))
    be = meshgen.load_tetgen_edges(os.path.join(data, "tet-bunny", "bunny.1.edge"))
    dx, dt = meshgen.load_tetgen(os.path.join(data, "tet-dragon", "dragon40k.node"),
                                 os.path.join(data, "tet-dragon", "dragon40k.ele"))
    arrays.update(bunny_x=bx, bunny_tets=bt.astype(np.int32), bunny_edges=be.astype(np.int32),
                  dragon_x=dx, dragon_tets=dt.astype(np.int32))
    for name, x, ep, card in (("bunny_tets", bx, bt, 4), ("bunny_edges", bx, be, 2),
                              ("dragon_tets", dx, dt, 4)):
        n = len(x) // 3
        rp, ci = oracle.ref_pattern(n, ep, card)
        sl = oracle.ref_slots(ep, card, rp, ci)
        digests[name] = {"n": int(n), "card": card, "nE": int(len(ep) // card),
                         "nnzb": int(len(ci)), "rowptr_sha256": sha(rp, np.uint32),
                         "colidx_sha256": sha(ci, np.uint32), "slots_sha256": sha(sl, np.uint32)}
    np.savez_compressed(os.path.join(HERE, "tetmeshes.npz"), **arrays)
    with open(os.path.join(HERE, "tetmeshes_golden.json"), "w") as f:
        json.dump(digests, f, indent=1)
    print("wrote golden fixtures to", HERE)


def lattice():
    """Digests of the reference builder's pattern and slot map on the
    configurations' lattices (a few minutes: the 128^3 pattern has 27.6M
    blocks)."""
    sys.path.insert(0, REPO)
    from oracle import oracle
    oracle.build_ref()
    from simit_gb300 import meshgen, problems
    cases = {"tet_grid_64": meshgen.tet_grid(64)["tets"],
             "tet_grid_128": meshgen.tet_grid(128)["tets"]}
    cases["tet_grid_128_morton"] = problems.reorder_hetero(problems.hetero_mesh(128))["tets"]
    out = {}
    for name, tets in cases.items():
        n = int(tets.max()) + 1
        rp, ci = oracle.ref_pattern(n, tets, 4)
        sl = oracle.ref_slots(tets, 4, rp, ci)
        out[name] = {"n": n, "card": 4, "nE": int(len(tets) // 4), "nnzb": int(len(ci)),
                     "endpoints_sha256": sha(tets, np.int32),
                     "rowptr_sha256": sha(rp, np.uint32), "colidx_sha256": sha(ci, np.uint32),
                     "slots_sha256": sha(sl, np.uint32)}
        print(name, out[name]["nnzb"], flush=True)
    with open(os.path.join(HERE, "lattice_golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if sys.argv[-1] == "lattice":
        lattice()
    else:
        main()
