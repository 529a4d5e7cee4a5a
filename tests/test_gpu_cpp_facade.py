"""The reference's program tests (isprings, cg, femTet) written in C++ against
the facade simit_gb300/cpp/simit.h (Set / FieldRef / Function::bind / init /
runSafe), compiled here and run on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_program_tests(tmp_path):
    from simit_gb300 import _lib
    _lib.load()
    exe = str(tmp_path / "test_programs")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-I", ROOT, "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_programs.cpp"),
           "-L", os.path.join(ROOT, "simit_gb300"), "-lsimit_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(ROOT, "simit_gb300"), "-o", exe]
    subprocess.check_call(cmd)
    r = subprocess.run([exe, os.path.join(ROOT, "tests", "golden")], capture_output=True,
                       text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all passed" in r.stdout


def _build_map_driver(tmp_path):
    from simit_gb300 import _lib
    _lib.load()
    exe = str(tmp_path / "map_driver")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", ROOT, "-I",
                           os.path.join(cuda, "include"),
                           os.path.join(ROOT, "tests", "cpp", "map_driver.cpp"),
                           "-L", os.path.join(ROOT, "simit_gb300"), "-lsimit_gb300",
                           "-L", os.path.join(cuda, "lib64"), "-lcudart",
                           "-Wl,-rpath," + os.path.join(ROOT, "simit_gb300"), "-o", exe])
    return exe


def _run_map(exe, tmp_path, tag, info, n, card, ep, fields, fp64=True):
    """One user map through simit_gb300::Map: info is simfront.compile_map's
    result, fields {(kind, name): array}."""
    import numpy as np
    src = tmp_path / (tag + ".cu")
    src.write_text(info["source"])
    nE = (len(ep) // card) if card else n
    lines = ["%s %d %d %d" % (src, info["bs"], int(info["kind"] == "vector"), int(fp64)),
             "%d %d %d" % (n, card, nE), " ".join(str(int(v)) for v in ep),
             str(len(info["fields"]))]
    for kind, name, shape, dt in info["fields"]:
        a = np.asarray(fields[(kind, name)] if (kind, name) in fields else fields[name])
        comps = int(np.prod(shape)) if shape else 1
        tcode = {"int": "i32", "bool": "b8"}.get(dt, "f64")
        lines.append("%s %s %s %d %s" % (kind, name, tcode,
                                         comps, " ".join(repr(float(x)) for x in a.reshape(-1))))
    inp, outp = tmp_path / (tag + ".in"), tmp_path / (tag + ".out")
    inp.write_text("\n".join(lines) + "\n")
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in outp.read_text().splitlines():
        k, *vals = line.split()
        out[k] = np.array([float(v) for v in vals])
    return out


def test_cpp_map_user_programs(tmp_path, oracle):
    """simit_gb300::Map (simit_gb300/cpp/map.h) runs user maps on facade
    Sets: the cloth program's stretching force over faces (a vector result),
    the nested-block coupling over links (3x3 blocks of 2x2, bs 6) and a map
    over the vertices with component writes, each bit for bit against the
    oracle or the restatement."""
    import numpy as np
    from simit_gb300 import meshgen, simfront
    from tests.test_simfront_cpu import _nested_case, nested_blocks_expected
    exe = _build_map_driver(tmp_path)
    sim = os.path.join(ROOT, "tests", "sim")
    # cloth stretching, faces of a perturbed 17 x 17 sheet
    mg = meshgen.cloth_mesh(17)
    K, rest = oracle.cloth_faces(mg["x"], mg["faces"])
    x = mg["x"] + meshgen.rng(51).normal(0.0, 0.03, mg["x"].size)
    info = simfront.compile_map(open(os.path.join(sim, "cloth_forces.sim")).read(), "stretch")
    got = _run_map(exe, tmp_path, "stretch", info, mg["n"], 3, mg["faces"],
                   {"x": x, "rest": rest, "K": K})
    want = oracle.cloth_stretch(mg["n"], x, mg["faces"], K, rest)
    assert np.array_equal(got["values"], want)
    # nested blocks over links
    n = 20
    links, w, s, rp, ci = _nested_case(oracle, n, 60, 52)
    Kw, _, _ = nested_blocks_expected(n, links, w, s)
    info = simfront.compile_map(open(os.path.join(sim, "nested_blocks.sim")).read(), "couple")
    got = _run_map(exe, tmp_path, "couple", info, n, 2, links.reshape(-1), {"w": w})
    assert np.array_equal(got["rowptr"], rp) and np.array_equal(got["colidx"], ci)
    for r in range(n):
        for k in range(rp[r], rp[r + 1]):
            blk = got["values"][k * 36:(k + 1) * 36].reshape(6, 6)
            assert np.array_equal(blk, Kw.get((r, int(ci[k])), np.zeros((6, 6))))
    # a map over the vertices with component writes
    n = 50
    m = meshgen.rng(53).uniform(1.0, 2.0, n)
    fixed = (meshgen.rng(54).uniform(0, 1, n) < 0.3).astype(np.int32)
    info = simfront.compile_map(open(os.path.join(sim, "point_mass.sim")).read(), "point_mass",
                                {"damp": 0.5}, result="M")
    got = _run_map(exe, tmp_path, "mass", info, n, 0, [], {"m": m, "fixed": fixed})
    want = m[:, None, None] * np.eye(3)[None]
    free = fixed == 0
    want[free, 0, 0] += 0.5 * m[free]
    want[free, 2, 2] += (2.0 * 0.5) * m[free]
    assert np.array_equal(got["values"].reshape(n, 3, 3), want)
