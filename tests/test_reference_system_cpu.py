"""The reference's system tests through the reference's own programs
(test/input/system/*.sim): each program's map functions generated by the
`.sim` front end and compiled for the host, its `main` restated here step
by step, on the sets the test builds, against the values the test asserts.
Sets, field values and assertions are read from the test files themselves.

* test/system-gemv-tests.cpp: the map's matrix, scalings, sums of
  matrices, the blocked SpMV from the oracle;
* test/system-matrices-tests.cpp and system-misc-tests.cpp (neg): sums,
  differences and transposes of maps over different edge sets, taken on
  dense copies of the assembled matrices, then the product.

The reference checkout is found in SIMIT_REFERENCE, else `reference`
beside the repository; the tests skip without it."""
import os
import re
import tempfile

import numpy as np
import pytest

from simit_gb300 import simfront
from tests.test_simfront_cpu import HostMap

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SIMIT_REFERENCE",
                     os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
TESTS = os.path.join(REF, "test", "system-gemv-tests.cpp")
TEST_FILES = [os.path.join(REF, "test", f) for f in
              ("system-gemv-tests.cpp", "system-matrices-tests.cpp", "system-misc-tests.cpp")]
PROGS = os.path.join(REF, "test", "input", "system")

# each test's main, restated: "Ab" c = A*b; "AplusA" c = (A+A)*b; "A2"
# c = (A*2)*b; "inplace" b = A*b; "input" c = A*b*c0*c1; "hA" c = (10 A)*b;
# "sysreduced" c(p) = (A + B)(p,p)(1,1)
MAINS = {
    "gemv": "Ab", "gemv_diagonal": "Ab", "gemv_nw": "Ab", "gemv_sw": "Ab",
    "gemv_assemble_from_points": "Ab", "gemv_generics": "Ab", "gemv_generics_hidden": "Ab",
    "gemv_pass_element": "Ab", "gemv_diagonal_extraparams": "Ab",
    "gemv_diagonal_storage": "Ab", "gemv_blocked_diagonal_storage": "Ab",
    "gemv_blocked": "Ab", "gemv_blocked_nw": "Ab", "gemv_blocked_computed": "Ab",
    "gemv_add": "AplusA", "gemv_storage": "A2", "gemv_inplace": "inplace",
    "gemv_input": "input", "gemv_blocked_scaled_diagonal": "hA",
    "gemv_diagonal_storage_and_sysreduced": "sysreduced",
}


def _block(name):
    if not os.path.exists(TESTS):
        pytest.skip("reference checkout not found (SIMIT_REFERENCE)")
    for path in TEST_FILES:
        m = re.search(r"TEST\(system, %s\) \{(.*?)\n\}" % name, open(path).read(), re.S)
        if m:
            return "\n".join(ln.split("//")[0] for ln in m.group(1).splitlines())
    raise AssertionError("no test " + name)


def _num(s):
    return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?(?:e-?\d+)?", s)]


def parse_test(name):
    """{set: {"n", "fields": {field: [per element values]}, "comps": {field: c},
    "ends": [[i, j], ...] (edge sets)}}, element refs, tensor arguments and
    the assertions [(expected, set, field, element index, component)]."""
    body = _block(name)
    sets, refs, fvars = {}, {}, {}
    for m in re.finditer(r"Set (\w+)(?:\(([\w, ]*)\))?;", body):
        sets[m.group(1)] = {"n": 0, "fields": {}, "comps": {}, "ends": []}
    for m in re.finditer(r"FieldRef<(?:simit_float|double|float|int)((?:,\s*\d+)*)>\s+(\w+)"
                         r"\s*=\s*(\w+)\.addField<[^>]*>\(\"(\w+)\"\)", body):
        comps = int(np.prod([int(d) for d in re.findall(r"\d+", m.group(1))] or [1]))
        fvars[m.group(2)] = (m.group(3), m.group(4))
        sets[m.group(3)]["comps"][m.group(4)] = comps
    for m in re.finditer(r"(?:ElementRef (\w+) = )?(\w+)\.add\(([\w, ]*)\);", body):
        s = sets[m.group(2)]
        if m.group(1):
            refs[m.group(1)] = (m.group(2), s["n"])
        if m.group(3).strip():
            s["ends"].append([refs[x.strip()][1] for x in m.group(3).split(",")])
        s["n"] += 1
    for sname, s in sets.items():
        for f, c in s["comps"].items():
            s["fields"][f] = np.zeros((s["n"], c))
    for m in re.finditer(r"(\w+)(?:\.set\((\w+),\s*|\((\w+)\)\s*=\s*)(\{[^}]*\}|[-\d.e]+)\)?;",
                         body):
        el = m.group(2) or m.group(3)
        if m.group(1) in fvars and el in refs:
            sname, fname = fvars[m.group(1)]
            sets[sname]["fields"][fname][refs[el][1]] = _num(m.group(4))
    tensors = {}
    for m in re.finditer(r"(\w+)\((\d+)\) = ([-\d.e]+);", body):
        tensors.setdefault(m.group(1), {})[int(m.group(2))] = float(m.group(3))
    asserts = []
    for m in re.finditer(r"ASSERT_EQ\(([-\d.e]+),\s*(?:\([\w ]+\))?\s*(\w+)(?:\.get)?\((\w+)\)"
                         r"(?:\((\d)\))?\)", body):
        if m.group(2) not in fvars or m.group(3) not in refs:
            continue
        sname, fname = fvars[m.group(2)]
        asserts.append((float(m.group(1)), sname, fname, refs[m.group(3)][1],
                        int(m.group(4) or 0)))
    # TensorRef<...> c0 = c.get(p0);  ASSERT_EQ(16.0, c0(0));
    alias = {m.group(1): (m.group(2), m.group(3)) for m in re.finditer(
        r"TensorRef<[^>]*>\s+(\w+)\s*=\s*(\w+)\.get\((\w+)\);", body)}
    for m in re.finditer(r"ASSERT_EQ\(([-\d.e]+),\s*(\w+)\((\d)\)\)", body):
        if m.group(2) in alias:
            fv, el = alias[m.group(2)]
            sname, fname = fvars[fv]
            asserts.append((float(m.group(1)), sname, fname, refs[el][1], int(m.group(3))))
    return sets, tensors, asserts


def _map(src, main_src, which=0):
    """(function, argument values, target set) of the which-th map in main."""
    maps = re.findall(r"map\s+(\w+)(?:\(([^)]*)\))?\s+to\s+(\w+)", main_src)
    fn, args, target = maps[which]
    f = simfront.parse(src)["funcs"][fn]
    vals = [float(x) for x in args.split(",")
            if re.fullmatch(r"\s*-?[\d.]+(e-?\d+)?\s*", x)] if args else []
    scal = [an for an, aty, _ in f["args"] if aty[0] == "scalar"]
    return fn, dict(zip(scal, vals)), target


def _assemble(oracle, tmp, src, fn, args, target, sets):
    """The map's matrix on its pattern: (values, rowptr, colidx, n, bs)."""
    info = simfront.compile_map(src, fn, args)
    assert info["kind"] == "matrix"
    pts_name = [k for k, v in sets.items() if not v["ends"]][0]
    n = sets[pts_name]["n"]
    if target == pts_name:
        ep = np.arange(n, dtype=np.int32)
        fields = {("element", f): v for f, v in sets[target]["fields"].items()}
    else:
        ep = np.array(sets[target]["ends"], np.int32).reshape(-1)
        fields = {("element", f): v for f, v in sets[target]["fields"].items()}
        fields.update({("vertex", f): v for f, v in sets[pts_name]["fields"].items()})
    card = info["card"]
    rp, ci = oracle.pattern(n, ep, card)
    sl = oracle.slots(ep, card, rp, ci)
    vals = HostMap(info, tmp).assemble(ep, sl, len(ci), fields)
    return vals, rp, ci, n, info["bs"]


@pytest.mark.parametrize("name", sorted(MAINS))
def test_reference_gemv(oracle, name):
    src = open(os.path.join(PROGS, name + ".sim")).read() if os.path.exists(PROGS) else None
    sets, tensors, asserts = parse_test(name)
    main_src = src[src.index("export func main"):]
    kind = MAINS[name]
    pts = [k for k, v in sets.items() if not v["ends"]][0]
    with tempfile.TemporaryDirectory() as tmp:
        fn, args, target = _map(src, main_src)
        A, rp, ci, n, bs = _assemble(oracle, tmp, src, fn, args, target, sets)
        b = sets[pts]["fields"].get("b")
        out = {}
        if kind == "sysreduced":
            fn2, args2, target2 = _map(src, main_src, 1)
            B, rp2, ci2, _, _ = _assemble(oracle, tmp, src, fn2, args2, target2, sets)
            C = oracle.add_diag(n, bs, rp2, ci2, B, diag=A)
            c = np.zeros(n)
            for p in range(n):
                k = rp2[p] + list(ci2[rp2[p]:rp2[p + 1]]).index(p)
                c[p] = C[k * bs * bs + 1 * bs + 1]
            out[("c", 0)] = c[:, None]
        else:
            if kind == "AplusA":
                A = A + A
            elif kind == "A2":
                A = A * 2.0
            elif kind == "hA":
                A = 10.0 * A
            y = oracle.spmv(n, bs, rp, ci, A, b.reshape(-1))
            if kind == "input":
                y = y * tensors["cs"][0] * tensors["cs"][1]
            out["b" if kind == "inplace" else "c"] = y.reshape(n, bs)
    assert asserts
    for expected, sname, fname, idx, comp in asserts:
        if fname in out:
            got = out[fname][idx, comp]
        elif (fname, 0) in out:
            got = out[(fname, 0)][idx, 0]
        else:   # an input the program leaves as it was
            got = sets[sname]["fields"][fname][idx, comp]
        assert got == expected, (name, fname, idx, comp, got, expected)


# test/system-matrices-tests.cpp and system-misc-tests.cpp: each main
# restated on dense copies of the assembled matrices
MATRIX_MAINS = {
    "add": "BpC", "add_named_tuples": "BpC", "add_generics": "BpC", "sub": "BmC",
    "add_twice": "twice", "add_transpose": "transpose", "neg": "neg",
    "add_blocked": "blocked+", "add_double_blocked": "blocked+", "sub_blocked": "blocked-",
}


def _dense(A, rp, ci, n, bs):
    D = np.zeros((n * bs, n * bs))
    for r in range(n):
        for k in range(rp[r], rp[r + 1]):
            c = int(ci[k])
            D[r * bs:(r + 1) * bs, c * bs:(c + 1) * bs] += A[k * bs * bs:(k + 1) * bs * bs].reshape(
                bs, bs)
    return D


def _vector_map(tmp, src, fn, args, sets, extra):
    info = simfront.compile_map(src, fn, args)
    assert info["kind"] == "vector"
    pts = [k for k, v in sets.items() if not v["ends"]][0]
    n = sets[pts]["n"]
    fields = {("element", f): v for f, v in sets[pts]["fields"].items()}
    fields.update(extra)
    return HostMap(info, tmp).assemble(np.arange(n, dtype=np.int32), None, n, fields)


@pytest.mark.parametrize("name", sorted(MATRIX_MAINS))
def test_reference_system_matrices(oracle, name):
    sets, _, asserts = parse_test(name)
    src = open(os.path.join(PROGS, name + ".sim")).read()
    main_src = src[src.index("export func main"):]
    kind = MATRIX_MAINS[name]
    pts = [k for k, v in sets.items() if not v["ends"]][0]
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        mats = []
        for which in range(1 if kind == "neg" else 2):
            fn, args, target = _map(src, main_src, which)
            A, rp, ci, n, bs = _assemble(oracle, tmp, src, fn, args, target, sets)
            mats.append(_dense(A, rp, ci, n, bs))
        F = sets[pts]["fields"]
        if kind == "neg":
            out["b"] = -(mats[0] @ F["a"].reshape(-1))
        elif kind.startswith("blocked"):
            A = mats[0] + mats[1] if kind == "blocked+" else mats[0] - mats[1]
            fn, args, _ = _map(src, main_src, 2)
            X = _vector_map(tmp, src, fn, args, sets, {})
            Y = A @ X
            fn, args, _ = _map(src, main_src, 3)
            yname = [an for an, aty, _ in simfront.parse(src)["funcs"][fn]["args"]
                     if aty[0] == "tensor"][0]
            out["a"] = _vector_map(tmp, src, fn, args, sets, {("arg", yname): Y})
        else:
            B, C = mats
            A = {"BpC": B + C, "BmC": B - C, "twice": (B + C) + B + C,
                 "transpose": (B + C) + (B + C).T}[kind]
            out["a"] = A @ F["b"].reshape(-1)
    assert asserts
    for expected, sname, fname, idx, comp in asserts:
        got = out[fname][idx] if fname in out else sets[sname]["fields"][fname][idx, comp]
        assert got == expected, (name, fname, idx, comp, got, expected)
