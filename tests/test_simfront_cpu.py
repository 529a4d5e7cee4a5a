"""The `.sim` front end on the CPU: the parser over Simit programs, the
generated element functions compiled by NVRTC for sm_103a, and the same
generated code compiled for the host (g++, contraction off) and assembled
in element order against the oracle's FP64 assembly.

The reference's own programs (apps/fem/*.sim and the test inputs) are read
from the reference checkout when it is present: the directory in
SIMIT_REFERENCE, else `reference` beside the repository; those tests skip
without it.  The programs under tests/sim were written for this repository.
"""
import ctypes
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

from simit_gb300 import meshgen, simfront

HERE = os.path.dirname(os.path.abspath(__file__))
SIM = os.path.join(HERE, "sim")
REF = os.environ.get("SIMIT_REFERENCE",
                     os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def _own(name):
    with open(os.path.join(SIM, name)) as f:
        return f.read()


def _ref(rel):
    p = os.path.join(REF, rel)
    if not os.path.exists(p):
        pytest.skip("reference checkout not found (SIMIT_REFERENCE)")
    with open(p) as f:
        return f.read()


# ---------------------------------------------------------------------------
# parser
# ---------------------------------------------------------------------------
def test_parser_reads_every_reference_program():
    """Every program of the reference's apps and test inputs (outside the
    inputs that are illegal on purpose) parses."""
    if not os.path.isdir(os.path.join(REF, "test", "input")):
        pytest.skip("reference checkout not found (SIMIT_REFERENCE)")
    files = sorted(glob.glob(os.path.join(REF, "apps", "**", "*.sim"), recursive=True) +
                   glob.glob(os.path.join(REF, "test", "input", "**", "*.sim"), recursive=True))
    files = [f for f in files if os.sep + "illegal" + os.sep not in f]
    assert len(files) > 100
    failed = []
    for p in files:
        with open(p) as f:
            try:
                simfront.parse(f.read())
            except simfront.SimError as e:
                failed.append((os.path.relpath(p, REF), str(e)))
    assert not failed, failed


def test_parser_structure():
    prog = simfront.parse(_own("tet_closed_form.sim"))
    assert set(prog["elements"]) == {"Tet", "Vert"}
    assert prog["elements"]["Tet"]["B"] == ("tensor", (3, 3), ("scalar", "float"), True)
    assert prog["externs"]["tets"] == ("set", "Tet", ("verts",) * 4)
    f = prog["funcs"]["tet_stiffness"]
    assert [a[0] for a in f["args"]] == ["h", "rho", "e", "v"]
    assert f["args"][3][1] == ("tuple", ((None, "Vert"),) * 4)
    assert f["results"][0][0] == "K"
    main = prog["funcs"]["main"]["body"][0]
    assert main[0] == "assign" and main[2][0] == "map" and main[2][4] == "+"


@pytest.mark.parametrize("src,msg", [
    ("func f(e : E, v : (V*2)) -> (K : tensor[V,V](float))\n  K(v(0), v(1)) = y;\nend",
     "unknown name"),
    ("func f(a : float, e : E, v : (V*2)) -> (K : tensor[V,V](float))\nend", "not bound"),
    ("func f(e : E, v : (V*2)) -> (b : float)\n  b = 1.0;\nend",
     "no system (vertex-indexed) result"),
    ("func f(e : E, v : (V*2)) -> (K : tensor[V,V](tensor[3,3](float)))\n"
     "  K(v(0), v(1)) = [1.0, 2.0];\nend", "written to a 3x3 block"),
    ("func f(e : E, v : (V*2)) -> (K : tensor[V,V](float))\n"
     "  x = [1.0, 2.0] * [1.0, 2.0];\nend", "product of shapes"),
    ("func f(e : E, v : (V*2)) -> (K : tensor[V,V](float))\n  K(v(0), v(1)) = (1.0;\nend",
     "expected )"),
])
def test_errors_are_reported(src, msg):
    prog = "element E\nend\nelement V\nend\nextern Vs : set{V};\n" + src
    with pytest.raises(simfront.SimError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        simfront.compile_map(prog, "f", {})


# ---------------------------------------------------------------------------
# NVRTC: the generated sources compile for sm_103a
# ---------------------------------------------------------------------------
def _nvrtc_check(src, card, bs, dtype, exact=True, vector=False):
    from simit_gb300 import _lib
    from simit_gb300.runtime import check_element_source
    try:
        check_element_source(src, card, bs, dtype=dtype, exact=exact, vector=vector)
    except _lib.SimitError as e:
        if e.code == _lib.ERR_UNSUPPORTED:
            pytest.skip("NVRTC not available: %s" % e)
        raise


FORCE_ARGS = {"h": 0.01, "rho": 1e3, "gx": 0.0, "gy": -9.81, "gz": 0.0}
OWN_MAPS = [("tet_closed_form.sim", "tet_stiffness", {"h": 0.01, "rho": 1e3}, None),
            ("heat_p1.sim", "heat", {"dt": 0.01}, None),
            ("point_mass.sim", "point_mass", {"damp": 0.5}, "M"),
            ("point_mass.sim", "point_mass", {"damp": 0.5}, "g"),
            ("tet_force.sim", "tet_force", FORCE_ARGS, None)]


@pytest.mark.parametrize("fname,func,args,result", OWN_MAPS)
def test_generated_sources_compile(fname, func, args, result):
    import torch
    r = simfront.compile_map(_own(fname), func, args, result)
    for dt in (torch.float32, torch.float64):
        _nvrtc_check(r["source"], r["card"], r["bs"], dt, vector=r["kind"] == "vector")


REF_MAPS = [("apps/fem/fem_linear.sim", "compute_stiffness", {"h": 0.01}, None),
            ("apps/fem/fem_linear.sim", "compute_force", {"h": 0.01}, None),
            ("apps/fem/fem_neohookean.sim", "compute_force", {"h": 0.01}, None),
            ("apps/cloth/cloth.sim", "stretchingForce", {}, None),
            ("apps/cloth/cloth.sim", "bendingForce", {}, None),
            ("test/input/program/isprings.sim", "compute_elasticity", {}, "K"),
            ("test/input/program/isprings.sim", "compute_elasticity", {}, "fe"),
            ("test/input/program/isprings.sim", "compute_mass_damping", {}, "MD"),
            ("test/input/program/isprings.sim", "compute_mass_damping", {}, "fmg"),
            ("apps/fem/poisson_2D_triangles.sim", "assemble", {}, "b"),
            ("apps/fem/fem_neohookean.sim", "compute_stiffness", {"h": 0.01}, None),
            ("apps/fem/fem_linear.sim", "compute_mass", {}, None),
            ("apps/fem/poisson_2D_triangles.sim", "assemble", {}, "A"),
            ("apps/fem/poisson_3D_tetrahedrons.sim", "assemble", {}, "A"),
            ("apps/cloth/cloth.sim", "invMassMatrix", {}, None),
            ("test/input/assembly/matrix_vv.sim", "f", {}, None),
            ("test/input/assembly/edges_two_results.sim", "f", {}, "A"),
            ("test/input/assembly/vertices_two_results.sim", "f", {}, "A")]


@pytest.mark.parametrize("rel,func,args,result", REF_MAPS)
def test_reference_maps_compile(rel, func, args, result):
    import torch
    r = simfront.compile_map(_ref(rel), func, args, result)
    _nvrtc_check(r["source"], r["card"], r["bs"], torch.float64,
                 vector=r["kind"] == "vector")


# ---------------------------------------------------------------------------
# host-compiled generated code against the oracle
# ---------------------------------------------------------------------------
HARNESS = r"""
#include <math.h>
#define __device__
typedef double real;
#define BS %(bs)d
#define CARD %(card)d
typedef real sg_block[BS][BS];
#define SG_TERMS 2
%(source)s
// elements in order, blocks (i, j) in order, terms in order: each term a
// separate += on its slot, as the lowered map adds them
extern "C" void sim_assemble(long long nE, const int *ep_all, const real *const *f,
                             const long long *slots, real *vals) {
  for (long long e = 0; e < nE; ++e)
    for (int i = 0; i < CARD; ++i)
      for (int j = 0; j < CARD; ++j) {
        sg_block blk[SG_TERMS];
        const int nt = element_block(e, i, j, ep_all + e * CARD, f, blk);
        real *v = vals + slots[(e * CARD + i) * CARD + j] * BS * BS;
        for (int q = 0; q < nt; ++q)
          for (int a = 0; a < BS; ++a)
            for (int b = 0; b < BS; ++b) v[a * BS + b] += blk[q][a][b];
      }
}
"""


HARNESS_VEC = r"""
#include <math.h>
#define __device__
typedef double real;
#define BS %(bs)d
#define CARD %(card)d
typedef real sg_vec[BS];
#define SG_VTERMS 8
%(source)s
// elements in order, endpoints in order, terms in order: each term a
// separate += on its vertex, as the lowered map adds them
extern "C" void sim_assemble(long long nE, const int *ep_all, const real *const *f,
                             const long long *unused, real *vals) {
  (void)unused;
  for (long long e = 0; e < nE; ++e)
    for (int i = 0; i < CARD; ++i) {
      sg_vec vec[SG_VTERMS];
      const int nt = element_vector(e, i, ep_all + e * CARD, f, vec);
      real *v = vals + (long long)ep_all[e * CARD + i] * BS;
      for (int q = 0; q < nt; ++q)
        for (int a = 0; a < BS; ++a) v[a] += vec[q][a];
    }
}
"""


class HostMap:
    """The generated element function compiled for the host."""

    _count = 0

    def __init__(self, info, tmp):
        # a fresh file name per library: dlopen hands back an already loaded
        # library for a path it has seen
        HostMap._count += 1
        src = os.path.join(tmp, "gen%d.cpp" % HostMap._count)
        so = os.path.join(tmp, "gen%d.so" % HostMap._count)
        text = HARNESS_VEC if info.get("kind") == "vector" else HARNESS
        with open(src, "w") as f:
            f.write(text % {"bs": info["bs"], "card": info["card"], "source": info["source"]})
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", so, src],
                       check=True, capture_output=True)
        self.lib = ctypes.CDLL(so)
        self.info = info

    def assemble(self, ep, slots, nnzb, fields):
        """Matrix maps: values [nnzb*bs*bs] through the slot map; vector
        maps: values [nnzb*bs] for nnzb vertices (slots unused)."""
        keep = []
        for kind, name, shape, dt in self.info["fields"]:
            a = fields[(kind, name)] if (kind, name) in fields else fields[name]
            a = np.ascontiguousarray(a, {"int": np.int32, "bool": np.bool_}.get(dt, np.float64))
            keep.append(a)
        arr = (ctypes.c_void_p * max(1, len(keep)))(*[a.ctypes.data for a in keep])
        bs = self.info["bs"]
        vals = np.zeros(nnzb * bs * (1 if self.info.get("kind") == "vector" else bs))
        ep = np.ascontiguousarray(ep, np.int32)
        sl = np.ascontiguousarray(slots if slots is not None else np.zeros(1), np.int64)
        self.lib.sim_assemble(ctypes.c_longlong(ep.size // self.info["card"]),
                              ep.ctypes.data_as(ctypes.c_void_p), arr,
                              sl.ctypes.data_as(ctypes.c_void_p),
                              vals.ctypes.data_as(ctypes.c_void_p))
        return vals


def _tet_case(oracle, seed=3):
    mg = meshgen.tet_grid(4, 3, 3, disp=2e-2, seed=seed)
    tets, n = mg["tets"], mg["n"]
    nT = len(tets) // 4
    g = meshgen.rng(seed + 10)
    B, W, _ = oracle.tet_precompute(mg["X0"], tets, 1e3)
    mu = 10 ** g.uniform(3, 5, nT)
    lam = 10 ** g.uniform(3, 5, nT)
    c = (g.uniform(0, 1, n) < 0.15).astype(np.int32)
    rowptr, colidx = oracle.pattern(n, tets, 4)
    slots = oracle.slots(tets, 4, rowptr, colidx)
    return dict(mg=mg, tets=tets, n=n, B=B, W=W, u=mu, l=lam, c=c, rowptr=rowptr,
                colidx=colidx, slots=slots)


@pytest.mark.parametrize("neo", [0, 1])
def test_reference_fem_stiffness_matches_oracle(oracle, neo):
    """The reference's compute_stiffness (apps/fem/fem_linear.sim and
    fem_neohookean.sim), generated and compiled for the host, assembles the
    oracle's matrix bit for bit (linear) / to rounding (neo-Hookean, whose
    log is the host's)."""
    rel = "apps/fem/fem_neohookean.sim" if neo else "apps/fem/fem_linear.sim"
    info = simfront.compile_map(_ref(rel), "compute_stiffness", {"h": 0.01})
    k = _tet_case(oracle)
    with tempfile.TemporaryDirectory() as tmp:
        hm = HostMap(info, tmp)
        got = hm.assemble(k["tets"], k["slots"], len(k["colidx"]),
                          {"B": k["B"], "W": k["W"], "u": k["u"], "l": k["l"], "c": k["c"],
                           "x": k["mg"]["x"]})
    want = oracle.tet_stiffness(neo, k["mg"]["x"], k["c"], k["tets"], k["B"], k["W"], k["u"],
                                k["l"], 0.01, 1e3, k["rowptr"], k["colidx"])
    if neo:
        scale = np.abs(want).max()
        assert np.abs(got - want).max() <= 1e-12 * scale
    else:
        assert np.array_equal(got, want)


def test_own_closed_form_tet_matches_oracle(oracle):
    """tests/sim/tet_closed_form.sim: the closed form of the linear element
    agrees with the oracle's B' E B product to rounding."""
    info = simfront.compile_map(_own("tet_closed_form.sim"), "tet_stiffness",
                                {"h": 0.01, "rho": 1e3})
    k = _tet_case(oracle, seed=5)
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(k["tets"], k["slots"], len(k["colidx"]), k)
    want = oracle.tet_stiffness(0, k["mg"]["x"], k["c"], k["tets"], k["B"], k["W"], k["u"],
                                k["l"], 0.01, 1e3, k["rowptr"], k["colidx"])
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_own_heat_matches_oracle(oracle):
    """tests/sim/heat_p1.sim assembles the oracle's P1 heat matrix bit for
    bit."""
    info = simfront.compile_map(_own("heat_p1.sim"), "heat", {"dt": 0.01})
    k = _tet_case(oracle, seed=7)
    kappa = 10 ** meshgen.rng(8).uniform(-1, 1, len(k["W"]))
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(k["tets"], k["slots"], len(k["colidx"]),
                                          {"B": k["B"], "W": k["W"], "kappa": kappa})
    want, _ = oracle.heat_assemble(k["n"], k["tets"], k["B"], k["W"], kappa, 0.01,
                                   np.zeros(k["n"]), k["rowptr"], k["colidx"])
    assert np.array_equal(got, want)


def test_point_mass_vertex_map_and_component_writes():
    """A map over the vertices (one endpoint per element): the full block,
    then component writes on free vertices; the vector result is left out."""
    info = simfront.compile_map(_own("point_mass.sim"), "point_mass", {"damp": 0.5}, "M")
    assert info["card"] == 1 and info["bs"] == 3
    n = 7
    m = np.linspace(1.0, 2.0, n)
    fixed = np.array([0, 1, 0, 0, 1, 0, 0], bool)
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(np.arange(n), np.arange(n), n,
                                          {"m": m, "fixed": fixed}).reshape(n, 3, 3)
    want = np.zeros((n, 3, 3))
    for p in range(n):
        want[p] = m[p] * np.eye(3)
        if not fixed[p]:
            want[p, 0, 0] += 0.5 * m[p]
            want[p, 2, 2] += (2.0 * 0.5) * m[p]
    assert np.array_equal(got, want)


def test_reference_poisson_triangles_matches_restatement():
    """The reference's 2D Poisson assembly (apps/fem/poisson_2D_triangles.sim,
    matrix A) against a numpy restatement of the same formulas."""
    info = simfront.compile_map(_ref("apps/fem/poisson_2D_triangles.sim"), "assemble", {}, "A")
    g = meshgen.rng(4)
    side = 6
    xs, ys = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    pts = np.stack([xs.ravel(), ys.ravel()], 1) + g.uniform(-0.2, 0.2, (side * side, 2))
    tri = []
    for i in range(side - 1):
        for j in range(side - 1):
            a, b, c, d = i * side + j, (i + 1) * side + j, i * side + j + 1, (i + 1) * side + j + 1
            tri += [(a, b, d), (a, d, c)]
    tri = np.array(tri, np.int32)
    n = side * side
    edge = np.zeros(n, bool)
    edge[[p for p in range(n) if p // side in (0, side - 1) or p % side in (0, side - 1)]] = True
    # dense pattern: one slot per (row, col) pair that any triangle touches
    pairs = sorted({(int(r), int(c)) for t in tri for r in t for c in t})
    index = {pc: k for k, pc in enumerate(pairs)}
    slots = np.array([index[(int(t[i]), int(t[j]))] for t in tri for i in range(3)
                      for j in range(3)], np.int64)
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(tri.ravel(), slots, len(pairs),
                                          {"x": pts, "edge": edge})
    want = np.zeros(len(pairs))
    for t in tri:
        X = np.ones((3, 3))
        X[:, :2] = pts[t]
        area = np.linalg.det(X)
        abc = np.linalg.inv(X)
        for i in range(3):
            for j in range(3):
                if not (edge[t[i]] or edge[t[j]]):
                    want[index[(int(t[i]), int(t[j]))]] += \
                        (abc[0, i] * abc[0, j] + abc[1, i] * abc[1, j]) * area
            if edge[t[i]]:
                want[index[(int(t[i]), int(t[i]))]] += 1.0
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("neo", [0, 1])
def test_reference_fem_force_matches_oracle(oracle, neo):
    """The reference's compute_force (a vector map: the element's nodal
    forces, gravity and momentum on free vertices), generated as an
    element_vector function and compiled for the host, equals the oracle's
    force bit for bit (linear) / to rounding (neo-Hookean)."""
    rel = "apps/fem/fem_neohookean.sim" if neo else "apps/fem/fem_linear.sim"
    info = simfront.compile_map(_ref(rel), "compute_force", {"h": 0.01})
    assert info["kind"] == "vector" and info["bs"] == 3
    k = _tet_case(oracle, seed=9)
    v = meshgen.rng(12).uniform(-0.01, 0.01, k["n"] * 3)
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(k["tets"], None, k["n"],
                                          {"B": k["B"], "W": k["W"], "u": k["u"], "l": k["l"],
                                           "c": k["c"], "x": k["mg"]["x"], "v": v})
    # the reference program's gravity is (0, -10, 0) and rho 1e3
    want = oracle.tet_force(neo, k["mg"]["x"], v, k["c"], k["tets"], k["B"], k["W"], k["u"],
                            k["l"], 0.01, 1e3, np.array([0.0, -10.0, 0.0]))
    if neo:
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    else:
        assert np.array_equal(got, want)


def test_own_tet_force_matches_oracle(oracle):
    """tests/sim/tet_force.sim assembles the oracle's linear force bit for
    bit."""
    info = simfront.compile_map(_own("tet_force.sim"), "tet_force", FORCE_ARGS)
    k = _tet_case(oracle, seed=13)
    v = meshgen.rng(14).uniform(-0.01, 0.01, k["n"] * 3)
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(k["tets"], None, k["n"],
                                          {"B": k["B"], "W": k["W"], "u": k["u"], "l": k["l"],
                                           "c": k["c"], "x": k["mg"]["x"], "v": v})
    want = oracle.tet_force(0, k["mg"]["x"], v, k["c"], k["tets"], k["B"], k["W"], k["u"],
                            k["l"], 0.01, 1e3, np.array([0.0, -9.81, 0.0]))
    assert np.array_equal(got, want)


# ---------------------------------------------------------------------------
# cloth: triangle stretching over faces (card 3), dihedral bending over
# hinges (card 4)
# ---------------------------------------------------------------------------
def _cloth_case(oracle, side=9, seed=21, noise=0.03):
    """A sheet, its rest quantities from the oracle's restatement of the
    cloth initialisation, and perturbed current positions."""
    mg = meshgen.cloth_mesh(side)
    K, rest = oracle.cloth_faces(mg["x"], mg["faces"])
    ang, ln, perp = oracle.cloth_hinges(mg["x"], mg["hinges"])
    x = mg["x"] + meshgen.rng(seed).normal(0.0, noise, mg["x"].size)
    return dict(mg=mg, n=mg["n"], K=K, rest=rest, ang=ang, ln=ln, perp=perp, x=x)


def test_cloth_oracle_rest_state_and_invariance(oracle):
    """The restated forces vanish at the rest positions, and at perturbed
    positions each sums to zero over the sheet (translation invariance)."""
    k = _cloth_case(oracle)
    X = k["mg"]["x"]
    fs0 = oracle.cloth_stretch(k["n"], X, k["mg"]["faces"], k["K"], k["rest"])
    fb0 = oracle.cloth_bend(k["n"], X, k["mg"]["hinges"], k["ang"], k["ln"], k["perp"])
    assert np.abs(fs0).max() < 1e-12 and np.abs(fb0).max() < 1e-12
    fs = oracle.cloth_stretch(k["n"], k["x"], k["mg"]["faces"], k["K"], k["rest"])
    fb = oracle.cloth_bend(k["n"], k["x"], k["mg"]["hinges"], k["ang"], k["ln"], k["perp"])
    for f in (fs, fb):
        assert np.abs(f).max() > 1e-3
        assert np.abs(f.reshape(-1, 3).sum(0)).max() < 1e-11 * np.abs(f).max() * k["n"]


def _cloth_host(info, k, which):
    mg = k["mg"]
    with tempfile.TemporaryDirectory() as tmp:
        hm = HostMap(info, tmp)
        if which == "stretch":
            fields = {"x": k["x"], "restLengths": k["rest"], "rest": k["rest"],
                      "precomputedStretchingMatrix": k["K"], "K": k["K"]}
            return hm.assemble(mg["faces"], None, k["n"], fields)
        fields = {"x": k["x"], "restLength": k["ln"], "len": k["ln"],
                  "restPerpLength": k["perp"], "perp": k["perp"],
                  "restBendingAngle": k["ang"], "theta0": k["ang"]}
        return hm.assemble(mg["hinges"], None, k["n"], fields)


@pytest.mark.parametrize("func,which", [("stretchingForce", "stretch"),
                                        ("bendingForce", "bend")])
def test_reference_cloth_forces_match_oracle(oracle, func, which):
    """The reference's own cloth forces (apps/cloth/cloth.sim:142-173),
    generated as element_vector functions and compiled for the host, equal
    the oracle's restatement bit for bit on a perturbed sheet."""
    info = simfront.compile_map(_ref("apps/cloth/cloth.sim"), func)
    assert info["kind"] == "vector" and info["card"] == (3 if which == "stretch" else 4)
    k = _cloth_case(oracle)
    got = _cloth_host(info, k, which)
    mg = k["mg"]
    if which == "stretch":
        want = oracle.cloth_stretch(k["n"], k["x"], mg["faces"], k["K"], k["rest"])
    else:
        want = oracle.cloth_bend(k["n"], k["x"], mg["hinges"], k["ang"], k["ln"], k["perp"])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("func,which", [("stretch", "stretch"), ("bend", "bend")])
def test_own_cloth_forces_match_oracle(oracle, func, which):
    """tests/sim/cloth_forces.sim's stretch and bend: the oracle's cloth
    forces bit for bit, on the host."""
    info = simfront.compile_map(_own("cloth_forces.sim"), func)
    k = _cloth_case(oracle, side=11, seed=22)
    got = _cloth_host(info, k, which)
    mg = k["mg"]
    if which == "stretch":
        want = oracle.cloth_stretch(k["n"], k["x"], mg["faces"], k["K"], k["rest"])
    else:
        want = oracle.cloth_bend(k["n"], k["x"], mg["hinges"], k["ang"], k["ln"], k["perp"])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("func", ["stretch", "bend", "gravity", "inv_mass"])
def test_own_cloth_maps_compile(func):
    import torch
    r = simfront.compile_map(_own("cloth_forces.sim"), func)
    for dt in (torch.float32, torch.float64):
        _nvrtc_check(r["source"], r["card"], r["bs"], dt, vector=r["kind"] == "vector")


def test_reference_cloth_gravity_accumulates_on_fixed_points():
    """cloth.sim's gravityForce writes (0, -9.8, 0) and then, on a fixed
    point, (0, 0, 0): the writes of a map's result accumulate, so fixed
    points keep gravity -- the oracle's cloth step restates it so."""
    info = simfront.compile_map(_ref("apps/cloth/cloth.sim"), "gravityForce")
    n = 6
    fixed = np.array([0, 1, 0, 1, 1, 0], np.int32)
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(np.arange(n, dtype=np.int32), None, n,
                                          {"fixed": fixed})
    want = np.tile([0.0, -9.8, 0.0], n)
    assert np.array_equal(got, want)


# ---------------------------------------------------------------------------
# nested block types and component writes into blocks
# ---------------------------------------------------------------------------
def _diag(n):
    """Pattern and slots of a map over the vertices (one diagonal block each)."""
    return np.arange(n + 1, dtype=np.uint32), np.arange(n, dtype=np.uint32), np.arange(n)


def test_reference_block_component_write():
    """test/assembly-tests.cpp:450-471 (block_component_write): each edge
    writes component 0 of its first endpoint's 2-vector; on the 3-vertex
    path the result is (1, 0), (1, 0), (0, 0)."""
    info = simfront.compile_map(_ref("test/input/assembly/block_component_write.sim"), "f")
    assert info["kind"] == "vector" and info["bs"] == 2
    with tempfile.TemporaryDirectory() as tmp:
        got = HostMap(info, tmp).assemble(np.array([0, 1, 1, 2], np.int32), None, 3, {})
    assert got.tolist() == [1, 0, 1, 0, 0, 0]


def test_reference_blocked_nested_blocks(oracle):
    """test/assembly-tests.cpp:429-448 (blocked): a diagonal system matrix
    of 3x3 blocks of 3x3 blocks, a vector of 3 blocks of 3, their product
    and a map reading it as an argument give z = 81, 324, 729 for
    x = 1, 2, 3."""
    src = _ref("test/input/assembly/blocked.sim")
    n = 3
    xs = np.array([1, 2, 3], np.int32)
    ep = np.arange(n, dtype=np.int32)
    rp, ci, sl = _diag(n)
    with tempfile.TemporaryDirectory() as tmp:
        bi = simfront.compile_map(src, "build_blocked")
        assert bi["bs"] == 9
        X = HostMap(bi, tmp + "/").assemble(ep, sl, n, {"x": xs})
    with tempfile.TemporaryDirectory() as tmp:
        vx = HostMap(simfront.compile_map(src, "promote"), tmp).assemble(ep, None, n, {"x": xs})
    y = oracle.spmv(n, 9, rp, ci, X, vx)
    with tempfile.TemporaryDirectory() as tmp:
        si = simfront.compile_map(src, "sum_vectors")
        assert si["fields"] == [("arg", "y", (3, 3), "int")]
        z = HostMap(si, tmp).assemble(ep, None, n, {"y": y})
    assert z.tolist() == [81, 324, 729]


def nested_blocks_expected(n, links, w, s):
    """tests/sim/nested_blocks.sim restated with numpy, in the maps' order of
    operations: K (per pattern slot, 6x6 row-major, slots in element order),
    v (6 per node), m (2 per node)."""
    K = {}

    def add(r, c, blk):
        K[(r, c)] = K.get((r, c), np.zeros((6, 6))) + blk

    m = np.zeros((n, 2))
    for e, (p0, p1) in enumerate(links):
        B = np.zeros((6, 6))
        for a in range(3):
            for b in range(3):
                for c in range(2):
                    for d in range(2):
                        B[a * 2 + c, b * 2 + d] = (w[e] * ((1.0 + a) + 2.0 * b) + 0.5 * c) - 0.25 * d
        add(p0, p0, B)
        add(p1, p1, B)
        C = np.zeros((6, 6))
        C[1 * 2 + 0, 2 * 2 + 1] = -w[e]
        add(p0, p1, C)
        D = np.zeros((6, 6))
        D[2 * 2 + 0, 0] = w[e]
        D[2 * 2 + 1, 1] = 2.0 * w[e]
        add(p1, p0, D)
        m[p0, 0] += 1.0
        m[p1, 1] += w[e]
    v = np.zeros((n, 6))
    v[:, 0::2] = s[:, None]
    v[:, 1::2] = -s[:, None]
    v[:, 3] = -s + 2.0 * s
    return K, v.reshape(-1), m.reshape(-1)


def _nested_case(oracle, n=12, nl=30, seed=41):
    g = meshgen.rng(seed)
    a = g.integers(0, n, nl)
    b = (a + g.integers(1, n, nl)) % n
    links = np.stack([a, b], 1).astype(np.int32)
    w = g.uniform(0.5, 2.0, nl)
    s = g.uniform(-1.0, 1.0, n)
    rp, ci = oracle.pattern(n, links.reshape(-1), 2)
    return links, w, s, rp, ci


def test_own_nested_blocks_match_restatement(oracle):
    """tests/sim/nested_blocks.sim on the host: the nested matrix and vector
    results bit for bit against the numpy restatement, and the map over a
    system-vector argument against K v reduced by hand."""
    src = _own("nested_blocks.sim")
    n = 12
    links, w, s, rp, ci = _nested_case(oracle, n)
    slots = oracle.slots(links.reshape(-1), 2, rp, ci)
    Kw, vw, mw = nested_blocks_expected(n, links, w, s)
    with tempfile.TemporaryDirectory() as tmp:
        K = HostMap(simfront.compile_map(src, "couple"), tmp).assemble(
            links.reshape(-1), slots, len(ci), {"w": w})
    for r in range(n):
        for k in range(rp[r], rp[r + 1]):
            want = Kw.get((r, int(ci[k])), np.zeros((6, 6)))
            assert np.array_equal(K[k * 36:(k + 1) * 36].reshape(6, 6), want), (r, ci[k])
    ep = np.arange(n, dtype=np.int32)
    with tempfile.TemporaryDirectory() as tmp:
        v = HostMap(simfront.compile_map(src, "spread"), tmp).assemble(ep, None, n, {"s": s})
    assert np.array_equal(v, vw)
    with tempfile.TemporaryDirectory() as tmp:
        m = HostMap(simfront.compile_map(src, "mark"), tmp).assemble(
            links.reshape(-1), None, n, {"w": w})
    assert np.array_equal(m, mw)
    y = oracle.spmv(n, 6, rp, ci, K, v)
    with tempfile.TemporaryDirectory() as tmp:
        z = HostMap(simfront.compile_map(src, "weigh"), tmp).assemble(ep, None, n, {"y": y})
    Y = y.reshape(n, 3, 2)
    want = np.zeros(n)
    for a in range(3):
        want = (want + (a + 1.0) * Y[:, a, 0]) - Y[:, a, 1]
    assert np.array_equal(z, want)


def test_own_nine_by_nine_nested_diagonal(oracle):
    """tests/sim/nested_blocks.sim's fill9 / lift9 / total9: the blocked
    assembly test's values (81, 324, 729 for k = 1, 2, 3) through this
    repository's program, on the host."""
    src = _own("nested_blocks.sim")
    n = 3
    k = np.array([1, 2, 3], np.int32)
    ep = np.arange(n, dtype=np.int32)
    rp, ci, sl = _diag(n)
    with tempfile.TemporaryDirectory() as tmp:
        X = HostMap(simfront.compile_map(src, "fill9"), tmp).assemble(ep, sl, n, {"k": k})
    with tempfile.TemporaryDirectory() as tmp:
        x = HostMap(simfront.compile_map(src, "lift9"), tmp).assemble(ep, None, n, {"k": k})
    y = oracle.spmv(n, 9, rp, ci, X, x)
    with tempfile.TemporaryDirectory() as tmp:
        z = HostMap(simfront.compile_map(src, "total9"), tmp).assemble(ep, None, n, {"y": y})
    assert z.tolist() == [81, 324, 729]


@pytest.mark.parametrize("func", ["couple", "spread", "weigh", "mark", "fill9", "lift9",
                                  "total9"])
def test_own_nested_block_maps_compile(func):
    import torch
    r = simfront.compile_map(_own("nested_blocks.sim"), func)
    for dt in (torch.float32, torch.float64):
        _nvrtc_check(r["source"], r["card"], r["bs"], dt, vector=r["kind"] == "vector")


# ---------------------------------------------------------------------------
# the reference's vector assembly tests (test/assembly-tests.cpp:12-217):
# maps over the vertices, over the edges themselves, over edge sets of one,
# two and three endpoints, and maps with two results whose product is taken
# ---------------------------------------------------------------------------
# (test, n vertices, endpoints (None: a map over the vertices, "self": over
#  the edges), card, field values, expected)
VECTOR_ASSEMBLY_CASES = [
    ("vertices", 3, None, 1, [1, 2, 3], [2, 4, 6]),
    ("vertices_two_results", 3, None, 1, [1, 2, 3], [6, 24, 54]),
    ("edges_no_endpoints", 2, "self", 1, [1, 2], [2, 4]),
    ("edges_unary", 3, [0, 2], 1, None, [1, 0, 1]),
    ("edges_binary", 3, [0, 1, 1, 2], 2, None, [1, 2, 1]),
    ("edges_tertiary", 4, [0, 1, 2, 1, 2, 3], 3, [10, 1], [10, 11, 11, 1]),
    ("edges_two_results", 3, [0, 1, 1, 2], 2, [1, 2], [43, 177, 168]),
]

# the reference program's function and field of each test
_REF_FORMS = {"vertices": ("asm", "a"), "vertices_two_results": ("f", "a"),
              "edges_no_endpoints": ("f", "a"), "edges_unary": ("asm", None),
              "edges_binary": ("asm", None), "edges_tertiary": ("dist", "a"),
              "edges_two_results": ("f", "a")}
# this repository's tests/sim/assembly_forms.sim
OWN_FORMS = {"vertices": ("twice", "a"), "vertices_two_results": ("scaled", "a"),
             "edges_no_endpoints": ("own", "w"), "edges_unary": ("touch1", None),
             "edges_binary": ("touch2", None), "edges_tertiary": ("spread3", "w"),
             "edges_two_results": ("both", "w")}


def run_vector_case(case, src, forms, vector_map, matrix_map, spmv):
    """One case through caller-given runners: vector_map(info, n, ep, fields)
    and matrix_map(info, n, ep, fields) -> (values, rowptr, colidx);
    spmv(n, rowptr, colidx, values, x).  Returns the case's result."""
    name, n, ep, card, vals, _ = case
    func, field = forms[name]
    fields = {} if field is None else {field: np.array(vals, np.float64)}
    if ep is None or ep == "self":
        ep = np.arange(n, dtype=np.int32)
    ep = np.asarray(ep, np.int32)
    if name.endswith("two_results"):
        names = [r for r, _ in simfront.parse(src)["funcs"][func]["results"]]
        vres = simfront.compile_map(src, func, result=names[0])
        mres = simfront.compile_map(src, func, result=names[1])
        assert vres["kind"] == "vector" and mres["kind"] == "matrix"
        b = vector_map(vres, n, ep, fields)
        A, rp, ci = matrix_map(mres, n, ep, fields)
        return spmv(n, rp, ci, A, b)
    info = simfront.compile_map(src, func)
    assert info["kind"] == "vector" and info["card"] == card
    return vector_map(info, n, ep, fields)


def _host_runners(oracle, tmp):
    def vmap(info, n, ep, fields):
        return HostMap(info, tmp).assemble(ep, None, n, fields)

    def mmap(info, n, ep, fields):
        rp, ci = oracle.pattern(n, ep, info["card"])
        sl = oracle.slots(ep, info["card"], rp, ci)
        return HostMap(info, tmp).assemble(ep, sl, len(ci), fields), rp, ci

    def spmv(n, rp, ci, A, x):
        return oracle.spmv(n, 1, rp, ci, A, x)
    return vmap, mmap, spmv


@pytest.mark.parametrize("case", VECTOR_ASSEMBLY_CASES, ids=[c[0] for c in VECTOR_ASSEMBLY_CASES])
def test_reference_vector_assembly(oracle, case):
    """The reference's own program of each test, its maps generated and
    compiled for the host, its main's product taken by the oracle's SpMV:
    the test's asserted values."""
    src = _ref("test/input/assembly/%s.sim" % case[0])
    with tempfile.TemporaryDirectory() as tmp:
        got = run_vector_case(case, src, _REF_FORMS, *_host_runners(oracle, tmp))
    assert got.tolist() == case[5]


@pytest.mark.parametrize("case", VECTOR_ASSEMBLY_CASES, ids=[c[0] for c in VECTOR_ASSEMBLY_CASES])
def test_own_assembly_forms(oracle, case):
    """tests/sim/assembly_forms.sim on the same inputs, on the host: the same
    values."""
    with tempfile.TemporaryDirectory() as tmp:
        got = run_vector_case(case, _own("assembly_forms.sim"), OWN_FORMS,
                              *_host_runners(oracle, tmp))
    assert got.tolist() == case[5]


def test_reference_isprings_maps_match_oracle(oracle):
    """test/input/program/isprings.sim's two maps generated and compiled for
    the host -- compute_mass_damping over the points (a fixed point's
    `MD(p,p) = 1.0`, a scalar written to a 3x3 block, lands on entry (0,0)
    alone, as in the lowered program) and compute_elasticity over the
    springs -- then MDK = MD + K in the lowered order: the oracle's MDK and
    f bit for bit."""
    src = _ref("test/input/program/isprings.sim")
    L = meshgen.springs_lattice(4, 4, 4, 0.1, 0.01, seed=3)
    n, ep = L["n"], L["ep"]
    g = meshgen.rng(61)
    fixed = g.uniform(0, 1, n) < 0.2
    v = g.uniform(-0.1, 0.1, n * 3)
    m = g.uniform(0.5, 1.5, n)
    k = g.uniform(50.0, 150.0, len(L["l0"]))
    rp, ci = oracle.pattern(n, ep, 2)
    sl = oracle.slots(ep, 2, rp, ci)
    prp, pci, psl = _diag(n)
    pts = np.arange(n, dtype=np.int32)
    vf = {"x": L["x"], "v": v, "m": m, "fixed": fixed, "k": k, "l0": L["l0"]}
    with tempfile.TemporaryDirectory() as tmp:
        MD = HostMap(simfront.compile_map(src, "compute_mass_damping", result="MD"),
                     tmp).assemble(pts, psl, n, vf)
        fmg = HostMap(simfront.compile_map(src, "compute_mass_damping", result="fmg"),
                      tmp).assemble(pts, None, n, vf)
        K = HostMap(simfront.compile_map(src, "compute_elasticity", result="K"),
                    tmp).assemble(ep, sl, len(ci), vf)
        fe = HostMap(simfront.compile_map(src, "compute_elasticity", result="fe"),
                     tmp).assemble(ep, None, n, vf)
    blocks = MD.reshape(n, 3, 3)
    assert np.array_equal(blocks[fixed], np.tile([[1.0, 0, 0], [0, 0, 0], [0, 0, 0]],
                                                 (int(fixed.sum()), 1, 1)))
    MDK = oracle.add_diag(n, 3, rp, ci, K, diag=MD)
    wA, wf = oracle.springs_assemble(1, L["x"], v, m, fixed.astype(np.uint8), ep, k, L["l0"],
                                     1e-2, 1e-1, np.array([0.0, 0.0, -9.81]), rp, ci)
    assert np.array_equal(MDK, wA)
    assert np.array_equal(fmg + fe, wf)


# ---------------------------------------------------------------------------
# explicit springs: test/program-esprings-test.cpp
# ---------------------------------------------------------------------------
def _esprings_host(src, names, tmp):
    """Ten steps of the esprings main with the program's three maps (names:
    gravity, masses, stiffness functions) compiled for the host."""
    from tests import scenarios
    s = scenarios.esprings_cube()
    maps = [HostMap(simfront.compile_map(src, f), tmp) for f in names]
    x, v = s["x"].copy(), s["v"].copy()
    for _ in range(s["steps"]):
        fields = {"x": x, "m": s["m"], "l0": s["l0"]}
        fg, M, fs = (m.assemble(s["ep"], None, s["n"], fields) for m in maps)
        x, v = scenarios.esprings_step(s, x, v, fg, M, fs)
    return x


GOLD_TOL = 1e-13     # SIMIT_ASSERT_FLOAT_EQ for doubles


def test_reference_esprings_golden():
    """test/input/program/esprings.sim's maps generated for the host and its
    main restated: after 10 steps the positions the test asserts
    (test/program-esprings-test.cpp:106-145), to 1e-13."""
    from tests import scenarios
    src = _ref("test/input/program/esprings.sim")
    with tempfile.TemporaryDirectory() as tmp:
        x = _esprings_host(src, ("distribute_gravity", "distribute_masses",
                                 "compute_stiffness"), tmp)
    gold = scenarios.golden("esprings")
    assert len(gold) == 24
    for g in gold:
        assert abs(scenarios.golden_lookup(g, {"x": x}) - g["expected"]) <= GOLD_TOL, g


def test_own_explicit_springs_golden():
    """tests/sim/explicit_springs.sim on the host: the esprings test's
    positions after 10 steps."""
    from tests import scenarios
    with tempfile.TemporaryDirectory() as tmp:
        x = _esprings_host(_own("explicit_springs.sim"), ("weight", "lumped", "pull"), tmp)
    for g in scenarios.golden("esprings"):
        assert abs(scenarios.golden_lookup(g, {"x": x}) - g["expected"]) <= GOLD_TOL, g
