"""`.sim` programs on the GPU: the front end's element functions, compiled
by NVRTC into the row-owner assembly, against the precompiled element
kernels and the oracle, bit for bit.  The programs are the ones under
tests/sim (written for this repository)."""
import os

import numpy as np
import pytest
import torch

from simit_gb300 import meshgen, simfront

pytestmark = pytest.mark.gpu

SIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sim")


def _own(name):
    with open(os.path.join(SIM, name)) as f:
        return f.read()


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_tet_matches_precompiled_kernel(ctx, dtype):
    """tests/sim/tet_closed_form.sim (per-element mu, lambda; constrained
    vertices; stiffness then lumped mass on the diagonal) compiled without
    contraction gives the precompiled linear-tet kernel's matrix bit for bit."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import Mesh, assemble_tet_stiffness, tet_precompute
    mg = meshgen.tet_grid(7, 6, 5, disp=1e-3, seed=2)
    nT, n = len(mg["tets"]) // 4, mg["n"]
    g = meshgen.rng(11)
    mu = 10 ** g.uniform(3, 5, nT)
    lam = 10 ** g.uniform(3, 5, nT)
    c = (g.uniform(0, 1, n) < 0.1).astype(np.int32)
    h, rho = 0.01, 1e3
    mesh = Mesh(ctx, n, mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], rho, dtype=dtype)
    A = assemble_tet_stiffness(mesh, _lib.MODEL_LINEAR, mg["x"], c, B, W, mu, lam, h, rho,
                               dtype=dtype, exact=False)
    sm = simfront.SimMap(ctx, _own("tet_closed_form.sim"), "tet_stiffness",
                         {"h": h, "rho": rho}, dtype=dtype, exact=True)
    got = sm.assemble(mesh, {"B": B, "W": W, "u": mu, "l": lam, "c": c})
    ctx.sync()
    k = mesh.nnzb * 9
    assert torch.equal(got[:k], A[:k])
    sm.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_heat_matches_precompiled_kernel_and_oracle(ctx, oracle, dtype):
    """tests/sim/heat_p1.sim: the precompiled heat kernel's matrix bit for
    bit, and in FP64 the oracle's."""
    from simit_gb300.runtime import Mesh, assemble_heat, tet_precompute
    mg = meshgen.tet_grid(6)
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(5)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, mg["n"])
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], 1.0, dtype=dtype)
    A, _ = assemble_heat(mesh, B, W, kappa, 1e-2, T0, dtype=dtype)
    sm = simfront.SimMap(ctx, _own("heat_p1.sim"), "heat", {"dt": 1e-2}, dtype=dtype)
    got = sm.assemble(mesh, {"B": B, "W": W, "kappa": kappa})
    ctx.sync()
    assert torch.equal(got[:mesh.nnzb], A[:mesh.nnzb])
    if dtype == torch.float64:
        rp, ci = mesh.pattern.host()
        o, _ = oracle.heat_assemble(mg["n"], mg["tets"], B.cpu().numpy(), W.cpu().numpy(),
                                    kappa, 1e-2, T0, rp, ci)
        assert np.array_equal(got[:mesh.nnzb].cpu().numpy(), o)
    sm.close()


def test_sim_vertex_map_with_component_writes(ctx):
    """tests/sim/point_mass.sim: a map over the vertices (a mesh whose
    elements are the vertices), a full block write and component writes."""
    from simit_gb300.runtime import Mesh
    n = 1000
    g = meshgen.rng(9)
    m = g.uniform(1.0, 2.0, n)
    fixed = g.uniform(0, 1, n) < 0.3
    mesh = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    sm = simfront.SimMap(ctx, _own("point_mass.sim"), "point_mass", {"damp": 0.5}, result="M")
    got = sm.assemble(mesh, {"m": m, "fixed": fixed})
    ctx.sync()
    rp, ci = mesh.pattern.host()
    assert np.array_equal(rp, np.arange(n + 1)) and np.array_equal(ci, np.arange(n))
    want = m[:, None, None] * np.eye(3)[None]
    free = ~fixed
    want[free, 0, 0] += 0.5 * m[free]
    want[free, 2, 2] += (2.0 * 0.5) * m[free]
    assert np.array_equal(got[:n * 9].cpu().numpy().reshape(n, 3, 3), want)
    sm.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_tet_force_vector_map_matches_precompiled_and_oracle(ctx, oracle, dtype):
    """tests/sim/tet_force.sim, a map whose result is a system vector,
    through the vertex-owner kernel generated for element_vector: the
    precompiled linear force kernel's values bit for bit, and in FP64 the
    oracle's (per-tet parameters, constrained vertices, momentum)."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import Mesh, assemble_tet_force, tet_precompute
    mg = meshgen.tet_grid(7, 6, 5, disp=1e-3, seed=4)
    nT, n = len(mg["tets"]) // 4, mg["n"]
    g = meshgen.rng(15)
    mu = 10 ** g.uniform(3, 5, nT)
    lam = 10 ** g.uniform(3, 5, nT)
    c = (g.uniform(0, 1, n) < 0.1).astype(np.int32)
    v = g.uniform(-0.01, 0.01, n * 3)
    h, rho, grav = 0.01, 1e3, np.array([0.0, -9.81, 0.0])
    mesh = Mesh(ctx, n, mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], rho, dtype=dtype)
    want = assemble_tet_force(mesh, _lib.MODEL_LINEAR, mg["x"], v, c, B, W, mu, lam, h, rho,
                              grav, dtype=dtype, exact=True)
    sm = simfront.SimMap(ctx, _own("tet_force.sim"), "tet_force",
                         {"h": h, "rho": rho, "gx": 0.0, "gy": -9.81, "gz": 0.0},
                         dtype=dtype, exact=True)
    got = sm.assemble(mesh, {"B": B, "W": W, "u": mu, "l": lam, "c": c, "x": mg["x"], "v": v})
    ctx.sync()
    assert torch.equal(got[:n * 3], want[:n * 3])
    if dtype == torch.float64:
        of = oracle.tet_force(0, mg["x"], v, c, mg["tets"], B.cpu().numpy(), W.cpu().numpy(),
                              mu, lam, h, rho, grav)
        assert np.array_equal(got[:n * 3].cpu().numpy(), of)
    sm.close()


def test_sim_vertex_map_vector_result(ctx):
    """tests/sim/point_mass.sim's vector result g (a map over the
    vertices): m (0, -9.8, 0) per vertex."""
    from simit_gb300.runtime import Mesh
    n = 777
    m = meshgen.rng(16).uniform(1.0, 2.0, n)
    fixed = np.zeros(n, bool)
    mesh = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    sm = simfront.SimMap(ctx, _own("point_mass.sim"), "point_mass", {"damp": 0.5}, result="g")
    got = sm.assemble(mesh, {"m": m, "fixed": fixed})
    ctx.sync()
    want = np.zeros((n, 3))
    want[:, 1] = -9.8 * m
    assert np.array_equal(got[:n * 3].cpu().numpy().reshape(n, 3), want)
    sm.close()


def _cloth_case(oracle, side, seed, noise=0.03):
    mg = meshgen.cloth_mesh(side)
    K, rest = oracle.cloth_faces(mg["x"], mg["faces"])
    ang, ln, perp = oracle.cloth_hinges(mg["x"], mg["hinges"])
    x = mg["x"] + meshgen.rng(seed).normal(0.0, noise, mg["x"].size)
    return dict(mg=mg, n=mg["n"], K=K, rest=rest, ang=ang, ln=ln, perp=perp, x=x)


def _relerr(got, want):
    return float(np.abs(got - want).max() / np.abs(want).max())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_cloth_forces_match_oracle(ctx, oracle, dtype):
    """tests/sim/cloth_forces.sim's stretch (faces, card 3) and bend (hinges,
    card 4) through the vertex-owner kernel against the oracle's
    restatement of apps/cloth/cloth.sim:142-173 on a perturbed 33 x 33
    sheet.  FP64: stretching bit for bit; bending within 1e-12 of the
    largest force (its angle is the device's atan2, a few ulps from the
    host's).  FP32: both within 1e-4 of the largest force."""
    from simit_gb300.runtime import Mesh
    k = _cloth_case(oracle, 33, 31)
    mg, n = k["mg"], k["n"]
    tris = Mesh(ctx, n, mg["faces"], 3)
    hin = Mesh(ctx, n, mg["hinges"], 4)
    src = _own("cloth_forces.sim")
    st = simfront.SimMap(ctx, src, "stretch", dtype=dtype, exact=True)
    bd = simfront.SimMap(ctx, src, "bend", dtype=dtype, exact=True)
    fs = st.assemble(tris, {"x": k["x"], "rest": k["rest"], "K": k["K"]})
    fb = bd.assemble(hin, {"x": k["x"], "len": k["ln"], "perp": k["perp"], "theta0": k["ang"]})
    ctx.sync()
    ws = oracle.cloth_stretch(n, k["x"], mg["faces"], k["K"], k["rest"])
    wb = oracle.cloth_bend(n, k["x"], mg["hinges"], k["ang"], k["ln"], k["perp"])
    gs = fs[:n * 3].double().cpu().numpy()
    gb = fb[:n * 3].double().cpu().numpy()
    if dtype == torch.float64:
        assert np.array_equal(gs, ws)
        assert _relerr(gb, wb) <= 1e-12
    else:
        assert _relerr(gs, ws) <= 1e-4
        assert _relerr(gb, wb) <= 1e-4
    st.close()
    bd.close()


def test_sim_cloth_step_matches_oracle(ctx, oracle):
    """One explicit step of the cloth example's `main` (cloth.sim:201-222)
    with tests/sim/cloth_forces.sim's maps on the GPU: x += dt v, points
    inside the radius-2 sphere projected onto it, stretching and bending
    forces, gravity, the inverse lumped mass (a diagonal system matrix)
    applied by the blocked SpMV, v += dt (g + Minv F).  Against the oracle's
    step: positions bit for bit, velocities within 1e-12 of the largest."""
    from simit_gb300.runtime import Mesh, bspmv
    k = _cloth_case(oracle, 25, 33, noise=0.01)
    mg, n = k["mg"], k["n"]
    g = meshgen.rng(34)
    # the sheet lies on y = 2 over the sphere's top: some points start inside
    x0 = k["x"].copy()
    x0[1::3] -= 0.02
    v0 = g.normal(0.0, 0.5, n * 3)
    m = g.uniform(0.5, 1.5, n)
    fixed = (g.uniform(0, 1, n) < 0.1).astype(np.int32)
    dt, ks, kb, damping = 1e-5, 1e5, 1.0, 1e-3
    src = _own("cloth_forces.sim")
    tris = Mesh(ctx, n, mg["faces"], 3)
    hin = Mesh(ctx, n, mg["hinges"], 4)
    pts = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    maps = {f: simfront.SimMap(ctx, src, f, exact=True)
            for f in ("stretch", "bend", "gravity", "inv_mass")}
    dev = ctx.device
    x = torch.as_tensor(x0, device=dev)
    v = torch.as_tensor(v0, device=dev)
    x = x + dt * v
    P = x.view(n, 3)
    dist = torch.sqrt((P[:, 0] * P[:, 0] + P[:, 1] * P[:, 1]) + P[:, 2] * P[:, 2])
    inside = (dist < 2.0)[:, None]
    newpos = (2.0 * P) / dist[:, None]
    V = torch.where(inside, v.view(n, 3) + (newpos - P) / dt, v.view(n, 3))
    P = torch.where(inside, 1.0 * newpos, P)
    x, v = P.reshape(-1).contiguous(), V.reshape(-1).contiguous()
    fs = maps["stretch"].assemble(tris, {"x": x, "rest": k["rest"], "K": k["K"]})
    fb = maps["bend"].assemble(hin, {"x": x, "len": k["ln"], "perp": k["perp"],
                                     "theta0": k["ang"]})
    gf = maps["gravity"].assemble(pts, {})
    Mi = maps["inv_mass"].assemble(pts, {"m": m, "fixed": fixed})
    tot = (fs * ks + fb * kb) - damping * v
    y = bspmv(ctx, n, 3, pts.pattern.rowptr, pts.pattern.colidx, Mi, tot)
    v = v + dt * (gf + y)
    ctx.sync()
    wx, wv = oracle.cloth_step(x0, v0, m, fixed, mg["faces"], k["K"], k["rest"], mg["hinges"],
                               k["ang"], k["ln"], k["perp"], dt, ks, kb, damping)
    assert bool(inside.any()) and not bool(inside.all())
    assert np.array_equal(x.cpu().numpy(), wx)
    assert _relerr(v.cpu().numpy(), wv) <= 1e-12
    for sm in maps.values():
        sm.close()


def test_sim_nested_blocks_on_gpu(ctx, oracle):
    """tests/sim/nested_blocks.sim on the GPU: couple (3x3 blocks of 2x2
    blocks over links, stored as 6x6: whole nested blocks, an inner block and
    a single component written) and spread / mark (vectors of nested rows,
    component writes) bit for bit against the numpy restatement; the blocked
    SpMV (bs 6) of the two within 1e-13 of the oracle's; weigh, a map over a
    system-vector argument, bit for bit against its restatement from that
    product."""
    from simit_gb300.runtime import Mesh, bspmv
    from tests.test_simfront_cpu import _nested_case, nested_blocks_expected
    src = _own("nested_blocks.sim")
    n = 40
    links, w, s, rp, ci = _nested_case(oracle, n, 150, 43)
    Kw, vw, mw = nested_blocks_expected(n, links, w, s)
    lk = Mesh(ctx, n, links.reshape(-1), 2)
    pts = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    grp, gci = lk.pattern.host()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
    maps = {f: simfront.SimMap(ctx, src, f, exact=True)
            for f in ("couple", "spread", "mark", "weigh")}
    K = maps["couple"].assemble(lk, {"w": w})
    v = maps["spread"].assemble(pts, {"s": s})
    m = maps["mark"].assemble(lk, {"w": w})
    y = bspmv(ctx, n, 6, lk.pattern.rowptr, lk.pattern.colidx, K, v)
    z = maps["weigh"].assemble(pts, {"y": y})
    ctx.sync()
    Kh = K[:len(ci) * 36].cpu().numpy()
    for r in range(n):
        for k in range(rp[r], rp[r + 1]):
            want = Kw.get((r, int(ci[k])), np.zeros((6, 6)))
            assert np.array_equal(Kh[k * 36:(k + 1) * 36].reshape(6, 6), want), (r, ci[k])
    assert np.array_equal(v[:n * 6].cpu().numpy(), vw)
    assert np.array_equal(m[:n * 2].cpu().numpy(), mw)
    yh = y[:n * 6].cpu().numpy()
    yo = oracle.spmv(n, 6, rp, ci, Kh, vw)
    assert np.abs(yh - yo).max() <= 1e-13 * np.abs(yo).max()
    Y = yh.reshape(n, 3, 2)
    want = np.zeros(n)
    for a in range(3):
        want = (want + (a + 1.0) * Y[:, a, 0]) - Y[:, a, 1]
    assert np.array_equal(z[:n].cpu().numpy(), want)
    for sm in maps.values():
        sm.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_nine_by_nine_nested_blocks(ctx, dtype):
    """tests/sim/nested_blocks.sim's fill9 / lift9 / total9 on the GPU: 3x3
    blocks of 3x3 blocks (bs 9 in the row-owner assembly and the SpMV) give
    the blocked assembly test's values, z = 81 k^2 (81, 324, 729 for
    k = 1, 2, 3), exactly."""
    from simit_gb300.runtime import Mesh, bspmv
    src = _own("nested_blocks.sim")
    k = np.array([1, 2, 3, 4, 5], np.int32)
    n = len(k)
    pts = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    maps = {f: simfront.SimMap(ctx, src, f, dtype=dtype, exact=True)
            for f in ("fill9", "lift9", "total9")}
    X = maps["fill9"].assemble(pts, {"k": k})
    x = maps["lift9"].assemble(pts, {"k": k})
    y = bspmv(ctx, n, 9, pts.pattern.rowptr, pts.pattern.colidx, X, x)
    z = maps["total9"].assemble(pts, {"y": y})
    ctx.sync()
    assert np.array_equal(X[:n * 81].cpu().numpy().reshape(n, 81),
                          np.repeat(k[:, None], 81, 1).astype(np.float64))
    assert z[:n].cpu().numpy().tolist() == (81 * k.astype(np.int64) ** 2).tolist()
    for sm in maps.values():
        sm.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_assembly_forms_give_reference_test_values(ctx, dtype):
    """tests/sim/assembly_forms.sim on the GPU, on the inputs of the
    reference's vector assembly tests (test/assembly-tests.cpp:12-217): maps
    over the vertices and over the edges themselves, over edge sets of one,
    two and three endpoints, and two-result maps whose matrix times vector
    is taken by the blocked SpMV give those tests' values exactly."""
    from simit_gb300.runtime import Mesh, bspmv
    from tests.test_simfront_cpu import OWN_FORMS, VECTOR_ASSEMBLY_CASES, run_vector_case
    keep = []

    def vmap(info, n, ep, fields):
        mesh = Mesh(ctx, n, ep, info["card"])
        sm = simfront.SimMap.from_info(ctx, info, dtype=dtype)
        keep.append(sm)
        return sm.assemble(mesh, fields)

    def mmap(info, n, ep, fields):
        mesh = Mesh(ctx, n, ep, info["card"])
        sm = simfront.SimMap.from_info(ctx, info, dtype=dtype)
        keep.append(sm)
        keep.append(mesh)
        return sm.assemble(mesh, fields), mesh.pattern.rowptr, mesh.pattern.colidx

    def spmv(n, rp, ci, A, x):
        return bspmv(ctx, n, 1, rp, ci, A, x)

    src = _own("assembly_forms.sim")
    for case in VECTOR_ASSEMBLY_CASES:
        got = run_vector_case(case, src, OWN_FORMS, vmap, mmap, spmv)
        ctx.sync()
        assert got[:case[1]].cpu().tolist() == case[5], case[0]
    for sm in keep:
        if isinstance(sm, simfront.SimMap):
            sm.close()


def test_sim_explicit_springs_golden(ctx):
    """tests/sim/explicit_springs.sim on the GPU: the three vector maps of
    the explicit springs step through the vertex-owner kernel, the update
    p = M v + h (fs + fg), v = p / M, x += h v in device arrays; after 10
    steps the positions test/program-esprings-test.cpp asserts, to 1e-13."""
    from simit_gb300.runtime import Mesh
    from tests import scenarios
    s = scenarios.esprings_cube()
    src = _own("explicit_springs.sim")
    mesh = Mesh(ctx, s["n"], s["ep"], 2)
    maps = [simfront.SimMap(ctx, src, f) for f in ("weight", "lumped", "pull")]
    d = ctx.device
    x = torch.tensor(s["x"], device=d)
    v = torch.tensor(s["v"], device=d)
    for _ in range(s["steps"]):
        fg, M, fs = (m.assemble(mesh, {"x": x, "m": s["m"], "l0": s["l0"]}) for m in maps)
        x, v = scenarios.esprings_step(s, x, v, fg[:s["n"] * 3], M[:s["n"] * 3],
                                       fs[:s["n"] * 3])
    ctx.sync()
    xh = x.cpu().numpy()
    for g in scenarios.golden("esprings"):
        assert abs(scenarios.golden_lookup(g, {"x": xh}) - g["expected"]) <= 1e-13, g
    for m in maps:
        m.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_precompiled_cloth_forces(ctx, oracle, dtype):
    """sg_assemble_cloth_stretch / sg_assemble_cloth_bend, the precompiled
    kernels of the cloth example's forces: FP64 stretching bit for bit
    against the oracle, bending within 1e-12 of the largest force (device
    atan2); in both precisions the run-time compiled maps of
    tests/sim/cloth_forces.sim give the same values bit for bit."""
    from simit_gb300.runtime import Mesh, assemble_cloth_bend, assemble_cloth_stretch
    k = _cloth_case(oracle, 29, 35)
    mg, n = k["mg"], k["n"]
    tris = Mesh(ctx, n, mg["faces"], 3)
    hin = Mesh(ctx, n, mg["hinges"], 4)
    fs = assemble_cloth_stretch(tris, k["x"], k["K"], k["rest"], dtype=dtype)
    fb = assemble_cloth_bend(hin, k["x"], k["ang"], k["ln"], k["perp"], dtype=dtype)
    src = _own("cloth_forces.sim")
    st = simfront.SimMap(ctx, src, "stretch", dtype=dtype, exact=True)
    bd = simfront.SimMap(ctx, src, "bend", dtype=dtype, exact=True)
    js = st.assemble(tris, {"x": k["x"], "rest": k["rest"], "K": k["K"]})
    jb = bd.assemble(hin, {"x": k["x"], "len": k["ln"], "perp": k["perp"], "theta0": k["ang"]})
    ctx.sync()
    assert torch.equal(fs[:n * 3], js[:n * 3])
    assert torch.equal(fb[:n * 3], jb[:n * 3])
    ws = oracle.cloth_stretch(n, k["x"], mg["faces"], k["K"], k["rest"])
    wb = oracle.cloth_bend(n, k["x"], mg["hinges"], k["ang"], k["ln"], k["perp"])
    gs, gb = fs[:n * 3].double().cpu().numpy(), fb[:n * 3].double().cpu().numpy()
    if dtype == torch.float64:
        assert np.array_equal(gs, ws)
        assert _relerr(gb, wb) <= 1e-12
    else:
        assert _relerr(gs, ws) <= 1e-4 and _relerr(gb, wb) <= 1e-4
    st.close()
    bd.close()
