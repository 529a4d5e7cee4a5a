"""GPU checks of the element-parallel assembly plans: the colouring is valid
and deterministic, the inverse slot map lists every element block once in
ascending order, and the stiffness, force and heat maps of both plans (the
coloured one and element blocks + slot gather) agree with the oracle (FP64)
and with the row-owner kernels, stay exactly symmetric in FP32 and are
bit-identical run to run."""
import numpy as np
import pytest
import torch

from simit_gb300 import _lib, meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


def _np(t):
    return t.detach().cpu().numpy()


def _tets(nx, ny=None, nz=None, seed=4):
    mg = meshgen.tet_grid(nx, ny, nz, disp=1e-3, seed=seed)
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(seed + 1)
    E = 10 ** g.uniform(3, 6, nT)
    nu = g.uniform(0.35, 0.45, nT)
    mg["mu"] = E / (2 * (1 + nu))
    mg["lam"] = E * nu / ((1 + nu) * (1 - 2 * nu))
    mg["c"] = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    return mg


@pytest.mark.parametrize("nx", [3, 9])
def test_coloring_is_valid_and_deterministic(ctx, nx):
    from simit_gb300.runtime import Mesh
    mg = _tets(nx)
    tets = mg["tets"].reshape(-1, 4)
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4, colored=True)
    cp, order = mesh.colors()
    assert cp[0] == 0 and cp[-1] == len(tets) and mesh.ncolors == len(cp) - 1
    assert np.array_equal(np.sort(order), np.arange(len(tets)))
    for k in range(mesh.ncolors):
        els = order[cp[k]:cp[k + 1]]
        assert len(els) > 0 and np.all(np.diff(els) > 0)
        verts = tets[els].reshape(-1)
        assert len(np.unique(verts)) == len(verts), "colour %d shares a vertex" % k
    mesh2 = Mesh(ctx, mg["n"], mg["tets"], 4, colored=True)
    cp2, order2 = mesh2.colors()
    assert cp == cp2 and np.array_equal(order, order2)
    print("%d^3 lattice: %d elements in %d colours" % (nx, len(tets), mesh.ncolors))


def test_coloring_repeated_endpoints(ctx):
    """Elements that list a vertex twice (degenerate springs) still colour:
    no two elements of a colour share a vertex."""
    from simit_gb300.runtime import Mesh
    n = 50
    g = meshgen.rng(3)
    ep = g.integers(0, n, size=(300, 2)).astype(np.int32)
    ep[::7, 1] = ep[::7, 0]
    mesh = Mesh(ctx, n, ep.reshape(-1), 2, colored=True)
    cp, order = mesh.colors()
    assert np.array_equal(np.sort(order), np.arange(len(ep)))
    for k in range(mesh.ncolors):
        verts = np.unique(ep[order[cp[k]:cp[k + 1]]].reshape(-1))
        used = [set(ep[e]) for e in order[cp[k]:cp[k + 1]]]
        assert sum(len(u) for u in used) == len(verts)


@pytest.mark.parametrize("plan", ["colored", "gather"])
def test_plan_linear_tet_f64_matches_oracle_and_row_owners(ctx, oracle, plan):
    from simit_gb300.runtime import Mesh, assemble_tet_force, assemble_tet_stiffness, \
        tet_precompute
    mg = _tets(7, 6, 5)
    n = mg["n"]
    plain = Mesh(ctx, n, mg["tets"], 4)
    col = Mesh(ctx, n, mg["tets"], 4, plan=plan)
    rp, ci = plain.pattern.host()
    B, W, _ = tet_precompute(plain, mg["X0"], 1e3)
    oB, oW, _ = oracle.tet_precompute(mg["X0"], mg["tets"], 1e3)
    args = (mg["x"], mg["c"], B, W, mg["mu"], mg["lam"], 1.0, 1e3)
    Ar = assemble_tet_stiffness(plain, _lib.MODEL_LINEAR, *args, exact=False)
    Ac = assemble_tet_stiffness(col, _lib.MODEL_LINEAR, *args, exact=False)
    oA = oracle.tet_stiffness(0, mg["x"], mg["c"], mg["tets"], oB, oW, mg["mu"], mg["lam"], 1.0,
                              1e3, rp, ci)
    v = meshgen.rng(7).uniform(-0.01, 0.01, n * 3)
    grav = np.array([0, 0, -9.81])
    fr = assemble_tet_force(plain, _lib.MODEL_LINEAR, mg["x"], v, mg["c"], B, W, mg["mu"],
                            mg["lam"], 1.0, 1e3, grav, exact=False)
    fc = assemble_tet_force(col, _lib.MODEL_LINEAR, mg["x"], v, mg["c"], B, W, mg["mu"],
                            mg["lam"], 1.0, 1e3, grav, exact=False)
    of = oracle.tet_force(0, mg["x"], v, mg["c"], mg["tets"], oB, oW, mg["mu"], mg["lam"], 1.0,
                          1e3, grav)
    ctx.sync()
    # assembled values within 1e-12 of the largest entry (colour-order sums)
    s = np.abs(oA).max()
    assert np.abs(_np(Ac) - oA).max() <= 1e-12 * s
    assert np.abs(_np(Ac) - _np(Ar)).max() <= 1e-12 * s
    sf = np.abs(of).max()
    assert np.abs(_np(fc) - of).max() <= 1e-12 * sf
    assert np.abs(_np(fc) - _np(fr)).max() <= 1e-12 * sf


@pytest.mark.parametrize("plan", ["colored", "gather"])
def test_plan_neohookean_f64_matches_oracle(ctx, oracle, plan):
    from simit_gb300.runtime import Mesh, assemble_tet_force, assemble_tet_stiffness, \
        tet_precompute
    mg = meshgen.tet_grid(6, 5, 4, disp=1e-3, seed=6)
    n = mg["n"]
    nT = len(mg["tets"]) // 4
    mu = np.full(nT, 1e5 / 2.8)
    lam = np.full(nT, 1e5 * 0.4 / (1.4 * 0.2))
    c = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    v = meshgen.rng(7).uniform(-0.01, 0.01, n * 3)
    grav = np.array([0, -9.81, 0])
    mesh = Mesh(ctx, n, mg["tets"], 4, plan=plan)
    rp, ci = mesh.pattern.host()
    B, W, _ = tet_precompute(mesh, mg["X0"], 1e3)
    oB, oW, _ = oracle.tet_precompute(mg["X0"], mg["tets"], 1e3)
    nm = _lib.MODEL_NEOHOOKEAN
    A = assemble_tet_stiffness(mesh, nm, mg["x"], c, B, W, mu, lam, 0.01, 1e3, exact=False)
    f = assemble_tet_force(mesh, nm, mg["x"], v, c, B, W, mu, lam, 0.01, 1e3, grav, exact=False)
    oA = oracle.tet_stiffness(1, mg["x"], c, mg["tets"], oB, oW, mu, lam, 0.01, 1e3, rp, ci)
    of = oracle.tet_force(1, mg["x"], v, c, mg["tets"], oB, oW, mu, lam, 0.01, 1e3, grav)
    ctx.sync()
    assert np.abs(_np(A) - oA).max() <= 1e-12 * np.abs(oA).max()
    assert np.abs(_np(f) - of).max() <= 1e-12 * np.abs(of).max()


@pytest.mark.parametrize("plan", ["colored", "gather"])
def test_plan_heat_matches_oracle(ctx, oracle, plan):
    from simit_gb300.runtime import Mesh, assemble_heat, tet_precompute
    mg = meshgen.tet_grid(8, 7, 6)
    n = mg["n"]
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(8)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, n)
    mesh = Mesh(ctx, n, mg["tets"], 4, plan=plan)
    rp, ci = mesh.pattern.host()
    B, W, _ = tet_precompute(mesh, mg["x"], 1.0)
    oB, oW, _ = oracle.tet_precompute(mg["x"], mg["tets"], 1.0)
    A, b = assemble_heat(mesh, B, W, kappa, 1e-2, T0, exact=False)
    oA, ob = oracle.heat_assemble(n, mg["tets"], oB, oW, kappa, 1e-2, T0, rp, ci)
    ctx.sync()
    assert np.abs(_np(A) - oA).max() <= 1e-12 * np.abs(oA).max()
    assert np.abs(_np(b) - ob).max() <= 1e-12 * np.abs(ob).max()
    # exact mode ignores the plan: the reference's element order, bit for bit
    Ae, be = assemble_heat(mesh, B, W, kappa, 1e-2, T0, exact=True)
    ctx.sync()
    assert np.array_equal(_np(Ae), oA) and np.array_equal(_np(be), ob)


@pytest.mark.parametrize("plan", ["colored", "gather"])
def test_plan_f32_symmetric_deterministic(ctx, plan):
    """FP32: the plan's stiffness equals the row-owner one to FP32
    rounding, is bitwise symmetric (block (j, i) the transpose of (i, j)),
    and two runs give the same bits."""
    from simit_gb300.runtime import Mesh, assemble_tet_stiffness, tet_precompute
    mg = _tets(10, seed=9)
    n = mg["n"]
    plain = Mesh(ctx, n, mg["tets"], 4)
    col = Mesh(ctx, n, mg["tets"], 4, plan=plan)
    f32 = torch.float32
    B, W, _ = tet_precompute(plain, mg["X0"], 1e3, dtype=f32)
    args = (mg["x"], mg["c"], B, W, mg["mu"], mg["lam"], 1.0, 1e3)
    Ar = assemble_tet_stiffness(plain, 0, *args, dtype=f32, exact=False)
    A1 = assemble_tet_stiffness(col, 0, *args, dtype=f32, exact=False).clone()
    A2 = assemble_tet_stiffness(col, 0, *args, dtype=f32, exact=False)
    ctx.sync()
    assert torch.equal(A1, A2)
    a, r = _np(A1).astype(np.float64), _np(Ar).astype(np.float64)
    # row sums of |A| bound the rounding of each entry's sum
    assert np.abs(a - r).max() <= 1e-6 * np.abs(r).max()
    rp, ci = plain.pattern.host()
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    blk = _np(A1).reshape(-1, 3, 3)
    key = {(int(i), int(j)): q for q, (i, j) in enumerate(zip(rows, ci))}
    tq = np.array([key[(int(j), int(i))] for i, j in zip(rows, ci)])
    assert np.array_equal(blk, np.transpose(blk[tq], (0, 2, 1)))


def test_slot_sources_invert_the_slot_map(ctx):
    """Every element block appears once, in its own slot's list, ascending."""
    from simit_gb300.runtime import Mesh
    mg = meshgen.tet_grid(5, 4, 3)
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4, plan="gather")
    slots = mesh.pattern.slots[:mesh.nE * 16].cpu().numpy().view(np.uint32).astype(np.int64)
    sp = mesh.slot_src_ptr.cpu().numpy().view(np.uint32).astype(np.int64)
    src = mesh.slot_src[:mesh.nE * 16].cpu().numpy().view(np.uint32).astype(np.int64)
    assert sp[0] == 0 and sp[-1] == len(slots)
    assert np.array_equal(np.sort(src), np.arange(len(slots)))
    for q in range(mesh.nnzb):
        lst = src[sp[q]:sp[q + 1]]
        assert np.all(np.diff(lst) > 0) and np.all(slots[lst] == q)


def test_gather_plan_repeated_endpoints(ctx):
    """Element blocks of springs that list a vertex twice land in one slot;
    the gather sums them with the rest (FP64, against the row owners)."""
    from simit_gb300.runtime import Mesh, assemble_blocks
    n = 40
    g = meshgen.rng(11)
    ep = g.integers(0, n, size=(200, 2)).astype(np.int32)
    ep[::5, 1] = ep[::5, 0]
    eb = g.normal(size=200 * 4 * 9)
    plain = Mesh(ctx, n, ep.reshape(-1), 2)
    gat = Mesh(ctx, n, ep.reshape(-1), 2, plan="gather")
    a = assemble_blocks(plain, eb, 3, exact=False)
    b = assemble_blocks(gat, eb, 3, exact=False)
    ctx.sync()
    assert np.allclose(_np(a), _np(b), rtol=1e-13, atol=1e-13 * np.abs(_np(a)).max())
