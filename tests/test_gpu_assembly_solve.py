"""GPU parity: element assembly and CG solves against the oracle and the
reference's golden values (all compute through the C ABI)."""
import numpy as np
import pytest
import torch

from simit_gb300 import _lib, meshgen, problems
from tests import scenarios

pytestmark = pytest.mark.gpu

GOLD_TOL = 1e-13


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


def _np(t):
    return t.detach().cpu().numpy()


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


def _cg_ref_form(ctx, mesh, vals, b, x0, bs, tol, maxiters, stop):
    """The reference's CG loop (no preconditioner, iterated residual test)."""
    from simit_gb300.runtime import Solver, solve_opts
    opts = solve_opts(precision=_lib.SOLVE_F64, precond=_lib.PRECOND_NONE, stop=stop, tol=tol,
                      maxiters=maxiters, verify=0)
    S = Solver(ctx, mesh.n, bs, mesh.pattern.rowptr, mesh.pattern.colidx, vals, mesh.nnzb, opts)
    x = x0.clone()
    res = S.solve(b, x)
    S.close()
    return x, res


# ---------------------------------------------------------------------------
# reference golden scenarios, end to end on the GPU
# ---------------------------------------------------------------------------
def test_isprings_golden_gpu(ctx, oracle):
    from simit_gb300.runtime import Mesh, assemble_springs
    s = scenarios.isprings_chain()
    mesh = Mesh(ctx, s["n"], s["ep"], 2)
    d = ctx.device
    x = torch.tensor(s["x"], device=d)
    v = torch.tensor(s["v"], device=d)
    for _ in range(s["steps"]):
        vals, f = assemble_springs(mesh, x, v, s["m"], s["fixed"], s["k"], s["l0"], s["h"],
                                   s["viscous"], s["grav"], form=s["form"])
        v, res = _cg_ref_form(ctx, mesh, vals, f, v, 3, s["tol2"], s["maxiters"],
                              _lib.STOP_NORMR2)
        with ctx.stream():
            x = x + s["h"] * v
    ctx.sync()
    fields = {"x": _np(x), "v": _np(v)}
    for g in scenarios.golden("isprings"):
        got = scenarios.golden_lookup(g, fields)
        assert abs(got - g["expected"]) <= GOLD_TOL, (g, got)


def test_springs_on_tetgen_edges_gpu(ctx, oracle, tmp_path):
    """apps/springs/springs.cpp end to end: the bar2k TetGen mesh's edges
    written as a .edge file, read back with the MeshVol::loadTetEdge rules,
    three implicit steps of apps/springs/isprings.sim (FP64, exact-mode
    assembly, at most 50 CG iterations) on the GPU against the oracle."""
    import os
    from simit_gb300.runtime import Mesh, assemble_springs
    node = os.path.join(scenarios.GOLDEN, "bar2k.node")
    _, tets = meshgen.load_tetgen(node, os.path.join(scenarios.GOLDEN, "bar2k.ele"))
    edge = str(tmp_path / "bar2k.edge")
    scenarios.write_tetgen_edges(edge, scenarios.tet_edges(tets))
    s = scenarios.springs_from_tetgen(node, edge)
    mesh = Mesh(ctx, s["n"], s["ep"], 2)
    rp, ci = mesh.pattern.host()
    d = ctx.device
    x, v = torch.tensor(s["x"], device=d), torch.tensor(s["v"], device=d)
    ox, ov = s["x"].copy(), s["v"].copy()
    for step in range(3):
        vals, f = assemble_springs(mesh, x, v, s["m"], s["fixed"], s["k"], s["l0"], s["h"],
                                   s["viscous"], s["grav"], form=s["form"])
        if step == 0:  # the ingested system itself: bit-exact with the oracle's
            oA, of = oracle.springs_assemble(s["form"], s["x"], s["v"], s["m"], s["fixed"],
                                             s["ep"], s["k"], s["l0"], s["h"], s["viscous"],
                                             s["grav"], rp, ci)
            assert np.array_equal(_np(vals), oA) and np.array_equal(_np(f), of)
        v, res = _cg_ref_form(ctx, mesh, vals, f, v, 3, s["tol2"], s["maxiters"],
                              _lib.STOP_NORMR2)
        with ctx.stream():
            x = x + s["h"] * v
        oracle.springs_step(s["form"], ox, ov, s["m"], s["fixed"], s["ep"], s["k"], s["l0"],
                            s["h"], s["viscous"], s["grav"], rp, ci, s["tol2"], s["maxiters"])
    ctx.sync()
    # 50 unconverged CG iterations per step (the app's cap): the iterates
    # follow the dot products' rounding, which differs in summation order
    assert np.abs(_np(v) - ov).max() <= 1e-4 * np.abs(ov).max()
    assert np.abs(_np(x) - ox).max() <= 1e-7 * np.abs(ox).max()


def test_cg_golden_gpu(ctx):
    from simit_gb300.runtime import Mesh, assemble_scalar_springs
    s = scenarios.cg_chain()
    mesh = Mesh(ctx, s["n"], s["ep"], 2)
    A = assemble_scalar_springs(mesh, s["a"], s["diag"], s["scale"])
    b = torch.tensor(s["b"], device=ctx.device)
    c, res = _cg_ref_form(ctx, mesh, A, b, torch.zeros_like(b), 1, s["tol"], s["maxiters"],
                          _lib.STOP_NORMR)
    for g in scenarios.golden("cg"):
        got = scenarios.golden_lookup(g, {"c": _np(c)})
        assert abs(got - g["expected"]) <= GOLD_TOL, (g, got)


def test_femtet_golden_gpu(ctx, oracle):
    from simit_gb300.runtime import (Mesh, assemble_tet_force, assemble_tet_stiffness,
                                     tet_precompute)
    s = scenarios.femtet_bar2k()
    mesh = Mesh(ctx, s["n"], s["tets"], 4)
    d = ctx.device
    x = torch.tensor(s["x"], device=d)
    v = torch.tensor(s["v"], device=d)
    B, W, m = tet_precompute(mesh, x, s["rho"])
    # parity of the precompute with the oracle (bit-exact inverse/det order)
    oB, oW, om = oracle.tet_precompute(s["x"], s["tets"], s["rho"])
    assert np.array_equal(_np(B), oB) and np.array_equal(_np(W), oW)
    assert np.array_equal(_np(m), om)
    nm = _lib.MODEL_NEOHOOKEAN
    for _ in range(s["steps"]):
        f = assemble_tet_force(mesh, nm, x, v, s["c"], B, W, s["u"], s["l"], s["h"], s["rho"],
                               s["grav"])
        A = assemble_tet_stiffness(mesh, nm, x, s["c"], B, W, s["u"], s["l"], s["h"], s["rho"])
        xs, res = _cg_ref_form(ctx, mesh, A, f, v, 3, s["tol2"], s["maxiters"],
                               _lib.STOP_NORMR2)
        v = xs
        with ctx.stream():
            x = s["h"] * xs + x
    ctx.sync()
    for g in scenarios.golden("femTet"):
        got = scenarios.golden_lookup(g, {"x": _np(x)})
        assert abs(got - g["expected"]) <= GOLD_TOL, (g, got)


# ---------------------------------------------------------------------------
# assembly parity on larger meshes
# ---------------------------------------------------------------------------
def test_element_block_assembly_golden_gpu(ctx):
    """sg_assemble_blocks + sg_bspmv reproduce the golden values of the
    reference's gemv_blocked, gemv_blocked_nw, gemv_blocked_computed and
    matrix_vv tests exactly (integers in FP64)."""
    from simit_gb300.runtime import Mesh, assemble_blocks, bspmv
    for name, n, ep, bs, eb, x in scenarios.element_block_scenarios():
        mesh = Mesh(ctx, n, ep, 2)
        vals = assemble_blocks(mesh, eb, bs, dtype=torch.float64, exact=True)
        with ctx.stream():
            xd = torch.tensor(x, dtype=torch.float64, device=ctx.device)
        y = _np(bspmv(ctx, n, bs, mesh.pattern.rowptr, mesh.pattern.colidx, vals, xd))
        want = [g["expected"] for g in scenarios.golden(name)]
        assert list(y) == want, (name, list(y), want)


@pytest.mark.parametrize("card,bs", [(2, 1), (2, 3), (3, 2), (4, 3), (4, 1)])
def test_element_block_assembly_matches_oracle(ctx, oracle, card, bs):
    """Random element blocks on a random edge set: FP64 exact mode
    bit-identical to the oracle's element-order `+=`; FP32 to 1e-6."""
    from simit_gb300.runtime import Mesh, assemble_blocks
    g = meshgen.rng(300 + 10 * card + bs)
    n, nE = 400, 1500
    ep = g.integers(0, n, size=nE * card).astype(np.int32)
    eb = g.uniform(-1, 1, size=(nE, card, card, bs, bs))
    mesh = Mesh(ctx, n, ep, card)
    rp, ci = mesh.pattern.host()
    ref = oracle.assemble_blocks(ep, card, bs, eb, rp, ci)
    got = _np(assemble_blocks(mesh, eb, bs, dtype=torch.float64, exact=True))
    assert np.array_equal(got, ref)
    got32 = _np(assemble_blocks(mesh, eb, bs, dtype=torch.float32, exact=False))
    scale = oracle.assemble_blocks(ep, card, bs, np.abs(eb), rp, ci)
    assert np.all(np.abs(got32 - ref) <= 1e-6 * scale + 1e-30)


@pytest.mark.parametrize("form", [0, 1])
def test_springs_assembly_exact(ctx, oracle, form):
    from simit_gb300.runtime import Mesh, assemble_springs
    L = meshgen.springs_lattice(10, 10, 10, 0.1, 0.01, seed=1)
    n = L["n"]
    g = meshgen.rng(2)
    v = g.uniform(-0.1, 0.1, n * 3)
    m = np.ones(n)
    k = np.full(len(L["l0"]), 1e4)
    l0 = L["l0"] * g.uniform(0.9, 1.1, len(L["l0"]))
    grav = np.array([0, 0, -9.81])
    mesh = Mesh(ctx, n, L["ep"], 2)
    rp, ci = mesh.pattern.host()
    vals, f = assemble_springs(mesh, L["x"], v, m, L["fixed"], k, l0, 1e-3, 0.5, grav, form=form)
    oA, of = oracle.springs_assemble(form, L["x"], v, m, L["fixed"], L["ep"], k, l0, 1e-3, 0.5,
                                     grav, rp, ci)
    ctx.sync()
    # same operation order, no contraction, element-order sums: bit-exact
    assert np.array_equal(_np(vals), oA)
    assert np.array_equal(_np(f), of)


def test_springs_assembly_fast_f32(ctx, oracle):
    from simit_gb300.runtime import Mesh, assemble_springs
    L = meshgen.springs_lattice(12, 11, 10, 0.1, 0.01, seed=3)
    n = L["n"]
    m = np.ones(n)
    k = np.full(len(L["l0"]), 1e4)
    l0 = L["l0"] * 0.97
    grav = np.array([0, 0, -9.81])
    v = np.zeros(n * 3)
    mesh = Mesh(ctx, n, L["ep"], 2)
    rp, ci = mesh.pattern.host()
    vals, f = assemble_springs(mesh, L["x"], v, m, L["fixed"], k, l0, 1e-3, 0.0, grav,
                               dtype=torch.float32, exact=False)
    oA, of = oracle.springs_assemble(0, L["x"], v, m, L["fixed"], L["ep"], k, l0, 1e-3, 0.0, grav,
                                     rp, ci)
    scale = np.abs(oA).max()
    assert np.abs(_np(vals).astype(np.float64) - oA).max() <= 1e-5 * scale


@pytest.mark.parametrize("exact", [True, False])
def test_linear_tet_stiffness(ctx, oracle, exact):
    from simit_gb300.runtime import Mesh, assemble_tet_stiffness, tet_precompute
    mg = meshgen.tet_grid(7, 6, 5, disp=1e-3, seed=4)
    n = mg["n"]
    g = meshgen.rng(5)
    nT = len(mg["tets"]) // 4
    E = 10 ** g.uniform(3, 6, nT)
    nu = g.uniform(0.35, 0.45, nT)
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    c = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    mesh = Mesh(ctx, n, mg["tets"], 4)
    rp, ci = mesh.pattern.host()
    B, W, m = tet_precompute(mesh, mg["X0"], 1e3)
    oB, oW, om = oracle.tet_precompute(mg["X0"], mg["tets"], 1e3)
    A = assemble_tet_stiffness(mesh, _lib.MODEL_LINEAR, mg["x"], c, B, W, mu, lam, 1.0, 1e3,
                               exact=exact)
    oA = oracle.tet_stiffness(0, mg["x"], c, mg["tets"], oB, oW, mu, lam, 1.0, 1e3, rp, ci)
    ctx.sync()
    if exact:
        assert np.array_equal(_np(A), oA)
    else:
        assert np.abs(_np(A) - oA).max() <= 1e-12 * np.abs(oA).max()


def test_neohookean_stiffness_and_force(ctx, oracle):
    from simit_gb300.runtime import (Mesh, assemble_tet_force, assemble_tet_stiffness,
                                     tet_precompute)
    mg = meshgen.tet_grid(6, 5, 4, disp=1e-3, seed=6)
    n = mg["n"]
    nT = len(mg["tets"]) // 4
    E, nu = 1e5, 0.4
    mu = np.full(nT, E / (2 * (1 + nu)))
    lam = np.full(nT, E * nu / ((1 + nu) * (1 - 2 * nu)))
    c = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    v = meshgen.rng(7).uniform(-0.01, 0.01, n * 3)
    grav = np.array([0, -9.81, 0])
    mesh = Mesh(ctx, n, mg["tets"], 4)
    rp, ci = mesh.pattern.host()
    B, W, _ = tet_precompute(mesh, mg["X0"], 1e3)
    oB, oW, _ = oracle.tet_precompute(mg["X0"], mg["tets"], 1e3)
    nm = _lib.MODEL_NEOHOOKEAN
    A = assemble_tet_stiffness(mesh, nm, mg["x"], c, B, W, mu, lam, 0.01, 1e3)
    f = assemble_tet_force(mesh, nm, mg["x"], v, c, B, W, mu, lam, 0.01, 1e3, grav)
    oA = oracle.tet_stiffness(1, mg["x"], c, mg["tets"], oB, oW, mu, lam, 0.01, 1e3, rp, ci)
    of = oracle.tet_force(1, mg["x"], v, c, mg["tets"], oB, oW, mu, lam, 0.01, 1e3, grav)
    ctx.sync()
    # within 1e-12 relative of the largest entry (log may differ by an ulp)
    assert np.abs(_np(A) - oA).max() <= 1e-12 * np.abs(oA).max()
    assert np.abs(_np(f) - of).max() <= 1e-12 * np.abs(of).max()
    fl = assemble_tet_force(mesh, _lib.MODEL_LINEAR, mg["x"], v, c, B, W, mu, lam, 0.01, 1e3,
                            grav)
    ofl = oracle.tet_force(0, mg["x"], v, c, mg["tets"], oB, oW, mu, lam, 0.01, 1e3, grav)
    ctx.sync()
    assert np.array_equal(_np(fl), ofl)


def test_heat_assembly(ctx, oracle):
    from simit_gb300.runtime import Mesh, assemble_heat, tet_precompute
    mg = meshgen.tet_grid(8, 7, 6)
    n = mg["n"]
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(8)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, n)
    mesh = Mesh(ctx, n, mg["tets"], 4)
    rp, ci = mesh.pattern.host()
    B, W, _ = tet_precompute(mesh, mg["x"], 1.0)
    oB, oW, _ = oracle.tet_precompute(mg["x"], mg["tets"], 1.0)
    A, b = assemble_heat(mesh, B, W, kappa, 1e-2, T0)
    oA, ob = oracle.heat_assemble(n, mg["tets"], oB, oW, kappa, 1e-2, T0, rp, ci)
    ctx.sync()
    assert np.array_equal(_np(A), oA) and np.array_equal(_np(b), ob)


def test_assembly_deterministic_f32(ctx):
    from simit_gb300.runtime import Mesh, assemble_tet_stiffness, tet_precompute
    mg = meshgen.tet_grid(10, disp=1e-3, seed=9)
    nT = len(mg["tets"]) // 4
    mu = np.full(nT, 3e4)
    lam = np.full(nT, 5e4)
    c = np.zeros(mg["n"], np.int32)
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], 1e3, dtype=torch.float32)
    a1 = assemble_tet_stiffness(mesh, 0, mg["x"], c, B, W, mu, lam, 1.0, 1e3,
                                dtype=torch.float32, exact=False).clone()
    a2 = assemble_tet_stiffness(mesh, 0, mg["x"], c, B, W, mu, lam, 1.0, 1e3,
                                dtype=torch.float32, exact=False)
    ctx.sync()
    assert torch.equal(a1, a2)


# ---------------------------------------------------------------------------
# solvers
# ---------------------------------------------------------------------------
def _elasticity_system(ctx, oracle, nx, dtype=torch.float64, seed=10):
    from simit_gb300.runtime import Mesh, assemble_tet_force, assemble_tet_stiffness, \
        tet_precompute
    mg = meshgen.tet_grid(nx, disp=1e-3, seed=seed)
    n = mg["n"]
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(seed + 1)
    E = 10 ** g.uniform(3, 6, nT)
    nu = g.uniform(0.35, 0.45, nT)
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    c = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    mesh = Mesh(ctx, n, mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], 1e3, dtype=dtype)
    A = assemble_tet_stiffness(mesh, 0, mg["x"], c, B, W, mu, lam, 1.0, 1e3, dtype=dtype,
                               exact=False)
    f = assemble_tet_force(mesh, 0, mg["x"], np.zeros(n * 3), c, B, W, mu, lam, 1.0, 1e3,
                           np.array([0, 0, -9.81]), dtype=dtype)
    return mesh, A, f.to(torch.float64)


def test_jacobi_pcg_f64_matches_oracle(ctx, oracle):
    from simit_gb300.runtime import Solver, solve_opts
    mesh, A, b = _elasticity_system(ctx, oracle, 8)
    rp, ci = mesh.pattern.host()
    S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
               solve_opts(precond=_lib.PRECOND_JACOBI, tol=1e-8, maxiters=20000))
    x = torch.zeros_like(b)
    res = S.solve(b, x)
    assert res.status == 1
    ox, oit, orr = oracle.jacobi_pcg(mesh.n, 3, rp, ci, _np(A), _np(b), np.zeros(mesh.n * 3),
                                     1e-8, 20000, refresh=0)
    assert orr <= 1e-8
    assert np.sqrt(res.true_normr2 / res.bnorm2) <= 1e-8
    assert abs(res.iters - oit) <= max(3, 0.02 * oit)
    assert oracle.relres(mesh.n, 3, rp, ci, _np(A), _np(b), _np(x)) <= 1.001e-8


@pytest.mark.parametrize("precond", [_lib.PRECOND_JACOBI, _lib.PRECOND_BLOCK_JACOBI])
def test_mixed_precision_reaches_fp64_tolerance(ctx, oracle, precond):
    from simit_gb300.runtime import Solver, solve_opts
    mesh, A32, b = _elasticity_system(ctx, oracle, 10, dtype=torch.float32)
    S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A32, mesh.nnzb,
               solve_opts(precision=_lib.SOLVE_MIXED, precond=precond, tol=1e-8,
                          maxiters=40000))
    x = torch.zeros_like(b)
    res = S.solve(b, x)
    assert res.status == 1, _lib.STATUS.get(res.status)
    assert np.sqrt(res.true_normr2 / res.bnorm2) <= 1e-8
    assert res.checks >= 1
    # the FP64 residual of the FP32-assembled system, recomputed by the oracle
    rp, ci = mesh.pattern.host()
    assert oracle.relres(mesh.n, 3, rp, ci, _np(A32), _np(b), _np(x)) <= 1.001e-8


def test_solver_deterministic_and_reusable(ctx, oracle):
    from simit_gb300.runtime import Solver, solve_opts
    mesh, A, b = _elasticity_system(ctx, oracle, 6)
    S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
               solve_opts(precond=_lib.PRECOND_JACOBI, tol=1e-9, maxiters=5000))
    x1 = torch.zeros_like(b)
    r1 = S.solve(b, x1)
    x2 = torch.zeros_like(b)
    r2 = S.solve(b, x2)
    assert r1.iters == r2.iters and torch.equal(x1, x2)


@pytest.mark.parametrize("precision", [_lib.SOLVE_MIXED, _lib.SOLVE_F64])
def test_zero_start_takes_b_as_residual(ctx, oracle, precision):
    """solve_ex(x_zero) starts from r = b without computing b - A 0: the
    same iterations and solution as a solve from an explicit zero guess."""
    from simit_gb300.runtime import Solver, solve_opts
    dt = torch.float32 if precision == _lib.SOLVE_MIXED else torch.float64
    mesh, A, b = _elasticity_system(ctx, oracle, 8, dtype=dt)
    S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
               solve_opts(precision=precision, precond=_lib.PRECOND_BLOCK_JACOBI, tol=1e-8,
                          maxiters=20000))
    x1 = torch.zeros_like(b)
    r1 = S.solve(b, x1)
    x2 = torch.full_like(b, 7.0)    # ignored: x_zero
    r2 = S.solve_ex(b, x2, x_zero=True)
    ctx.sync()
    assert r1.status == r2.status == 1
    assert r2.checks == r1.checks
    assert abs(r1.iters - r2.iters) <= 1
    assert float((x1 - x2).abs().max()) <= 1e-9 * float(x1.abs().max())
    rp, ci = mesh.pattern.host()
    assert oracle.relres(mesh.n, 3, rp, ci, _np(A), _np(b), _np(x2)) <= 1.001e-8


def test_solver_status_codes(ctx):
    from simit_gb300.runtime import Mesh, Solver, assemble_scalar_springs, solve_opts
    ep, n = meshgen.box_springs(5, 4, 3)
    mesh = Mesh(ctx, n, ep, 2)
    a = np.ones(len(ep) // 2)
    # negative definite: -I - 0.5*Laplacian -> p'Ap < 0 on the first step
    A = assemble_scalar_springs(mesh, a, -1.0, -0.5)
    b = torch.ones(n, dtype=torch.float64, device=ctx.device)
    S = Solver(ctx, n, 1, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
               solve_opts(tol=1e-12, maxiters=500))
    r = S.solve(b, torch.zeros_like(b))
    assert r.status == 3 and r.iters == 0
    # SPD, but too few iterations
    A2 = assemble_scalar_springs(mesh, a, 1.0, 0.5)
    S2 = Solver(ctx, n, 1, mesh.pattern.rowptr, mesh.pattern.colidx, A2, mesh.nnzb,
                solve_opts(tol=1e-14, maxiters=3))
    b = torch.tensor(meshgen.rng(5).uniform(-1, 1, n), device=ctx.device)
    r2 = S2.solve(b, torch.zeros_like(b))
    assert r2.status == 2 and r2.iters == 3
    # NaN in the right-hand side
    bn = b.clone()
    bn[3] = float("nan")
    r3 = S2.solve(bn, torch.zeros_like(b))
    assert r3.status == 4


def test_reordered_workload_solves_to_the_same_displacements(ctx, oracle):
    """The Hilbert-reordered workload (simit::reorder) is the same system
    renumbered: its solution, mapped back, solves the lattice-ordered system
    to the same FP64 residual (FP64 assembly, so the two matrices differ by
    element-order rounding only)."""
    h = problems.hetero_mesh(10)
    r = problems.reorder_hetero(h)
    vo = r["vertex_ordering"]
    sysm = []
    for H in (h, r):
        p = problems.HeteroElasticity(ctx, H, dtype=torch.float64, precond=_lib.PRECOND_JACOBI)
        res = p.step()
        ctx.sync()
        assert res.status == 1
        rp, ci = p.mesh.pattern.host()
        sysm.append((rp, ci, _np(p.A), _np(p.b), _np(p.u).reshape(-1, 3)))
        p.close()
    rp, ci, A0, b0, u0 = sysm[0]
    u1 = sysm[1][4][vo].reshape(-1)
    r0 = b0 - oracle.spmv(h["n"], 3, rp, ci, A0, u1)
    assert np.linalg.norm(r0) <= 1.01e-8 * np.linalg.norm(b0)


def test_thermal_jacobi_pcg_refresh_matches_oracle(ctx, oracle):
    """apps/thermal/thermal.sim:102-130's solver form on the P1 heat system
    (12^3 lattice, kappa log-uniform [1e-2, 1e2], dt 1e-2): point-Jacobi PCG
    with the true residual recomputed every 50 iterations (check_every), FP64,
    against the oracle's restatement of that loop — same convergence to
    1e-8 and iteration counts within 2 %."""
    from simit_gb300.runtime import Mesh, Solver, assemble_heat, solve_opts, tet_precompute
    mg = meshgen.tet_grid(12)
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(31)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, mg["n"])
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], 1.0)
    A, b = assemble_heat(mesh, B, W, kappa, 1e-2, T0)
    rp, ci = mesh.pattern.host()
    oB, oW, _ = oracle.tet_precompute(mg["X0"], mg["tets"], 1.0)
    oA, ob = oracle.heat_assemble(mg["n"], mg["tets"], oB, oW, kappa, 1e-2, T0, rp, ci)
    ctx.sync()
    assert np.array_equal(_np(A), oA) and np.array_equal(_np(b), ob)
    S = Solver(ctx, mesh.n, 1, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
               solve_opts(precond=_lib.PRECOND_JACOBI, tol=1e-8, maxiters=20000,
                          check_every=50))
    x = torch.zeros_like(b)
    res = S.solve(b, x)
    S.close()
    assert res.status == 1, _lib.STATUS.get(res.status)
    assert res.checks >= res.iters // 50
    ox, oit, orr = oracle.jacobi_pcg(mesh.n, 1, rp, ci, oA, ob, np.zeros(mesh.n), 1e-8, 20000,
                                     refresh=50)
    assert orr <= 1e-8 and np.sqrt(res.true_normr2 / res.bnorm2) <= 1e-8
    assert abs(res.iters - oit) <= max(3, 0.02 * oit)
    assert oracle.relres(mesh.n, 1, rp, ci, oA, ob, _np(x)) <= 1.001e-8
