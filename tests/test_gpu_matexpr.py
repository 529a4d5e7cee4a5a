"""GPU parity of the system-matrix expression D + s*K (sg_bsr_add_diag)
against the oracle's lowered `MDK = MD + K` loop, bit-exact, and the unfused
isprings composition (K alone, then MD + K) against the fused assembly."""
import numpy as np
import pytest
import torch

from simit_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


def _system(oracle, n, nE, bs, seed, dt, with_diag=True):
    g = meshgen.rng(seed)
    ep = g.integers(0, n, size=nE * 2).astype(np.int32)
    if with_diag:  # a self-edge per vertex: every row holds its diagonal block
        ep = np.concatenate([ep, np.repeat(np.arange(n, dtype=np.int32), 2)])
    rp, ci = oracle.pattern(n, ep, 2)
    K = g.uniform(-1, 1, size=len(ci) * bs * bs).astype(dt)
    K[::7] = -0.0  # signed zeros: 0 + (-0) is +0 in the lowered loop
    D = g.uniform(-2, 2, size=n * bs * bs).astype(dt)
    return rp, ci, K, D


def _t(a, d):
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [1, 2, 3])
@pytest.mark.parametrize("mode", ["diag", "ident", "none"])
@pytest.mark.parametrize("scale", [1.0, -0.37])
def test_add_diag_bit_exact(ctx, oracle, dt, bs, mode, scale):
    from simit_gb300.runtime import bsr_add_diag
    n = 1500
    rp, ci, K, D = _system(oracle, n, 5000, bs, 11 + bs, dt)
    d = ctx.device
    kw = {"diag": D, "ident": 0.0} if mode == "diag" else (
        {"diag": None, "ident": 2.5} if mode == "ident" else {"diag": None, "ident": 0.0})
    ref = oracle.add_diag(n, bs, rp, ci, K, scale=scale, **kw)
    got = bsr_add_diag(ctx, n, bs, _t(rp, d), _t(ci, d), _t(K, d),
                       diag=None if kw["diag"] is None else _t(D, d), ident=kw["ident"],
                       scale=scale)
    ctx.sync()
    g = got.cpu().numpy()
    assert g.tobytes() == ref.tobytes()  # bit-exact, signed zeros included


def test_add_diag_in_place(ctx, oracle):
    from simit_gb300.runtime import bsr_add_diag
    n = 800
    rp, ci, K, D = _system(oracle, n, 3000, 3, 5, np.float32)
    d = ctx.device
    ref = oracle.add_diag(n, 3, rp, ci, K, diag=D, scale=0.5)
    Kd = _t(K.copy(), d)
    out = bsr_add_diag(ctx, n, 3, _t(rp, d), _t(ci, d), Kd, diag=_t(D, d), scale=0.5, out=Kd)
    ctx.sync()
    assert out.data_ptr() == Kd.data_ptr()
    assert Kd.cpu().numpy().tobytes() == ref.tobytes()


def test_add_diag_missing_diagonal(ctx, oracle):
    """A vertex without incident elements has no diagonal slot: adding a
    diagonal fails the next sync (and the error is cleared)."""
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import bsr_add_diag
    n = 300
    rp, ci, K, D = _system(oracle, n, 50, 1, 9, np.float64, with_diag=False)
    assert np.any(np.diff(rp.astype(np.int64)) == 0)
    d = ctx.device
    args = (ctx, n, 1, _t(rp, d), _t(ci, d), _t(K, d))
    bsr_add_diag(*args, diag=_t(D, d))
    with pytest.raises(SimitError):
        ctx.sync()
    bsr_add_diag(*args, diag=None, ident=0.0)  # no diagonal term: fine
    ctx.sync()


def test_add_diag_empty_and_bad_args(ctx, oracle):
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import bsr_add_diag
    d = ctx.device
    z = torch.zeros(1, dtype=torch.int32, device=d)
    e = torch.zeros(0, dtype=torch.float64, device=d)
    bsr_add_diag(ctx, 0, 3, z, z, e)
    ctx.sync()
    rp, ci, K, D = _system(oracle, 20, 40, 3, 2, np.float64)
    with pytest.raises(SimitError):  # both a diagonal array and ident
        bsr_add_diag(ctx, 20, 3, _t(rp, d), _t(ci, d), _t(K, d), diag=_t(D, d), ident=1.0)
    with pytest.raises(SimitError):  # block size out of range
        bsr_add_diag(ctx, 20, 4, _t(rp, d), _t(ci, d), _t(K, d))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_isprings_unfused_matches_fused(ctx, oracle, dtype):
    """isprings.sim unchanged: K from the springs map alone (zero mass and
    damping, so its diagonal term is 0), MD = (m + h*viscous)*I per point as
    Diagonal storage, then MDK = MD + K — equal to the fused assembly (the
    exact kernels, so h*viscous + m is not contracted)."""
    from simit_gb300.runtime import Mesh, assemble_springs, bsr_add_diag
    L = meshgen.springs_lattice(10, 10, 10, 0.1, 0.01, seed=4)
    n = L["n"]
    g = meshgen.rng(8)
    v = g.uniform(-0.1, 0.1, n * 3)
    m = g.uniform(0.5, 2.0, n)
    k = np.full(len(L["l0"]), 1e4)
    l0 = L["l0"] * g.uniform(0.9, 1.1, len(L["l0"]))
    fixed = np.zeros(n, np.uint8)
    grav = np.array([0, 0, -9.81])
    h, visc = 1e-3, 0.5
    mesh = Mesh(ctx, n, L["ep"], 2)
    fused, _ = assemble_springs(mesh, L["x"], v, m, fixed, k, l0, h, visc, grav, dtype=dtype)
    K, _ = assemble_springs(mesh, L["x"], v, np.zeros(n), fixed, k, l0, h, 0.0, grav,
                            dtype=dtype)
    np_dt = np.float64 if dtype == torch.float64 else np.float32
    md = (m.astype(np_dt) + np_dt(h) * np_dt(visc)).astype(np_dt)
    MD = (md[:, None, None] * np.eye(3, dtype=np_dt)[None]).reshape(-1)
    p = mesh.pattern
    MDK = bsr_add_diag(ctx, n, 3, p.rowptr, p.colidx, K,
                       diag=torch.from_numpy(MD).to(ctx.device))
    ctx.sync()
    assert torch.equal(MDK, fused)


@pytest.mark.parametrize("case", range(6))
def test_incidence_matrices_golden_gpu(ctx, oracle, case):
    """test/assembly-tests.cpp matrix_ve / matrix_ev (+ heterogeneous):
    pattern and values equal to the oracle's Link::ev / Link::ve and `loc`
    assembly, and A * field equal to the reference's asserted values."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import IncidenceMatrix
    from tests import scenarios
    kind, n, sel, npos, eb, vec, expected, name = scenarios.incidence_scenarios()[case]
    M = IncidenceMatrix(ctx, kind, n, sel.reshape(-1), npos)
    vals = M.assemble(eb, 1)
    y = M.spmv(1, vals, torch.tensor(vec, dtype=torch.float64, device=ctx.device))
    ctx.sync()
    rp, ci = oracle.incidence_pattern(kind, n, sel, npos)
    assert np.array_equal(M.rowptr.cpu().numpy().view(np.uint32), rp)
    assert np.array_equal(M.colidx[:M.nnzb].cpu().numpy().view(np.uint32), ci)
    assert np.array_equal(vals[:M.nnzb].cpu().numpy(),
                          oracle.assemble_incidence(kind, sel, npos, 1, eb, rp, ci))
    assert y.cpu().numpy().tolist() == [float(v) for v in expected], name
    assert kind in (_lib.INCIDENCE_EV, _lib.INCIDENCE_VE)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("bs", [1, 3])
def test_incidence_random_repeats(ctx, oracle, kind, bs):
    """Random elements over 300 vertices with repeated endpoints (a repeat's
    second slot stays zero), FP64 3x3 or scalar blocks: bit-exact with the
    oracle; the rectangular SpMV A x within 1e-14 of the oracle's."""
    from simit_gb300.runtime import IncidenceMatrix
    g = meshgen.rng(40 + kind + bs)
    n, nE, npos = 300, 700, 4
    sel = g.integers(0, n, size=(nE, npos))
    sel[::5, 2] = sel[::5, 0]  # repeats
    eb = g.uniform(-1, 1, size=(nE, npos, bs, bs))
    M = IncidenceMatrix(ctx, kind, n, sel.reshape(-1), npos)
    vals = M.assemble(eb, bs)
    rp, ci = oracle.incidence_pattern(kind, n, sel, npos)
    ref = oracle.assemble_incidence(kind, sel, npos, bs, eb, rp, ci)
    cols = n if kind == 0 else nE
    x = g.uniform(-1, 1, size=cols * bs)
    y = M.spmv(bs, vals, torch.tensor(x, device=ctx.device))
    ctx.sync()
    assert np.array_equal(vals[:M.nnzb * bs * bs].cpu().numpy(), ref)
    yr = oracle.spmv(len(rp) - 1, bs, rp, ci, ref, x)
    sc = oracle.spmv(len(rp) - 1, bs, rp, ci, np.abs(ref), np.abs(x))
    assert np.all(np.abs(y.cpu().numpy() - yr) <= 1e-14 * sc + 1e-300)


@pytest.mark.parametrize("case", range(2))
def test_rect_matrix_golden_gpu(ctx, oracle, case):
    """matrix_vv_heterogeneous: the rectangular pattern, its values and
    A * field on the GPU against the oracle and the reference's results."""
    from simit_gb300.runtime import RectMatrix
    from tests import scenarios
    nr, nc, sr, npr, sc, npc, eb, vec, expected, name = scenarios.rect_scenarios()[case]
    M = RectMatrix(ctx, nr, nc, sr.reshape(-1), npr, sc.reshape(-1), npc)
    vals = M.assemble(eb, 1)
    y = M.spmv(1, vals, torch.tensor(vec, dtype=torch.float64, device=ctx.device))
    ctx.sync()
    rp, ci = oracle.rect_pattern(nr, sr, npr, sc, npc)
    assert np.array_equal(M.rowptr.cpu().numpy().view(np.uint32), rp)
    assert np.array_equal(M.colidx[:M.nnzb].cpu().numpy().view(np.uint32), ci)
    assert np.array_equal(vals[:M.nnzb].cpu().numpy(),
                          oracle.assemble_rect(sr, npr, sc, npc, 1, eb, rp, ci))
    assert y.cpu().numpy().tolist() == [float(v) for v in expected], name


def test_rect_matrix_random(ctx, oracle):
    """Random two-set edge set (3 row-set and 2 column-set endpoints, with
    repeats), 3x3 FP64 blocks: pattern and values bit-exact with the oracle."""
    from simit_gb300.runtime import RectMatrix
    g = meshgen.rng(77)
    nr, nc, nE = 200, 150, 600
    sr = g.integers(0, nr, size=(nE, 3))
    sc = g.integers(0, nc, size=(nE, 2))
    sr[::7, 1] = sr[::7, 0]
    eb = g.uniform(-1, 1, size=(nE, 3, 2, 3, 3))
    M = RectMatrix(ctx, nr, nc, sr.reshape(-1), 3, sc.reshape(-1), 2)
    vals = M.assemble(eb, 3)
    ctx.sync()
    rp, ci = oracle.rect_pattern(nr, sr, 3, sc, 2)
    assert np.array_equal(M.colidx[:M.nnzb].cpu().numpy().view(np.uint32), ci)
    ref = oracle.assemble_rect(sr, 3, sc, 2, 3, eb, rp, ci)
    assert np.array_equal(vals[:M.nnzb * 9].cpu().numpy(), ref)


def test_cg_sim_unfused_matches_golden(ctx):
    """test/input/program/cg.sim as written: K from the scalar springs map
    alone, then A = I - 0.01 K as the matrix expression, CG from 0 — the
    values of test/program-cg-test.cpp, and bit-equal to the fused map."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import Mesh, Solver, assemble_scalar_springs, solve_opts
    from tests import scenarios
    s = scenarios.cg_chain()
    mesh = Mesh(ctx, s["n"], s["ep"], 2)
    p = mesh.pattern
    fused = assemble_scalar_springs(mesh, s["a"], s["diag"], s["scale"])
    K = assemble_scalar_springs(mesh, s["a"], 0.0, 1.0)
    from simit_gb300.runtime import bsr_add_diag
    A = bsr_add_diag(ctx, s["n"], 1, p.rowptr, p.colidx, K, ident=s["diag"], scale=s["scale"])
    ctx.sync()
    assert torch.equal(A, fused)
    b = torch.tensor(s["b"], device=ctx.device)
    opts = solve_opts(precision=_lib.SOLVE_F64, precond=_lib.PRECOND_NONE, stop=_lib.STOP_NORMR,
                      tol=s["tol"], maxiters=s["maxiters"], verify=0)
    S = Solver(ctx, mesh.n, 1, p.rowptr, p.colidx, A, mesh.nnzb, opts)
    c = torch.zeros_like(b)
    S.solve(b, c)
    S.close()
    for g in scenarios.golden("cg"):
        got = scenarios.golden_lookup(g, {"c": c.cpu().numpy()})
        assert abs(got - g["expected"]) <= 1e-13, (g, got)
