"""The apps' TetGen meshes through the GPU path: bunny.1 (3,607 vertices,
12,687 tets, 19,233 .edge springs) and dragon40k (11,083 vertices, 40,715
tets).  Pattern and slot map against the reference PathIndexBuilder's
digests, FP64 assembly against the oracle (bit for bit; the neo-Hookean
model within 1e-12, for log), solves to the FP64
tolerance, the springs app's set-up over the bunny's edges, and the
run-time compiled linear-tet element on the dragon."""
import numpy as np
import pytest
import torch

from simit_gb300 import _lib, jit_elements, meshgen
from tests import scenarios

pytestmark = pytest.mark.gpu

CASES = [("bunny_tets", "bunny_x", "bunny_tets", 4), ("bunny_edges", "bunny_x", "bunny_edges", 2),
         ("dragon_tets", "dragon_x", "dragon_tets", 4)]


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


@pytest.fixture(scope="module")
def meshes():
    return scenarios.tetmeshes()


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name,xkey,epkey,card", CASES)
def test_pattern_and_slots_match_reference_builder(ctx, meshes, name, xkey, epkey, card):
    from simit_gb300.runtime import Pattern
    m, dig = meshes
    g = dig[name]
    n = len(m[xkey]) // 3
    p = Pattern(ctx, n, m[epkey], card, with_slots=True)
    rp, ci = p.host()
    ctx.sync()
    assert p.nnzb == g["nnzb"]
    assert scenarios.sha(rp) == g["rowptr_sha256"]
    assert scenarios.sha(ci) == g["colidx_sha256"]
    assert scenarios.sha(_np(p.slots)[:g["nE"] * card * card]) == g["slots_sha256"]


def _tet_problem(m, key, seed):
    x0 = m[key + "_x"]
    tets = m[key + "_tets"]
    n, nT = len(x0) // 3, len(tets) // 4
    g = meshgen.rng(seed)
    E = 10 ** g.uniform(3, 6, nT)
    nu = g.uniform(0.35, 0.45, nT)
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    y = x0.reshape(-1, 3)[:, 1]
    c = (y < y.min() + 0.05 * (y.max() - y.min())).astype(np.int32)
    x = x0 + g.uniform(-1e-5, 1e-5, x0.size) * (y.max() - y.min())
    return {"n": n, "tets": tets, "X0": x0, "x": x, "c": c, "mu": mu, "lam": lam}


@pytest.mark.parametrize("key", ["bunny", "dragon"])
@pytest.mark.parametrize("model", [_lib.MODEL_LINEAR, _lib.MODEL_NEOHOOKEAN])
def test_fp64_assembly_matches_oracle(ctx, oracle, meshes, key, model):
    from simit_gb300.runtime import (Mesh, assemble_tet_force, assemble_tet_stiffness,
                                     tet_precompute)
    s = _tet_problem(meshes[0], key, 3)
    h, rho, grav = 1e-2, 1e3, np.array([0.0, -9.81, 0.0])
    v = meshgen.rng(4).uniform(-0.1, 0.1, s["n"] * 3)
    mesh = Mesh(ctx, s["n"], s["tets"], 4)
    rp, ci = mesh.pattern.host()
    B, W, mv = tet_precompute(mesh, s["X0"], rho)
    oB, oW, om = oracle.tet_precompute(s["X0"], s["tets"], rho)
    A = assemble_tet_stiffness(mesh, model, s["x"], s["c"], B, W, s["mu"], s["lam"], h, rho)
    f = assemble_tet_force(mesh, model, s["x"], v, s["c"], B, W, s["mu"], s["lam"], h, rho, grav)
    oA = oracle.tet_stiffness(model, s["x"], s["c"], s["tets"], oB, oW, s["mu"], s["lam"], h, rho,
                              rp, ci)
    of = oracle.tet_force(model, s["x"], v, s["c"], s["tets"], oB, oW, s["mu"], s["lam"], h, rho,
                          grav)
    ctx.sync()
    assert np.array_equal(_np(B), oB) and np.array_equal(_np(W), oW)
    assert np.array_equal(_np(mv), om)
    if model == _lib.MODEL_LINEAR:
        assert np.array_equal(_np(A), oA)
        assert np.array_equal(_np(f), of)
    else:
        # log(det F): the device log and the host libm may differ by an ulp
        assert np.abs(_np(A) - oA).max() <= 1e-12 * np.abs(oA).max()
        assert np.abs(_np(f) - of).max() <= 1e-12 * np.abs(of).max()


@pytest.mark.parametrize("precision,dtype", [(_lib.SOLVE_F64, torch.float64),
                                             (_lib.SOLVE_MIXED, torch.float32)])
def test_dragon_solve_reaches_fp64_tolerance(ctx, oracle, meshes, precision, dtype):
    """The dragon's linear-elastic system (one implicit step, h = 1) solved by
    block-Jacobi PCG in FP64 and in mixed precision (FP32 matrix), to a 1e-8
    FP64 residual recomputed by the oracle."""
    from simit_gb300.runtime import (Mesh, Solver, assemble_tet_force, assemble_tet_stiffness,
                                     solve_opts, tet_precompute)
    s = _tet_problem(meshes[0], "dragon", 5)
    mesh = Mesh(ctx, s["n"], s["tets"], 4)
    B, W, _ = tet_precompute(mesh, s["X0"], 1e3, dtype=dtype)
    A = assemble_tet_stiffness(mesh, _lib.MODEL_LINEAR, s["x"], s["c"], B, W, s["mu"], s["lam"],
                               1.0, 1e3, dtype=dtype, exact=False)
    f = assemble_tet_force(mesh, _lib.MODEL_LINEAR, s["x"], np.zeros(s["n"] * 3), s["c"], B, W,
                           s["mu"], s["lam"], 1.0, 1e3, np.array([0, -9.81, 0]), dtype=dtype)
    with ctx.stream():
        b = f.to(torch.float64)
        x = torch.zeros_like(b)
    S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
               solve_opts(precision=precision, precond=_lib.PRECOND_BLOCK_JACOBI, tol=1e-8,
                          maxiters=100000))
    res = S.solve(b, x)
    assert res.status == 1, _lib.STATUS.get(res.status)
    rp, ci = mesh.pattern.host()
    assert oracle.relres(mesh.n, 3, rp, ci, _np(A), _np(b), _np(x)) <= 1.001e-8
    S.close()


def test_bunny_springs_app_step(ctx, oracle, meshes):
    """apps/springs/springs.cpp's set-up over bunny.1.edge: the first step's
    system bit for bit against the oracle and the step's CG result."""
    from simit_gb300.runtime import Mesh, Solver, assemble_springs, solve_opts
    m = meshes[0]
    s = scenarios.springs_from_arrays(m["bunny_x"], m["bunny_edges"])
    mesh = Mesh(ctx, s["n"], s["ep"], 2)
    rp, ci = mesh.pattern.host()
    vals, f = assemble_springs(mesh, s["x"], s["v"], s["m"], s["fixed"], s["k"], s["l0"], s["h"],
                               s["viscous"], s["grav"], form=s["form"])
    oA, of = oracle.springs_assemble(s["form"], s["x"], s["v"], s["m"], s["fixed"], s["ep"],
                                     s["k"], s["l0"], s["h"], s["viscous"], s["grav"], rp, ci)
    ctx.sync()
    assert np.array_equal(_np(vals), oA) and np.array_equal(_np(f), of)
    S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, vals, mesh.nnzb,
               solve_opts(precond=_lib.PRECOND_BLOCK_JACOBI, tol=1e-10, maxiters=20000))
    with ctx.stream():
        x = torch.zeros_like(f)
    res = S.solve(f, x)
    assert res.status == 1, _lib.STATUS.get(res.status)
    assert oracle.relres(mesh.n, 3, rp, ci, oA, of, _np(x)) <= 1.001e-10
    S.close()


def test_dragon_jit_linear_tet(ctx, meshes):
    from simit_gb300.runtime import JitAssembly, Mesh, assemble_tet_stiffness, tet_precompute
    s = _tet_problem(meshes[0], "dragon", 7)
    mesh = Mesh(ctx, s["n"], s["tets"], 4)
    B, W, _ = tet_precompute(mesh, s["X0"], 1e3, dtype=torch.float32)
    A = assemble_tet_stiffness(mesh, _lib.MODEL_LINEAR, s["x"], s["c"], B, W, s["mu"], s["lam"],
                               1e-2, 1e3, dtype=torch.float32, exact=False)
    jit = JitAssembly(ctx, jit_elements.linear_tet(1e-2, 1e3), 4, 3, dtype=torch.float32,
                      exact=False)
    got = jit.assemble(mesh, [B, W, s["mu"], s["lam"], s["c"]])
    ctx.sync()
    assert torch.equal(got[:mesh.nnzb * 9], A[:mesh.nnzb * 9])
    jit.close()
