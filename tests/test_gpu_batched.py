"""GPU checks of the batched PCG (many uneven cloth sheets in one launch)."""
import numpy as np
import pytest
import torch

from simit_gb300 import _lib, problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


@pytest.fixture(scope="module")
def batch(ctx):
    host = problems.cloth_batch(nsheets=12, lo=8, hi=40, seed=3)
    return problems.ClothBatch(ctx, host)


def test_every_sheet_converges_on_the_true_residual(ctx, batch, oracle):
    batch.step()
    ctx.sync()
    st = batch.status.cpu().numpy()
    assert np.all(st == 1), st
    assert np.all(batch.relres.cpu().numpy() <= 1e-6)
    # independent check: each sheet's FP64 residual with the oracle SpMV
    rp, ci = batch.mesh.pattern.host()
    A = batch.A.cpu().numpy().astype(np.float64)
    f = batch.f.cpu().numpy().astype(np.float64)
    v = batch.vout.cpu().numpy().astype(np.float64)
    r = f - oracle.spmv(batch.mesh.n, 3, rp, ci, A, v)
    sp = batch.host["sys_ptr"]
    for s in range(batch.nsys):
        a, b = sp[s] * 3, sp[s + 1] * 3
        assert np.linalg.norm(r[a:b]) <= 1.001e-6 * np.linalg.norm(f[a:b]), s


def test_matches_one_at_a_time_solves(ctx, batch):
    """Each sheet solved alone by the general mixed-precision solver reaches
    the same solution (both to a 1e-6 relative residual)."""
    from simit_gb300.runtime import Mesh, Solver, assemble_springs, solve_opts
    batch.step()
    ctx.sync()
    vb = batch.vout.cpu().numpy()
    h = batch.host
    sp = h["sys_ptr"]
    ep = h["ep"].reshape(-1, 2)
    for s in range(batch.nsys):
        v0, v1 = sp[s], sp[s + 1]
        sel = (ep[:, 0] >= v0) & (ep[:, 0] < v1)
        mesh = Mesh(ctx, int(v1 - v0), (ep[sel] - v0).reshape(-1), 2)
        c = problems.CLOTH
        A, f = assemble_springs(mesh, h["x"][v0 * 3:v1 * 3], np.zeros((v1 - v0) * 3),
                                np.full(v1 - v0, c["mass"]), h["fixed"][v0:v1], h["k"][sel],
                                h["l0"][sel], c["dt"], c["viscous"], c["grav"], form=0,
                                dtype=torch.float32, exact=False)
        S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
                   solve_opts(precision=_lib.SOLVE_MIXED, precond=_lib.PRECOND_BLOCK_JACOBI,
                              tol=1e-6, maxiters=10000))
        x = torch.zeros(mesh.n * 3, dtype=torch.float64, device=ctx.device)
        res = S.solve(f.double(), x)
        S.close()
        assert res.status == 1
        xs = x.cpu().numpy()
        assert np.linalg.norm(xs - vb[v0 * 3:v1 * 3]) <= 1e-4 * np.linalg.norm(xs)


def test_graph_replay_is_deterministic(ctx, batch):
    batch.capture()
    batch.replay()
    ctx.sync()
    v1 = batch.vout.clone()
    batch.replay()
    ctx.sync()
    assert torch.equal(v1, batch.vout)
    assert 0 <= batch.config < _lib.load().sg_batched_configs()
