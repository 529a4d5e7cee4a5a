"""Symmetric storage (sg_symbsr_*, SG_STORAGE_SYMMETRIC): the upper-half SpMV
against the oracle's full blocked SpMV, the checks on the pattern, the
exact symmetry of the FP32 linear-tet assembly it relies on, and solves."""
import numpy as np
import pytest
import torch

from simit_gb300 import _lib, meshgen, problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


def _t(a, d):
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)


def _sym_system(oracle, n, nE, seed):
    """A random symmetric pattern with all diagonal blocks and symmetric FP32
    values: block (c, r) is the transpose of block (r, c)."""
    g = meshgen.rng(seed)
    ep = np.concatenate([g.integers(0, n, size=nE * 2),
                         np.repeat(np.arange(n), 2)]).astype(np.int32)
    rp, ci = oracle.pattern(n, ep, 2)
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    vals = g.uniform(-1, 1, size=(len(ci), 3, 3)).astype(np.float32)
    key = rows.astype(np.int64) * n + ci
    mirror = np.searchsorted(key, ci.astype(np.int64) * n + rows)
    lower = ci < rows
    vals[lower] = vals[mirror[lower]].transpose(0, 2, 1)
    diag = ci == rows
    vals[diag] = (vals[diag] + vals[diag].transpose(0, 2, 1)) / 2
    return rp, ci, vals.reshape(-1)


@pytest.mark.parametrize("n,nE,seed", [(1, 0, 1), (7, 10, 2), (900, 4000, 3), (5000, 60000, 4)])
def test_symmetric_spmv_matches_full(ctx, oracle, n, nE, seed):
    from simit_gb300.runtime import SymBsr, bspmv
    rp, ci, vals = _sym_system(oracle, n, nE, seed)
    d = ctx.device
    x = meshgen.rng(seed + 50).uniform(-1, 1, size=n * 3).astype(np.float32)
    ref = oracle.spmv(n, 3, rp, ci, vals.astype(np.float64), x.astype(np.float64))
    scale = oracle.spmv(n, 3, rp, ci, np.abs(vals).astype(np.float64),
                        np.abs(x).astype(np.float64))
    sb = SymBsr(ctx, n, _t(rp, d), _t(ci, d), len(ci))
    sb.fill(_t(vals, d))
    y = sb.spmv(_t(x, d))
    ctx.sync()
    got = y.cpu().numpy().astype(np.float64)
    assert np.all(np.abs(got - ref) <= 2e-6 * scale + 1e-30)
    # deterministic, and equal to the full-storage kernel to FP32 rounding
    y2 = sb.spmv(_t(x, d))
    yf = bspmv(ctx, n, 3, _t(rp, d), _t(ci, d), _t(vals, d), _t(x, d))
    ctx.sync()
    assert torch.equal(y, y2)
    assert np.all(np.abs(yf.cpu().numpy() - got) <= 4e-6 * scale + 1e-30)
    sb.close()


def test_symmetric_storage_rejects_bad_patterns(ctx, oracle):
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import SymBsr
    d = ctx.device
    # row 1 has no diagonal block
    rp = np.array([0, 2, 3], np.uint32)
    ci = np.array([0, 1, 0], np.uint32)
    with pytest.raises(SimitError):
        SymBsr(ctx, 2, _t(rp, d), _t(ci, d), 3)
    # (0, 1) without (1, 0)
    rp = np.array([0, 2, 3], np.uint32)
    ci = np.array([0, 1, 1], np.uint32)
    with pytest.raises(SimitError):
        SymBsr(ctx, 2, _t(rp, d), _t(ci, d), 3)
    # (1, 0) without (0, 1)
    rp = np.array([0, 1, 3], np.uint32)
    ci = np.array([0, 0, 1], np.uint32)
    with pytest.raises(SimitError):
        SymBsr(ctx, 2, _t(rp, d), _t(ci, d), 3)
    ctx.sync()  # the failed checks left no pending device error


def test_fp32_linear_tet_assembly_is_exactly_symmetric(ctx):
    """The closed-form linear-tet stiffness (FP32 and FP64, contracted
    kernels) assembles block (c, r) as the bitwise transpose of (r, c)."""
    h = problems.hetero_mesh(10)
    for dt in (torch.float32, torch.float64):
        p = problems.HeteroElasticity(ctx, h, dtype=dt)
        ctx.sync()
        rp, ci = p.mesh.pattern.host()
        n = p.mesh.n
        A = p.A.cpu().numpy().reshape(-1, 3, 3)
        rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
        key = rows.astype(np.int64) * n + ci
        mirror = np.searchsorted(key, ci.astype(np.int64) * n + rows)
        assert np.array_equal(A, A[mirror].transpose(0, 2, 1)), dt


@pytest.mark.parametrize("size", [12, 20])
def test_solver_on_symmetric_storage(ctx, oracle, size):
    """Mixed block-Jacobi PCG iterating on symmetric storage reaches the
    1e-8 FP64 true residual of the full matrix in about as many iterations
    as on full storage, with a solution within the FP32 noise of it."""
    h = problems.reorder_hetero(problems.hetero_mesh(size))
    out = {}
    for name, storage in (("full", _lib.STORAGE_FULL), ("sym", _lib.STORAGE_SYMMETRIC)):
        p = problems.HeteroElasticity(ctx, h, dtype=torch.float32, storage=storage)
        assert p.opts.storage == storage
        res = p.step()
        ctx.sync()
        out[name] = (res, p.u.cpu().numpy().copy())
    (rf, uf), (rs, us) = out["full"], out["sym"]
    for r in (rf, rs):
        assert r.status == 1, _lib.STATUS.get(r.status)  # SG_STATUS_CONVERGED
        assert (r.true_normr2 / r.bnorm2) ** 0.5 <= 1e-8
    assert abs(rs.iters - rf.iters) <= 0.1 * rf.iters + 5
    assert np.linalg.norm(us - uf) <= 1e-5 * np.linalg.norm(uf)


def test_symmetric_storage_needs_mixed_bs3(ctx):
    from simit_gb300._lib import SimitError
    h = problems.hetero_mesh(4)
    with pytest.raises(SimitError):
        problems.HeteroElasticity(ctx, h, dtype=torch.float64, storage=_lib.STORAGE_SYMMETRIC)


@pytest.mark.parametrize("n,nE,seed", [(5, 8, 1), (2000, 9000, 2)])
def test_residual_modes_against_oracle(ctx, oracle, n, nE, seed):
    """sg_residual: FP64 accumulation within 1e-14 and the compensated FP32
    mode within 1e-12 of sum |A||x| + |b| (per entry) of the oracle's FP64
    residual of the FP32 matrix (plain FP32 accumulation: ~1e-7); both
    return ||r||^2 consistently."""
    from simit_gb300.runtime import residual
    rp, ci, vals = _sym_system(oracle, n, nE, seed)
    g = meshgen.rng(seed + 7)
    x = g.uniform(-1, 1, size=n * 3) * 10.0 ** g.uniform(-3, 3, size=n * 3)
    b = g.uniform(-1, 1, size=n * 3)
    v64 = vals.astype(np.float64)
    ref = b - oracle.spmv(n, 3, rp, ci, v64, x)
    scale = oracle.spmv(n, 3, rp, ci, np.abs(v64), np.abs(x)) + np.abs(b)
    d = ctx.device
    args = (ctx, n, 3, _t(rp, d), _t(ci, d), _t(vals, d), len(ci), _t(x, d), _t(b, d))
    for mode, tol in ((_lib.RESIDUAL_FP64, 1e-14), (_lib.RESIDUAL_COMPENSATED, 1e-12)):
        r, rr = residual(*args, mode=mode)
        got = r.cpu().numpy()
        assert np.all(np.abs(got - ref) <= tol * scale), mode
        assert abs(rr - float(got @ got)) <= 1e-12 * rr
    with pytest.raises(_lib.SimitError):  # compensated mode needs FP32 values
        residual(ctx, n, 3, _t(rp, d), _t(ci, d), _t(v64, d), len(ci), _t(x, d), _t(b, d),
                 mode=_lib.RESIDUAL_COMPENSATED)


def test_solver_pdl_same_result(ctx):
    """Programmatic dependent launch inside the iteration graph (opt-in)
    changes no arithmetic: the same iterations and the same solution bits."""
    h = problems.reorder_hetero(problems.hetero_mesh(12))
    out = []
    for pdl in (0, 1):
        p = problems.HeteroElasticity(ctx, h, dtype=torch.float32, pdl=pdl)
        assert p.opts.pdl == pdl
        res = p.step()
        ctx.sync()
        out.append((res.iters, res.true_normr2, p.u.cpu().numpy().copy()))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
