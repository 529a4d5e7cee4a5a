"""GPU parity: pattern, slot map and blocked SpMV against the oracle."""
import json
import os

import numpy as np
import pytest
import torch

from simit_gb300 import meshgen
from tests import scenarios

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


def _check_pattern(ctx, oracle, n, ep, card):
    from simit_gb300.runtime import Pattern
    p = Pattern(ctx, n, ep, card)
    rp, ci = p.host()
    orp, oci = oracle.pattern(n, ep, card)
    assert np.array_equal(rp, orp)
    assert np.array_equal(ci, oci)
    sl = p.slots[:len(ep) * card].cpu().numpy().view(np.uint32)
    assert np.array_equal(sl, oracle.slots(ep, card, orp, oci))
    # incidence rows sorted ascending and complete
    vp = p.ve_ptr.cpu().numpy().view(np.uint32)
    vi = p.ve_idx[:len(ep)].cpu().numpy().view(np.uint32)
    for v in range(min(n, 64)):
        lst = vi[vp[v]:vp[v + 1]]
        assert np.all(np.diff(lst.astype(np.int64)) > 0)
        assert np.all(np.asarray(ep)[lst] == v)
    return p


def test_pattern_golden_fixtures(ctx, oracle):
    with open(os.path.join(scenarios.GOLDEN, "pattern_golden.json")) as f:
        cases = json.load(f)
    from simit_gb300.runtime import Pattern
    for name, c in cases.items():
        ep = np.array(c["endpoints"], np.int32)
        p = Pattern(ctx, c["n"], ep, c["card"])
        rp, ci = p.host()
        assert rp.tolist() == c["rowptr"], name
        assert ci.tolist() == c["colidx"], name
        assert p.slots[:len(c["slots"])].cpu().numpy().view(np.uint32).tolist() == c["slots"]


@pytest.mark.parametrize("card,n,nE,seed", [(2, 50, 120, 1), (3, 64, 90, 2), (4, 80, 150, 3),
                                            (4, 30, 400, 4), (1, 10, 7, 5), (2, 1000, 1, 6)])
def test_pattern_random(ctx, oracle, card, n, nE, seed):
    ep = meshgen.rng(seed).integers(0, n, size=nE * card).astype(np.int32)
    _check_pattern(ctx, oracle, n, ep, card)


def test_pattern_high_degree(ctx, oracle):
    """A hub vertex in every element (long incidence list, shared-memory sort)."""
    n, nE = 300, 2000
    r = meshgen.rng(11).integers(1, n, size=(nE, 2)).astype(np.int32)
    ep = np.concatenate([np.zeros((nE, 1), np.int32), r], 1).reshape(-1)
    _check_pattern(ctx, oracle, n, ep, 3)


def test_pattern_tet_lattice(ctx, oracle):
    m = meshgen.tet_grid(12, 9, 7)
    _check_pattern(ctx, oracle, m["n"], m["tets"], 4)


def test_pattern_springs_box(ctx, oracle):
    ep, n = meshgen.box_springs(10, 10, 10)
    p = _check_pattern(ctx, oracle, n, ep, 2)
    assert p.nnzb == 6400


def test_pattern_empty_edge_set(ctx):
    from simit_gb300.runtime import Pattern
    p = Pattern(ctx, 5, np.zeros(0, np.int32), 2)
    assert p.nnzb == 0
    assert p.rowptr.cpu().tolist() == [0] * 6


def test_pattern_bad_endpoint_is_an_error(ctx):
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import Pattern
    with pytest.raises(SimitError):
        Pattern(ctx, 4, np.array([0, 1, 2, 9], np.int32), 2)
    # the context stays usable
    Pattern(ctx, 4, np.array([0, 1, 2, 3], np.int32), 2)


def _random_bsr(oracle, n, nE, bs, seed, dt):
    ep = meshgen.rng(seed).integers(0, n, size=nE * 2).astype(np.int32)
    rp, ci = oracle.pattern(n, ep, 2)
    g = meshgen.rng(seed + 100)
    vals = g.uniform(-1, 1, size=len(ci) * bs * bs).astype(dt)
    x = g.uniform(-1, 1, size=n * bs).astype(dt)
    return rp, ci, vals, x


@pytest.mark.parametrize("bs", [1, 2, 3, 5])
@pytest.mark.parametrize("g", [0, 1, 2, 4, 8, 16, 32])
def test_spmv_f64(ctx, oracle, bs, g):
    from simit_gb300.runtime import bspmv
    if bs == 5 and g not in (0,):
        pytest.skip("generic bs uses one thread per row")
    n = 700
    rp, ci, vals, x = _random_bsr(oracle, n, 3000, bs, 3 + bs, np.float64)
    ref = oracle.spmv(n, bs, rp, ci, vals, x)
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    y = bspmv(ctx, n, bs, t(rp), t(ci), t(vals), t(x), g=g)
    ctx.sync()
    scale = oracle.spmv(n, bs, rp, ci, np.abs(vals), np.abs(x))
    err = np.abs(y.cpu().numpy() - ref)
    assert np.all(err <= 1e-14 * scale + 1e-300)


@pytest.mark.parametrize("bs", [1, 3])
def test_spmv_f32(ctx, oracle, bs):
    from simit_gb300.runtime import bspmv
    n = 2000
    rp, ci, vals, x = _random_bsr(oracle, n, 9000, bs, 40 + bs, np.float32)
    ref = oracle.spmv(n, bs, rp, ci, vals.astype(np.float64), x.astype(np.float64))
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    y = bspmv(ctx, n, bs, t(rp), t(ci), t(vals), t(x))
    ctx.sync()
    scale = oracle.spmv(n, bs, rp, ci, np.abs(vals).astype(np.float64),
                        np.abs(x).astype(np.float64))
    assert np.all(np.abs(y.cpu().numpy() - ref) <= 2e-6 * scale + 1e-30)


N_TMA_VARIANTS = 15


@pytest.mark.parametrize("bs", [3, 1])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("variant", range(N_TMA_VARIANTS))
def test_spmv_tma_variants(ctx, oracle, variant, dt, bs):
    """Every TMA-staged SpMV variant (CTA tiles and per-warp pipelines; for
    scalar CSR the per-warp ones, the others run the streaming kernel), on
    a random graph plus a hub vertex whose ~60-block row runs past the
    predicated part of each lane's loop; unaligned tile heads and tails
    throughout (36- and 72-byte blocks)."""
    from simit_gb300.runtime import bspmv
    n = 3001
    g0 = meshgen.rng(90 + variant)
    ep = np.concatenate([g0.integers(0, n, size=12000 * 2),
                         np.stack([np.full(60, 7), g0.integers(0, n, 60)], 1).reshape(-1)])
    rp, ci = oracle.pattern(n, ep.astype(np.int32), 2)
    g = meshgen.rng(91 + variant)
    vals = g.uniform(-1, 1, size=len(ci) * bs * bs).astype(dt)
    x = g.uniform(-1, 1, size=n * bs).astype(dt)
    ref = oracle.spmv(n, bs, rp, ci, vals.astype(np.float64), x.astype(np.float64))
    scale = oracle.spmv(n, bs, rp, ci, np.abs(vals).astype(np.float64),
                        np.abs(x).astype(np.float64))
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    y = bspmv(ctx, n, bs, t(rp), t(ci), t(vals), t(x), g=-1 - variant)
    ctx.sync()
    tol = 2e-6 if dt == np.float32 else 1e-14
    assert np.all(np.abs(y.cpu().numpy() - ref) <= tol * scale + 1e-300)


def test_spmv_tma_stale_statistics(ctx, oracle):
    """Pattern statistics are cached per (rowptr address, n); a new pattern
    written at the same address with longer rows must still multiply
    correctly (oversize tiles are read from global memory, never staged
    past the buffers)."""
    from simit_gb300.runtime import bspmv
    n = 4000
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    ep = meshgen.rng(5).integers(0, n, size=8000 * 2).astype(np.int32)
    rp1, ci1 = oracle.pattern(n, ep, 2)
    ep2 = np.concatenate([ep, np.stack([np.full(80, 3), np.arange(100, 180)], 1).reshape(-1)
                          .astype(np.int32)])
    rp2, ci2 = oracle.pattern(n, ep2, 2)
    assert len(ci2) > len(ci1)
    with ctx.stream():
        rp_d = torch.zeros(n + 1, dtype=torch.int32, device=d)
        ci_d = torch.zeros(len(ci2), dtype=torch.int32, device=d)
    g = meshgen.rng(6)
    for rp, ci in ((rp1, ci1), (rp2, ci2)):
        rp_d.copy_(t(rp))
        ci_d[:len(ci)].copy_(t(ci))
        vals = g.uniform(-1, 1, size=len(ci) * 9).astype(np.float32)
        x = g.uniform(-1, 1, size=n * 3).astype(np.float32)
        ref = oracle.spmv(n, 3, rp, ci, vals.astype(np.float64), x.astype(np.float64))
        scale = oracle.spmv(n, 3, rp, ci, np.abs(vals).astype(np.float64),
                            np.abs(x).astype(np.float64))
        for variant in range(N_TMA_VARIANTS):
            y = bspmv(ctx, n, 3, rp_d, ci_d, t(vals), t(x), g=-1 - variant)
            ctx.sync()
            assert np.all(np.abs(y.cpu().numpy() - ref) <= 2e-6 * scale + 1e-30), variant


def test_spmv_tma_variant_out_of_range(ctx, oracle):
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import bspmv
    n = 50
    rp, ci, vals, x = _random_bsr(oracle, n, 100, 3, 1, np.float32)
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    with pytest.raises(SimitError):
        bspmv(ctx, n, 3, t(rp), t(ci), t(vals), t(x), g=-1 - N_TMA_VARIANTS)


def test_spmv_f32_matrix_f64_vector(ctx, oracle):
    """FP32 values, FP64 x/y and accumulation (the refinement residual path)."""
    from simit_gb300.runtime import bspmv
    n = 900
    rp, ci, vals, x = _random_bsr(oracle, n, 4000, 3, 77, np.float32)
    x = x.astype(np.float64) + 1e-9
    ref = oracle.spmv(n, 3, rp, ci, vals.astype(np.float64), x)
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    y = bspmv(ctx, n, 3, t(rp), t(ci), t(vals), t(x))
    ctx.sync()
    scale = oracle.spmv(n, 3, rp, ci, np.abs(vals).astype(np.float64), np.abs(x))
    assert np.all(np.abs(y.cpu().numpy() - ref) <= 1e-14 * scale)


def test_spmv_deterministic(ctx, oracle):
    from simit_gb300.runtime import bspmv
    n = 5000
    rp, ci, vals, x = _random_bsr(oracle, n, 30000, 3, 5, np.float32)
    d = ctx.device
    t = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(d)  # noqa
    a = t(rp), t(ci), t(vals), t(x)
    y1 = bspmv(ctx, n, 3, *a).clone()
    y2 = bspmv(ctx, n, 3, *a)
    ctx.sync()
    assert torch.equal(y1, y2)


def test_dot(ctx):
    from simit_gb300.runtime import dot
    g = meshgen.rng(9)
    a = g.uniform(-1, 1, 100003)
    b = g.uniform(-1, 1, 100003)
    d = ctx.device
    got = dot(ctx, torch.from_numpy(a).to(d), torch.from_numpy(b).to(d))
    assert abs(got - float(np.dot(a, b))) <= 1e-12 * float(np.dot(np.abs(a), np.abs(b)))


def test_fp64_fma_rate_is_plausible(ctx):
    """sg_fp64_fma_rate, the FP64 roofline the bench reports the FP64 SpMV
    against: a positive rate well below the FP32 one (GB300's FP64 is about
    1.2 TFLOP/s)."""
    from simit_gb300.runtime import fp64_fma_rate
    r = fp64_fma_rate(ctx)
    assert 0.1 < r < 20.0, r
