"""sg_dot_noalloc: the dot product for callers that may not allocate device
memory while they run (their host owns a fixed GPU memory pool, or their
loop must not call cudaMalloc/cudaFree, which can synchronise the device).

Collected last on purpose (file name), so that a failing run stopped at the
first failure has already run every other test.  It passes alone in a fresh
process (the session fixture creates the context) and after the others.
"""
import ctypes

import numpy as np
import pytest
import torch

from simit_gb300 import _lib, meshgen

pytestmark = pytest.mark.gpu


def _dot_ctx(ctx, a, b):
    out = ctypes.c_double()
    _lib.call("sg_dot", ctx.h, a.numel(), 1 if a.dtype == torch.float64 else 0,
              ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()), ctypes.byref(out))
    return out.value


def _dot_noalloc(ctx, a, b, out):
    _lib.call("sg_dot_noalloc", ctypes.c_void_p(_lib.load().sg_ctx_stream(ctx.h)), a.numel(),
              1 if a.dtype == torch.float64 else 0, ctypes.c_void_p(a.data_ptr()),
              ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(out.data_ptr()))
    ctx.sync()
    return float(out.item())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_no_alloc_dot_matches_sg_dot_twice(gpu_ctx, dtype):
    ctx = gpu_ctx
    d = ctx.device
    out = torch.zeros(1, dtype=torch.float64, device=d)
    # two calls in a row with different sizes: the second must not see the
    # first one's partial sums left in the shared static array; each result
    # against the context's sg_dot and an FP64 sum on the host
    for seed, n in ((1, 3_000_001), (2, 12_345)):
        g = meshgen.rng(seed)
        a = torch.tensor(g.uniform(-1, 1, n), dtype=dtype, device=d)
        b = torch.tensor(g.uniform(-1, 1, n), dtype=dtype, device=d)
        ref = _dot_ctx(ctx, a, b)
        got = _dot_noalloc(ctx, a, b, out)
        ah, bh = a.double().cpu().numpy(), b.double().cpu().numpy()
        host = float(np.dot(ah, bh))
        scale = float(np.abs(ah) @ np.abs(bh))
        assert abs(got - ref) <= 1e-12 * scale, (n, got, ref)
        assert abs(got - host) <= 1e-12 * scale, (n, got, host)


def test_no_alloc_dot_allocates_nothing(gpu_ctx):
    """After the first call on the device, further calls leave the device's
    free memory unchanged."""
    ctx = gpu_ctx
    d = ctx.device
    out = torch.zeros(1, dtype=torch.float64, device=d)
    a = torch.rand(1_000_003, dtype=torch.float32, device=d)
    b = torch.rand(1_000_003, dtype=torch.float32, device=d)
    _dot_noalloc(ctx, a, b, out)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(d)
    for _ in range(5):
        _dot_noalloc(ctx, a, b, out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(d)
    assert free1 == free0


MAX_LEN = 4096 * 65536  # SG_DOT_NOALLOC_MAX_LEN


def test_no_alloc_dot_limits(gpu_ctx):
    ctx = gpu_ctx
    d = ctx.device
    out = torch.full((1,), 7.0, dtype=torch.float64, device=d)
    a = torch.ones(4, dtype=torch.float64, device=d)
    # an empty vector gives 0
    assert _dot_noalloc(ctx, a[:0], a[:0], out) == 0.0
    # a length beyond the static scratch is rejected before any launch
    with pytest.raises(_lib.SimitError, match="outside"):
        _lib.call("sg_dot_noalloc", ctypes.c_void_p(0), MAX_LEN + 1, 1,
                  ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(a.data_ptr()),
                  ctypes.c_void_p(out.data_ptr()))
