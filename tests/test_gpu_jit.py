"""Element kernels compiled at run time (sg_jit_assembly_*): CUDA source for
the element function, NVRTC, the generated row-owner assembly — against the
built-in kernels and the oracle, bit for bit."""
import numpy as np
import pytest
import torch

from simit_gb300 import jit_elements, meshgen

pytestmark = pytest.mark.gpu

BLOCKS_SRC = jit_elements.BLOCKS
HEAT_SRC = jit_elements.heat(0.01)


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


@pytest.mark.parametrize("bs,card,dtype", [(3, 4, torch.float64), (1, 2, torch.float32),
                                           (2, 3, torch.float64)])
def test_jit_blocks_match_builtin_and_oracle(ctx, oracle, bs, card, dtype):
    from simit_gb300.runtime import JitAssembly, Mesh, assemble_blocks
    g = meshgen.rng(3 * bs + card)
    n, nE = 400, 900
    ep = g.integers(0, n, size=(nE, card)).astype(np.int32)
    ep[::6, card - 1] = ep[::6, 0]  # an element that lists a vertex twice
    eb = g.uniform(-1, 1, size=(nE, card, card, bs, bs))
    mesh = Mesh(ctx, n, ep.reshape(-1), card)
    jit = JitAssembly(ctx, BLOCKS_SRC, card, bs, dtype=dtype)
    got = jit.assemble(mesh, [eb.reshape(-1)])
    ref = assemble_blocks(mesh, eb, bs, dtype=dtype)
    ctx.sync()
    assert torch.equal(got, ref)
    if dtype == torch.float64:
        rp, ci = mesh.pattern.host()
        o = oracle.assemble_blocks(ep.reshape(-1), card, bs, eb, rp, ci)
        assert np.array_equal(got[:mesh.nnzb * bs * bs].cpu().numpy(), o)
    jit.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_jit_heat_element_matches_builtin(ctx, dtype):
    """The P1 heat element written as CUDA source assembles the same matrix
    as the built-in heat kernel, bit for bit (both without contraction)."""
    from simit_gb300.runtime import JitAssembly, Mesh, assemble_heat, tet_precompute
    mg = meshgen.tet_grid(6)
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(5)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, mg["n"])
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], 1.0, dtype=dtype)
    A, _ = assemble_heat(mesh, B, W, kappa, 1e-2, T0, dtype=dtype)
    jit = JitAssembly(ctx, HEAT_SRC, 4, 1, dtype=dtype)
    with ctx.stream():
        kap = torch.tensor(kappa, dtype=dtype, device=ctx.device)
    got = jit.assemble(mesh, [B, W, kap])
    ctx.sync()
    assert torch.equal(got[:mesh.nnzb], A[:mesh.nnzb])
    jit.close()


@pytest.mark.parametrize("dtype,exact", [(torch.float32, False), (torch.float64, False),
                                         (torch.float32, True)])
def test_jit_linear_tet_matches_builtin(ctx, dtype, exact):
    """The linear-elastic tetrahedron (stiffness where both vertices are free,
    then the lumped mass as a second write on the diagonal block) as CUDA
    source: the same matrix, bit for bit, as the precompiled closed-form
    kernel, with per-element parameters and constrained vertices."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import JitAssembly, Mesh, assemble_tet_stiffness, tet_precompute
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
    jit = JitAssembly(ctx, jit_elements.linear_tet(h, rho), 4, 3, dtype=dtype, exact=exact)
    got = jit.assemble(mesh, [B, W, mu, lam, c])
    ctx.sync()
    k = mesh.nnzb * 9
    assert torch.equal(got[:k], A[:k])
    jit.close()


def test_jit_wide_elements_match_oracle(ctx, oracle):
    """card 8, 5x5 blocks: more (j, row) pairs than lanes, fewer warps per
    block for shared memory, elements that repeat vertices."""
    from simit_gb300.runtime import JitAssembly, Mesh
    card, bs = 8, 5
    g = meshgen.rng(21)
    n, nE = 300, 260
    ep = g.integers(0, n, size=(nE, card)).astype(np.int32)
    ep[::5, 3] = ep[::5, 6]
    ep[::7, 1] = ep[::7, 0]
    eb = g.uniform(-1, 1, size=(nE, card, card, bs, bs))
    mesh = Mesh(ctx, n, ep.reshape(-1), card)
    jit = JitAssembly(ctx, BLOCKS_SRC, card, bs, dtype=torch.float64)
    got = jit.assemble(mesh, [eb.reshape(-1)])
    ctx.sync()
    rp, ci = mesh.pattern.host()
    o = oracle.assemble_blocks(ep.reshape(-1), card, bs, eb, rp, ci)
    assert np.array_equal(got[:mesh.nnzb * bs * bs].cpu().numpy(), o)
    jit.close()


def test_jit_compile_error_is_reported(ctx):
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import JitAssembly
    with pytest.raises(SimitError, match="does not compile"):
        JitAssembly(ctx, "__device__ int element_block(this is not C++", 2, 1)
