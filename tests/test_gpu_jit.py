"""Element kernels compiled at run time (sg_jit_assembly_*): CUDA source for
the element function, NVRTC, the generated row-owner assembly — against the
built-in kernels and the oracle, bit for bit."""
import numpy as np
import pytest
import torch

from simit_gb300 import meshgen

pytestmark = pytest.mark.gpu

BLOCKS_SRC = r"""
// block (i, j) of element e read from a precomputed array f[0]
__device__ int element_block(long long e, int i, int j, const int *ep, const real *const *f,
                             real blk[BS][BS]) {
  const real *b = f[0] + ((e * CARD + i) * CARD + j) * BS * BS;
  for (int a = 0; a < BS; ++a)
    for (int c = 0; c < BS; ++c) blk[a][c] = b[a * BS + c];
  return 1;
}
"""

# the P1 heat element (A_ij = W/20 (1 + d_ij) + (dt kappa W) g_i.g_j, dt = 0.01)
# in the operation order of the built-in kernel, from fields B, W, kappa
HEAT_SRC = r"""
__device__ void grad(const real *Bt, int i, real g[3]) {
  for (int d = 0; d < 3; ++d)
    g[d] = (i < 3) ? Bt[i * 3 + d] : -((Bt[0 * 3 + d] + Bt[1 * 3 + d]) + Bt[2 * 3 + d]);
}
__device__ int element_block(long long e, int i, int j, const int *ep, const real *const *f,
                             real blk[BS][BS]) {
  const real *Bt = f[0] + 9 * e;
  real gi[3], gj[3];
  grad(Bt, i, gi);
  grad(Bt, j, gj);
  const real dt = (real)0.01;
  const real mw = f[1][e] / real(20.0);
  const real kw = (dt * f[2][e]) * f[1][e];
  const real mij = (i == j) ? real(2.0) * mw : mw;
  const real gg = (gi[0] * gj[0] + gi[1] * gj[1]) + gi[2] * gj[2];
  blk[0][0] = mij + kw * gg;
  return 1;
}
"""


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


def test_jit_compile_error_is_reported(ctx):
    from simit_gb300._lib import SimitError
    from simit_gb300.runtime import JitAssembly
    with pytest.raises(SimitError, match="does not compile"):
        JitAssembly(ctx, "__device__ int element_block(this is not C++", 2, 1)
