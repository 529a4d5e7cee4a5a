"""`.sim` programs on the GPU: the front end's element functions, compiled
by NVRTC into the row-owner assembly, against the precompiled element
kernels and the oracle, bit for bit.  The programs are the ones under
tests/sim (written for this repository)."""
import os

import numpy as np
import pytest
import torch

from simit_gb300 import meshgen, simfront

pytestmark = pytest.mark.gpu

SIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sim")


def _own(name):
    with open(os.path.join(SIM, name)) as f:
        return f.read()


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_tet_matches_precompiled_kernel(ctx, dtype):
    """tests/sim/tet_closed_form.sim (per-element mu, lambda; constrained
    vertices; stiffness then lumped mass on the diagonal) compiled without
    contraction gives the precompiled linear-tet kernel's matrix bit for bit."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import Mesh, assemble_tet_stiffness, tet_precompute
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
    sm = simfront.SimMap(ctx, _own("tet_closed_form.sim"), "tet_stiffness",
                         {"h": h, "rho": rho}, dtype=dtype, exact=True)
    got = sm.assemble(mesh, {"B": B, "W": W, "u": mu, "l": lam, "c": c})
    ctx.sync()
    k = mesh.nnzb * 9
    assert torch.equal(got[:k], A[:k])
    sm.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_heat_matches_precompiled_kernel_and_oracle(ctx, oracle, dtype):
    """tests/sim/heat_p1.sim: the precompiled heat kernel's matrix bit for
    bit, and in FP64 the oracle's."""
    from simit_gb300.runtime import Mesh, assemble_heat, tet_precompute
    mg = meshgen.tet_grid(6)
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(5)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, mg["n"])
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], 1.0, dtype=dtype)
    A, _ = assemble_heat(mesh, B, W, kappa, 1e-2, T0, dtype=dtype)
    sm = simfront.SimMap(ctx, _own("heat_p1.sim"), "heat", {"dt": 1e-2}, dtype=dtype)
    got = sm.assemble(mesh, {"B": B, "W": W, "kappa": kappa})
    ctx.sync()
    assert torch.equal(got[:mesh.nnzb], A[:mesh.nnzb])
    if dtype == torch.float64:
        rp, ci = mesh.pattern.host()
        o, _ = oracle.heat_assemble(mg["n"], mg["tets"], B.cpu().numpy(), W.cpu().numpy(),
                                    kappa, 1e-2, T0, rp, ci)
        assert np.array_equal(got[:mesh.nnzb].cpu().numpy(), o)
    sm.close()


def test_sim_vertex_map_with_component_writes(ctx):
    """tests/sim/point_mass.sim: a map over the vertices (a mesh whose
    elements are the vertices), a full block write and component writes."""
    from simit_gb300.runtime import Mesh
    n = 1000
    g = meshgen.rng(9)
    m = g.uniform(1.0, 2.0, n)
    fixed = g.uniform(0, 1, n) < 0.3
    mesh = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    sm = simfront.SimMap(ctx, _own("point_mass.sim"), "point_mass", {"damp": 0.5}, result="M")
    got = sm.assemble(mesh, {"m": m, "fixed": fixed})
    ctx.sync()
    rp, ci = mesh.pattern.host()
    assert np.array_equal(rp, np.arange(n + 1)) and np.array_equal(ci, np.arange(n))
    want = m[:, None, None] * np.eye(3)[None]
    free = ~fixed
    want[free, 0, 0] += 0.5 * m[free]
    want[free, 2, 2] += (2.0 * 0.5) * m[free]
    assert np.array_equal(got[:n * 9].cpu().numpy().reshape(n, 3, 3), want)
    sm.close()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_sim_tet_force_vector_map_matches_precompiled_and_oracle(ctx, oracle, dtype):
    """tests/sim/tet_force.sim, a map whose result is a system vector,
    through the vertex-owner kernel generated for element_vector: the
    precompiled linear force kernel's values bit for bit, and in FP64 the
    oracle's (per-tet parameters, constrained vertices, momentum)."""
    from simit_gb300 import _lib
    from simit_gb300.runtime import Mesh, assemble_tet_force, tet_precompute
    mg = meshgen.tet_grid(7, 6, 5, disp=1e-3, seed=4)
    nT, n = len(mg["tets"]) // 4, mg["n"]
    g = meshgen.rng(15)
    mu = 10 ** g.uniform(3, 5, nT)
    lam = 10 ** g.uniform(3, 5, nT)
    c = (g.uniform(0, 1, n) < 0.1).astype(np.int32)
    v = g.uniform(-0.01, 0.01, n * 3)
    h, rho, grav = 0.01, 1e3, np.array([0.0, -9.81, 0.0])
    mesh = Mesh(ctx, n, mg["tets"], 4)
    B, W, _ = tet_precompute(mesh, mg["X0"], rho, dtype=dtype)
    want = assemble_tet_force(mesh, _lib.MODEL_LINEAR, mg["x"], v, c, B, W, mu, lam, h, rho,
                              grav, dtype=dtype, exact=True)
    sm = simfront.SimMap(ctx, _own("tet_force.sim"), "tet_force",
                         {"h": h, "rho": rho, "gx": 0.0, "gy": -9.81, "gz": 0.0},
                         dtype=dtype, exact=True)
    got = sm.assemble(mesh, {"B": B, "W": W, "u": mu, "l": lam, "c": c, "x": mg["x"], "v": v})
    ctx.sync()
    assert torch.equal(got[:n * 3], want[:n * 3])
    if dtype == torch.float64:
        of = oracle.tet_force(0, mg["x"], v, c, mg["tets"], B.cpu().numpy(), W.cpu().numpy(),
                              mu, lam, h, rho, grav)
        assert np.array_equal(got[:n * 3].cpu().numpy(), of)
    sm.close()


def test_sim_vertex_map_vector_result(ctx):
    """tests/sim/point_mass.sim's vector result g (a map over the
    vertices): m (0, -9.8, 0) per vertex."""
    from simit_gb300.runtime import Mesh
    n = 777
    m = meshgen.rng(16).uniform(1.0, 2.0, n)
    fixed = np.zeros(n, bool)
    mesh = Mesh(ctx, n, np.arange(n, dtype=np.int32), 1)
    sm = simfront.SimMap(ctx, _own("point_mass.sim"), "point_mass", {"damp": 0.5}, result="g")
    got = sm.assemble(mesh, {"m": m, "fixed": fixed})
    ctx.sync()
    want = np.zeros((n, 3))
    want[:, 1] = -9.8 * m
    assert np.array_equal(got[:n * 3].cpu().numpy().reshape(n, 3), want)
    sm.close()
