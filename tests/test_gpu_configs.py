"""GPU parity at the benchmark configurations' own sizes: the five-tet
lattices of the neo-Hookean (64^3) and elasticity / heat (128^3) configs,
their sparsity patterns and element-to-slot maps against SHA-256 digests of
the reference's own PathIndexBuilder and `loc` (tests/golden/
lattice_golden.json, generated by tests/golden/make_golden.py), the 64^3
pattern against the oracle restatement, and the 64^3 FP64 assembly against
the oracle: bit-exact for the linear tet in exact mode, 1e-12 relative for
neo-Hookean and for the element-parallel plan."""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from simit_gb300 import _lib, meshgen, problems

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ctx(gpu_ctx):
    return gpu_ctx


def _sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.dtype(dtype).newbyteorder("<"))
                          .tobytes()).hexdigest()


def _golden():
    with open(os.path.join(HERE, "golden", "lattice_golden.json")) as f:
        return json.load(f)


def _tets(name):
    if name == "tet_grid_64":
        return meshgen.tet_grid(64)["tets"]
    if name == "tet_grid_128":
        return meshgen.tet_grid(128)["tets"]
    return problems.reorder_hetero(problems.hetero_mesh(128))["tets"]


@pytest.mark.parametrize("name", ["tet_grid_64", "tet_grid_128", "tet_grid_128_morton"])
def test_lattice_pattern_and_slots_match_reference_builder(ctx, name):
    """The GPU pattern builder and slot map on the configs' lattices, bit for
    bit the reference builder's (compared through digests)."""
    from simit_gb300.runtime import Mesh
    g = _golden()[name]
    tets = _tets(name)
    assert _sha(tets, np.int32) == g["endpoints_sha256"], "generator differs from the fixture"
    mesh = Mesh(ctx, g["n"], tets, 4, with_slots=True)
    assert mesh.nnzb == g["nnzb"]
    rp, ci = mesh.pattern.host()
    sl = mesh.pattern.slots[:mesh.nE * 16].cpu().numpy().view(np.uint32)
    assert _sha(rp, np.uint32) == g["rowptr_sha256"]
    assert _sha(ci, np.uint32) == g["colidx_sha256"]
    assert _sha(sl, np.uint32) == g["slots_sha256"]


def _neo_config(ncell=64, seed=1):
    """Config 2's instance: E 1e5, nu 0.4, density 1e3, displacement
    U(+-1e-3), bottom face fixed."""
    mg = meshgen.tet_grid(ncell, disp=1e-3, seed=seed)
    nT = len(mg["tets"]) // 4
    E, nu = 1e5, 0.4
    mg["mu"] = np.full(nT, E / (2 * (1 + nu)))
    mg["lam"] = np.full(nT, E * nu / ((1 + nu) * (1 - 2 * nu)))
    mg["c"] = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    return mg


def test_64cube_pattern_matches_oracle(ctx, oracle):
    from simit_gb300.runtime import Mesh
    mg = meshgen.tet_grid(64)
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4, with_slots=True)
    rp, ci = mesh.pattern.host()
    orp, oci = oracle.pattern(mg["n"], mg["tets"], 4)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    osl = oracle.slots(mg["tets"], 4, orp, oci)
    assert np.array_equal(mesh.pattern.slots[:mesh.nE * 16].cpu().numpy().view(np.uint32), osl)


def test_64cube_fp64_assembly_matches_oracle(ctx, oracle):
    """Config 2 at its own size in FP64: the linear-tet stiffness bit for bit
    (exact mode, the reference's element order), neo-Hookean stiffness and
    force within 1e-12 of the largest entry, and the element-parallel plan's
    linear-tet stiffness within 1e-12."""
    from simit_gb300.runtime import (Mesh, assemble_tet_force, assemble_tet_stiffness,
                                     tet_precompute)
    mg = _neo_config()
    n = mg["n"]
    mesh = Mesh(ctx, n, mg["tets"], 4, plan="gather")
    rp, ci = mesh.pattern.host()
    B, W, _ = tet_precompute(mesh, mg["X0"], 1e3)
    oB, oW, _ = oracle.tet_precompute(mg["X0"], mg["tets"], 1e3)
    args = (mg["x"], mg["c"], B, W, mg["mu"], mg["lam"], 1.0, 1e3)
    oargs = (mg["x"], mg["c"], mg["tets"], oB, oW, mg["mu"], mg["lam"], 1.0, 1e3, rp, ci)
    A = assemble_tet_stiffness(mesh, _lib.MODEL_LINEAR, *args, exact=True)
    oA = oracle.tet_stiffness(0, *oargs)
    ctx.sync()
    assert np.array_equal(A.cpu().numpy(), oA)
    Ag = assemble_tet_stiffness(mesh, _lib.MODEL_LINEAR, *args, exact=False)
    ctx.sync()
    assert np.abs(Ag.cpu().numpy() - oA).max() <= 1e-12 * np.abs(oA).max()
    del A, Ag
    nm = _lib.MODEL_NEOHOOKEAN
    An = assemble_tet_stiffness(mesh, nm, *args, exact=True)
    oAn = oracle.tet_stiffness(1, *oargs)
    ctx.sync()
    assert np.abs(An.cpu().numpy() - oAn).max() <= 1e-12 * np.abs(oAn).max()
    v = np.zeros(n * 3)
    grav = np.array([0.0, 0.0, -9.81])
    f = assemble_tet_force(mesh, nm, mg["x"], v, mg["c"], B, W, mg["mu"], mg["lam"], 1.0, 1e3,
                           grav, exact=True)
    of = oracle.tet_force(1, mg["x"], v, mg["c"], mg["tets"], oB, oW, mg["mu"], mg["lam"], 1.0,
                          1e3, grav)
    ctx.sync()
    assert np.abs(f.cpu().numpy() - of).max() <= 1e-12 * np.abs(of).max()
