"""Synthetic workloads of the sparse-system path, built on the C ABI.

HeteroElasticity: linear-tetrahedral elasticity in the apps/fem/fem_linear.sim
form (compute_stiffness + compute_force, lumped element mass on the diagonal)
on the n^3 five-tet unit-cube lattice, Young's modulus log-uniform in
[1e3, 1e6] and Poisson ratio uniform in [0.35, 0.45] per tet, density 1e3,
time step h = 1 (the stiffness dominates the mass), gravity -9.81 on z,
vertices on the z = 0 face constrained, deformed positions = rest + uniform
+/-1e-3.  The system A u = b is solved to a 1e-8 FP64 relative residual.
"""
import numpy as np
import torch

from . import _lib, meshgen
from .runtime import (Mesh, Solver, assemble_tet_force, assemble_tet_stiffness, solve_opts,
                      tet_precompute)

RHO = 1e3
H = 1.0
GRAV = np.array([0.0, 0.0, -9.81])


def hetero_params(nT, seed):
    g = meshgen.rng(seed + 1)
    E = 10 ** g.uniform(3, 6, nT)
    nu = g.uniform(0.35, 0.45, nT)
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    return mu, lam


def hetero_mesh(ncell, seed=1):
    """Host arrays of the workload (numpy)."""
    mg = meshgen.tet_grid(ncell, disp=1e-3, seed=seed)
    nT = len(mg["tets"]) // 4
    mu, lam = hetero_params(nT, seed)
    c = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    return {"n": mg["n"], "tets": mg["tets"], "X0": mg["X0"], "x": mg["x"], "mu": mu,
            "lam": lam, "c": c, "ncell": ncell}


class HeteroElasticity:
    """Device-resident instance: pattern, B/W, parameters, matrix and solver.

    dtype float32: FP32 assembly and the mixed-precision solver
    (FP32 matrix/SpMV, FP64 dots and reliable updates); float64: FP64
    assembly and FP64 CG.
    """

    def __init__(self, ctx, host, dtype=torch.float32, precond=_lib.PRECOND_BLOCK_JACOBI,
                 precision=None, tol=1e-8, maxiters=200000, lanes=0):
        self.ctx, self.host, self.dtype = ctx, host, dtype
        self.mesh = Mesh(ctx, host["n"], host["tets"], 4)
        d = ctx.device
        with ctx.stream():
            self.X0 = torch.tensor(host["X0"], dtype=dtype, device=d)
            self.x = torch.tensor(host["x"], dtype=dtype, device=d)
            self.mu = torch.tensor(host["mu"], dtype=dtype, device=d)
            self.lam = torch.tensor(host["lam"], dtype=dtype, device=d)
            self.c = torch.tensor(host["c"], device=d)
            self.v0 = torch.zeros(host["n"] * 3, dtype=dtype, device=d)
            self.u = torch.zeros(host["n"] * 3, dtype=torch.float64, device=d)
        self.B, self.W, _ = tet_precompute(self.mesh, self.X0, RHO, dtype=dtype)
        self.assemble()
        if precision is None:
            precision = _lib.SOLVE_MIXED if dtype == torch.float32 else _lib.SOLVE_F64
        self.opts = solve_opts(precision=precision, precond=precond, stop=_lib.STOP_RELATIVE,
                               tol=tol, maxiters=maxiters, verify=1, lanes=lanes)
        self.solver = Solver(ctx, self.mesh.n, 3, self.mesh.pattern.rowptr,
                             self.mesh.pattern.colidx, self.A, self.mesh.nnzb, self.opts)

    @property
    def dofs(self):
        return self.mesh.n * 3

    def assemble(self):
        """A (stiffness*h^2 + lumped mass) and b (compute_force) on the device."""
        m = self.mesh
        self.A = assemble_tet_stiffness(m, _lib.MODEL_LINEAR, self.x, self.c, self.B, self.W,
                                        self.mu, self.lam, H, RHO, dtype=self.dtype, exact=False)
        f = assemble_tet_force(m, _lib.MODEL_LINEAR, self.x, self.v0, self.c, self.B, self.W,
                               self.mu, self.lam, H, RHO, GRAV, dtype=self.dtype, exact=False)
        with self.ctx.stream():
            self.b = f.to(torch.float64)
        return self.A, self.b

    def step(self):
        """One pass of the hot path: assemble in place, refresh, solve from 0."""
        m = self.mesh
        from .runtime import call, ptr, dtype_code
        call("sg_assemble_tet_stiffness", self.ctx.h, m.ref(), dtype_code(self.A),
             _lib.MODEL_LINEAR, ptr(self.x), ptr(self.c), ptr(self.B), ptr(self.W), ptr(self.mu),
             ptr(self.lam), H, RHO, ptr(self.A), 0)
        f = assemble_tet_force(m, _lib.MODEL_LINEAR, self.x, self.v0, self.c, self.B, self.W,
                               self.mu, self.lam, H, RHO, GRAV, dtype=self.dtype, exact=False)
        with self.ctx.stream():
            self.b.copy_(f)
            self.u.zero_()
        self.solver.refresh()
        return self.solver.solve(self.b, self.u)

    def step_host(self, x_host, mu_host, lam_host, u_host):
        """End to end through host buffers: pinned inputs (positions and the
        per-tet parameters) copied in, one step, the solution copied out."""
        with self.ctx.stream():
            self.x.copy_(x_host, non_blocking=True)
            self.mu.copy_(mu_host, non_blocking=True)
            self.lam.copy_(lam_host, non_blocking=True)
        res = self.step()
        with self.ctx.stream():
            u_host.copy_(self.u, non_blocking=True)
        self.ctx.sync()
        return res

    def close(self):
        self.solver.close()
