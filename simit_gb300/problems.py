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


def reorder_hetero(host, bits=10, curve="morton"):
    """The workload with vertices along a space-filling curve of their rest
    positions (Morton by default; "hilbert" as simit::reorder) and elements
    sorted by their endpoints; also returns vertex_ordering (old -> new) to
    map solutions back: u_old = u_new.reshape(-1, 3)[vo]."""
    from .runtime import reorder_mesh
    vo, eo, tets = reorder_mesh(host["n"], host["tets"], 4, host["X0"], bits, curve)
    out = dict(host)
    out["tets"] = tets
    for k in ("X0", "x"):
        a = np.empty_like(host[k].reshape(-1, 3))
        a[vo] = host[k].reshape(-1, 3)
        out[k] = a.reshape(-1)
    c = np.empty_like(host["c"])
    c[vo] = host["c"]
    out["c"] = c
    out["mu"], out["lam"] = host["mu"][eo], host["lam"][eo]
    out["vertex_ordering"] = vo
    return out


class HeteroElasticity:
    """Device-resident instance: pattern, B/W, parameters, matrix and solver.

    dtype float32: FP32 assembly and the mixed-precision solver
    (FP32 matrix/SpMV, FP64 dots and reliable updates); float64: FP64
    assembly and FP64 CG.  storage = STORAGE_SYMMETRIC iterates on the
    matrix's upper half (the FP32 linear-tet stiffness is exactly symmetric).
    """

    def __init__(self, ctx, host, dtype=torch.float32, precond=_lib.PRECOND_BLOCK_JACOBI,
                 precision=None, tol=1e-8, maxiters=200000, lanes=0, storage=None, pdl=0,
                 plan="gather", learned_params=None, learned_exec=_lib.MPNN_EXEC_FOLDED,
                 tune=False, reliable_delta=0.1):
        self.ctx, self.host, self.dtype = ctx, host, dtype
        # plan: the element-parallel assembly plan ("gather", "colored"; each
        # element computed once), or None for the row-owner kernels
        self.mesh = Mesh(ctx, host["n"], host["tets"], 4, plan=plan)
        d = ctx.device
        with ctx.stream():
            self.X0 = torch.tensor(host["X0"], dtype=dtype, device=d)
            self.x = torch.tensor(host["x"], dtype=dtype, device=d)
            self.mu = torch.tensor(host["mu"], dtype=dtype, device=d)
            self.lam = torch.tensor(host["lam"], dtype=dtype, device=d)
            self.c = torch.tensor(host["c"], device=d)
            self.v0 = torch.zeros(host["n"] * 3, dtype=dtype, device=d)
            self.u = torch.zeros(host["n"] * 3, dtype=torch.float64, device=d)
            self.f = torch.zeros(host["n"] * 3, dtype=dtype, device=d)
        self.B, self.W, _ = tet_precompute(self.mesh, self.X0, RHO, dtype=dtype)
        self.assemble()
        # tune: the assembly plan and element tile, and the solver's SpMV
        # schedule, from timings on this mesh and matrix
        if precision is None:
            precision = _lib.SOLVE_MIXED if dtype == torch.float32 else _lib.SOLVE_F64
        self.tuned = None
        if tune:
            from .runtime import tune_spmv
            m = self.mesh
            self.tuned = {"assembly": m.tune_assembly(self.assemble_in_place)}
            xdt = torch.float32 if precision == _lib.SOLVE_MIXED else torch.float64
            # timed here (and cached); the solver's set-up takes the cached choice
            self.tuned["spmv"] = tune_spmv(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx,
                                           self.A, m.nnzb, xdt=xdt)
            lanes = _lib.LANES_AUTOTUNE
        if storage is None:
            storage = _lib.STORAGE_FULL
        # precond PRECOND_LEARNED: the learned preconditioner with
        # learned_params (a device FP32 tensor), symmetric form
        self.opts = solve_opts(precision=precision, precond=precond, stop=_lib.STOP_RELATIVE,
                               tol=tol, maxiters=maxiters, verify=1, lanes=lanes,
                               reliable_delta=reliable_delta,
                               storage=storage, pdl=pdl, learned_params=learned_params,
                               learned_form=_lib.MPNN_SYM, learned_exec=learned_exec)
        self.solver = Solver(ctx, self.mesh.n, 3, self.mesh.pattern.rowptr,
                             self.mesh.pattern.colidx, self.A, self.mesh.nnzb, self.opts,
                             learned_params_keep=learned_params)

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

    def assemble_in_place(self):
        """The step's assembly: the stiffness map into A and the force map
        into f, in place; returns f."""
        m = self.mesh
        from .runtime import call, ptr, dtype_code, _host_f64
        call("sg_assemble_tet_stiffness", self.ctx.h, m.ref(), dtype_code(self.A),
             _lib.MODEL_LINEAR, ptr(self.x), ptr(self.c), ptr(self.B), ptr(self.W), ptr(self.mu),
             ptr(self.lam), H, RHO, ptr(self.A), 0)
        call("sg_assemble_tet_force", self.ctx.h, m.ref(), dtype_code(self.f), _lib.MODEL_LINEAR,
             ptr(self.x), ptr(self.v0), ptr(self.c), ptr(self.B), ptr(self.W), ptr(self.mu),
             ptr(self.lam), H, RHO, _host_f64(GRAV), ptr(self.f), 0)
        return self.f

    def step(self):
        """One pass of the hot path: assemble in place, refresh the solver's
        matrix data, solve from zero (the solver widens the force to FP64
        itself); only the library's own kernels run."""
        f = self.assemble_in_place()
        self.solver.refresh()
        return self.solver.solve_ex(f, self.u, x_zero=True)

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


# ---------------------------------------------------------------------------
# Batched cloth (apps/cloth form, implicit springs as apps/springs/isprings.sim)
# ---------------------------------------------------------------------------
CLOTH = {"k_stretch": 5e3, "k_bend": 50.0, "mass": 1e-3, "dt": 1.0 / 240.0, "viscous": 0.0,
         "grav": (0.0, 0.0, -9.81), "tol": 1e-6}


def cloth_sides(nsheets=256, lo=32, hi=256, seed=5):
    """Side lengths (vertices per side) of the seeded sheet batch."""
    return meshgen.rng(seed).integers(lo, hi + 1, size=nsheets)


def cloth_batch(nsheets=256, lo=32, hi=256, seed=5, jitter=0.2, select=None):
    """nsheets triangulated square sheets with side lengths uniform in
    [lo, hi] vertices, concatenated (vertex and spring offsets) into one
    edge set.  Positions: unit sheet, z jittered by +/- jitter * spacing
    (seeded), rest lengths of the flat sheet, v = 0, two corners pinned.
    select: the indices of the sheets to build (a shard); each sheet is the
    same whichever shard holds it."""
    sides = cloth_sides(nsheets, lo, hi, seed)
    idx = range(nsheets) if select is None else [int(i) for i in select]
    xs, eps, ks, l0s, fixed, sys_ptr = [], [], [], [], [], [0]
    off = 0
    for i in idx:
        s = sides[i]
        sh = meshgen.cloth_sheet(int(s))
        x = sh["x"].reshape(-1, 3).copy()
        spacing = 1.0 / (s - 1)
        x[:, 2] += meshgen.rng(seed * 7919 + i).uniform(-jitter, jitter, len(x)) * spacing
        xs.append(x.reshape(-1))
        eps.append(sh["ep"] + off)
        ks.append(np.where(sh["is_bend"] > 0, CLOTH["k_bend"], CLOTH["k_stretch"]))
        l0s.append(sh["l0"])
        fixed.append(sh["fixed"])
        off += sh["n"]
        sys_ptr.append(off)
    return {"n": off, "x": np.concatenate(xs), "ep": np.concatenate(eps).astype(np.int32),
            "k": np.concatenate(ks), "l0": np.concatenate(l0s), "fixed": np.concatenate(fixed),
            "sys_ptr": np.array(sys_ptr, np.int32), "sides": np.asarray(sides)[list(idx)]}


class ClothBatch:
    """Device-resident cloth batch: assembly of all sheets in one launch and
    the batched PCG (one persistent launch), optionally captured as one CUDA
    graph."""

    def __init__(self, ctx, host, config=None):
        from .runtime import assemble_springs
        self.ctx, self.host = ctx, host
        self.mesh = Mesh(ctx, host["n"], host["ep"], 2)
        d = ctx.device
        n = host["n"]
        sp = host["sys_ptr"]
        sizes = np.diff(sp)
        order = np.argsort(-sizes, kind="stable").astype(np.int32)
        with ctx.stream():
            self.x = torch.tensor(host["x"], dtype=torch.float32, device=d)
            self.v = torch.zeros(n * 3, dtype=torch.float32, device=d)
            self.m = torch.full((n,), CLOTH["mass"], dtype=torch.float32, device=d)
            self.fixed = torch.tensor(host["fixed"], dtype=torch.uint8, device=d)
            self.k = torch.tensor(host["k"], dtype=torch.float32, device=d)
            self.l0 = torch.tensor(host["l0"], dtype=torch.float32, device=d)
            self.sys_ptr = torch.tensor(sp, device=d)
            self.order = torch.tensor(order, device=d)
            self.iters = torch.zeros(len(sizes), dtype=torch.int32, device=d)
            self.status = torch.zeros(len(sizes), dtype=torch.int32, device=d)
            self.relres = torch.zeros(len(sizes), dtype=torch.float64, device=d)
            self.vout = torch.zeros(n * 3, dtype=torch.float32, device=d)
        self.nsys = len(sizes)
        self.A, self.f = assemble_springs(self.mesh, self.x, self.v, self.m, self.fixed, self.k,
                                          self.l0, CLOTH["dt"], CLOTH["viscous"], CLOTH["grav"],
                                          form=0, dtype=torch.float32, exact=False)
        self.Am = _lib.Matrix(n, 3, self.mesh.nnzb, self.mesh.pattern.rowptr.data_ptr(),
                              self.mesh.pattern.colidx.data_ptr(), _lib.F32, self.A.data_ptr())
        self.config = config if config is not None else self.autotune()
        self.graph = None

    def step(self, config=None, maxiters=10000):
        """Assemble every sheet and solve every system (the batched path)."""
        import ctypes
        from .runtime import call, ptr, dtype_code
        m = self.mesh
        call("sg_assemble_springs", self.ctx.h, m.ref(), dtype_code(self.A), 0, ptr(self.x),
             ptr(self.v), ptr(self.m), ptr(self.fixed), ptr(self.k), ptr(self.l0), CLOTH["dt"],
             CLOTH["viscous"], (ctypes.c_double * 3)(*CLOTH["grav"]), ptr(self.A), ptr(self.f), 0)
        with self.ctx.stream():
            self.vout.copy_(self.v)
        call("sg_batched_pcg", self.ctx.h, self.nsys, ptr(self.sys_ptr), ptr(self.order),
             ctypes.byref(self.Am), ptr(self.f), ptr(self.vout), CLOTH["tol"], maxiters,
             self.config if config is None else config, ptr(self.iters), ptr(self.status),
             ptr(self.relres))

    def autotune(self):
        """Time every batched-PCG configuration once; keep the fastest."""
        best, best_ms = 0, None
        st = self.ctx.torch_stream
        self.config = 0
        self.step(config=0)  # sizes the scratch arena
        for cfg in range(_lib.load().sg_batched_configs()):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            self.step(config=cfg)
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            if best_ms is None or ms < best_ms:
                best, best_ms = cfg, ms
        self.tuned_ms = best_ms
        return best

    def capture(self):
        """One CUDA graph holding the assembly and the batched solve."""
        self.step()  # warm (arena sized, attributes set)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.ctx.torch_stream):
            self.step()
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
