"""Benchmark: time and DOF/s to a 1e-8 FP64 relative residual on the 128^3
heterogeneous-elasticity system (6,440,067 DOF), mixed-precision PCG on the
GB300 against plain FP64 Jacobi-CG on the same GPU.

A step is one pass of the hot path: assemble the FP32 stiffness matrix and
right-hand side from the resident mesh, refresh the preconditioner, and
solve to ||b - A x|| <= 1e-8 ||b|| (true FP64 residual).  The matrix (1.0 GB
in FP32) is larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--size S]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time & DOF/s to 1e-8 residual: learned+FP32 PCG vs plain FP64 CG, 1 GB300"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=128, help="cells per cube edge")
    ap.add_argument("--cpu-sample", type=int, default=48,
                    help="cells per edge of the instance whose oracle FP64 solution the GPU "
                         "solutions are compared to (48: about 15-25 s of one core)")
    ap.add_argument("--no-tune", action="store_true",
                    help="default schedules instead of the autotuners' choices")
    ap.add_argument("--reliable-delta", type=float, default=0.01,
                    help="mixed PCG: the true residual replaces the iterated one each time "
                         "the latter falls by this factor (0.01: 5 replacements per 128^3 "
                         "solve instead of 8 at 0.1, 2.4 ms less per step)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the heat / neo-Hookean / springs / cloth measurements that "
                         "follow the headline")
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU baseline and the solution check against the oracle")
    ap.add_argument("--no-block-jacobi", action="store_true",
                    help="skip the block-Jacobi step (the method without the network)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 Jacobi-CG comparison")
    ap.add_argument("--no-reorder", action="store_true",
                    help="keep the lattice vertex order (no space-filling-curve reordering)")
    ap.add_argument("--no-jit", action="store_true",
                    help="skip timing the stiffness map compiled at run time (NVRTC)")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-preconditioner comparison")
    ap.add_argument("--spmv-only", action="store_true",
                    help="profiling driver: build the --size matrix and run sg_bspmv --reps times")
    ap.add_argument("--lanes", type=int, default=0, help="sg_bspmv lanes (g) for --spmv-only")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--f64", action="store_true", help="FP64 matrix for --spmv-only")
    ap.add_argument("--tune-spmv", action="store_true",
                    help="--spmv-only: also run the SpMV autotuner and print its timings")
    ap.add_argument("--scalar", action="store_true",
                    help="--spmv-only on the P1 heat matrix (one value per entry)")
    ap.add_argument("--sym", action="store_true",
                    help="symmetric storage for the iteration's SpMV (and for --spmv-only)")
    ap.add_argument("--pdl", action="store_true",
                    help="programmatic dependent launch inside the solver's iteration graph")
    ap.add_argument("--stages", type=int, default=0,
                    help="--spmv-only --sym: bulk-copy stages per warp (2..4, 0 = default)")
    ap.add_argument("--cloth", action="store_true",
                    help="batched cloth: 256 uneven sheets in one graph launch vs one at a time")
    ap.add_argument("--sheets", type=int, default=256)
    ap.add_argument("--neo", action="store_true",
                    help="neo-Hookean Newton step (64^3): FP64 vs FP32-bulk mixed precision")
    ap.add_argument("--solve-only", action="store_true",
                    help="profiling driver: two steps of the --size system (the headline's "
                         "method) with the solver capped at --iters iterations")
    ap.add_argument("--iters", type=int, default=64)
    ap.add_argument("--block-jacobi", action="store_true",
                    help="--solve-only: mixed block-Jacobi PCG instead of the learned method")
    ap.add_argument("--learned-solve", action="store_true",
                    help="profiling driver: the --size system with the learned preconditioner, "
                         "capped at --iters iterations")
    ap.add_argument("--assembly-only", action="store_true",
                    help="profiling driver: the --size workload's assembly (stiffness map in "
                         "place + force map), element-parallel over the colouring and by row "
                         "owners, event-timed")
    ap.add_argument("--layered", action="store_true",
                    help="--learned-solve: evaluate the network layer by layer on the tensor "
                         "cores instead of folded")
    ap.add_argument("--springs", action="store_true",
                    help="createBox springs 10^3: 10 implicit FP64 steps, parity vs the oracle")
    ap.add_argument("--heat", action="store_true",
                    help="P1 heat (128^3): 1000 SpMVs FP32 vs FP64, CG FP64 vs mixed")
    return ap.parse_args()


def _ev_ms(st, fn, reps=1):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        out = fn()
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps, out


def _reorder_grid(mg, with_orders=False):
    """A meshgen.tet_grid mesh renumbered along the Morton curve of its rest
    positions, elements sorted by endpoints (as the elasticity workload)."""
    import numpy as np
    from simit_gb300.runtime import reorder_mesh
    vo, eo, tets = reorder_mesh(mg["n"], mg["tets"], 4, mg["X0"], curve="morton")
    out = dict(mg)
    out["tets"] = tets
    for k in ("X0", "x"):
        a = np.empty_like(mg[k].reshape(-1, 3))
        a[vo] = mg[k].reshape(-1, 3)
        out[k] = a.reshape(-1)
    return (out, vo, eo) if with_orders else out


def run_neo(args):
    """femTet.sim form: one implicit Newton step (A = M + h^2 K_neo(x), b =
    compute_force, h = 0.01) on the 64^3 five-tet lattice, E = 1e5, nu = 0.4,
    rho = 1e3, displacement +/-1e-3, bottom face fixed; CG to 1e-8.  FP64
    assembly + FP64 Jacobi-CG against FP32 assembly + mixed block-Jacobi PCG;
    the mixed solution's relative error against the FP64 one."""
    import numpy as np
    import torch
    from simit_gb300 import _lib, meshgen
    from simit_gb300.runtime import (Context, Mesh, Solver, assemble_tet_force,
                                     assemble_tet_stiffness, solve_opts, tet_precompute)
    size = args.size if args.size != 128 else 64
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    st = ctx.torch_stream
    mg = meshgen.tet_grid(size, disp=1e-3, seed=2)
    if not args.no_reorder:
        mg = _reorder_grid(mg)
    nT = len(mg["tets"]) // 4
    E, nu = 1e5, 0.4
    mu = np.full(nT, E / (2 * (1 + nu)))
    lam = np.full(nT, E * nu / ((1 + nu) * (1 - 2 * nu)))
    c = (mg["X0"].reshape(-1, 3)[:, 2] == 0).astype(np.int32)
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    d = ctx.device
    out = {"workload": "neo-Hookean Newton step %d^3 (%d tets, %d DOF)" % (size, nT, mg["n"] * 3)}
    sols = {}
    for name, dt, prec, pc in (("fp64", torch.float64, _lib.SOLVE_F64, _lib.PRECOND_JACOBI),
                               ("fp32_bulk", torch.float32, _lib.SOLVE_MIXED,
                                _lib.PRECOND_BLOCK_JACOBI)):
        t = lambda a: torch.tensor(a, dtype=dt, device=d)  # noqa: E731
        x, X0, v = t(mg["x"]), t(mg["X0"]), t(np.zeros(mg["n"] * 3))
        mu_d, lam_d, c_d = t(mu), t(lam), torch.tensor(c, device=d)
        B, W, _ = tet_precompute(mesh, X0, 1e3, dtype=dt)
        asm = lambda: (assemble_tet_stiffness(mesh, _lib.MODEL_NEOHOOKEAN, x, c_d, B, W, mu_d,  # noqa
                                              lam_d, 0.01, 1e3, dtype=dt, exact=False),
                       assemble_tet_force(mesh, _lib.MODEL_NEOHOOKEAN, x, v, c_d, B, W, mu_d, lam_d,
                                          0.01, 1e3, np.array([0, 0, -9.81]), dtype=dt,
                                          exact=False))
        asm()
        ms_asm, (A, f) = _ev_ms(st, asm, reps=3)
        S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
                   solve_opts(precision=prec, precond=pc, tol=1e-8, maxiters=100000))
        b = f.double()
        xs = torch.zeros_like(b)
        ms_solve, r = _ev_ms(st, lambda: S.solve(b, xs.zero_()))
        S.close()
        sols[name] = xs.cpu().numpy()
        out[name] = {"assembly_ms": ms_asm, "elements_per_s": nT / (ms_asm / 1e3),
                     "solve_ms": ms_solve, "iters": r.iters,
                     "relres": (r.true_normr2 / r.bnorm2) ** 0.5}
    out["fp32_bulk_rel_error_vs_fp64"] = float(np.linalg.norm(sols["fp32_bulk"] - sols["fp64"]) /
                                               np.linalg.norm(sols["fp64"]))
    out["speedup_solve"] = out["fp64"]["solve_ms"] / out["fp32_bulk"]["solve_ms"]
    return out


def run_springs(args):
    """createBox springs 10x10x10 (spacing 0.1, jitter 0.01, k = 1e4, m = 1,
    dt = 1e-3, gravity, bottom layer pinned), 10 implicit steps in FP64
    (apps/springs/isprings.sim form): pattern build, exact-mode assembly and
    CG to a 1e-8 relative residual per step, against the oracle (the
    reference's pattern builder and `loc`; its loops restated) on one core."""
    import numpy as np
    import torch
    from oracle import oracle
    from simit_gb300 import _lib, meshgen
    from simit_gb300.runtime import Context, Mesh, Solver, assemble_springs, solve_opts
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    L = meshgen.springs_lattice(10, 10, 10, 0.1, 0.01, seed=1)
    n, ep = L["n"], L["ep"]
    k = np.full(len(L["l0"]), 1e4)
    m = np.ones(n)
    h, grav, steps = 1e-3, np.array([0.0, 0.0, -9.81]), 10
    Mesh(ctx, n, ep, 2)  # warm (module load, scratch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mesh = Mesh(ctx, n, ep, 2, with_slots=True)
    torch.cuda.synchronize()
    pattern_ms = (time.perf_counter() - t0) * 1e3
    rp, ci = mesh.pattern.host()
    # the oracle's pattern and slots (pinned bit-exact to the reference's
    # PathIndexBuilder and loc by the CPU tests)
    orp, oci = oracle.pattern(n, ep, 2)
    pattern_exact = bool(np.array_equal(rp, orp) and np.array_equal(ci, oci))
    slots_exact = bool(np.array_equal(mesh.pattern.slots.cpu().numpy().view(np.uint32),
                                      oracle.slots(ep, 2, orp, oci)))
    d = ctx.device
    x = torch.tensor(L["x"], device=d)
    v = torch.zeros(n * 3, dtype=torch.float64, device=d)
    xo, vo = L["x"].copy(), np.zeros(n * 3)
    asm_ms, cg_ms, iters, vals_err = [], [], [], 0.0
    for _ in range(steps):
        torch.cuda.synchronize()
        ms, (vals, f) = _ev_ms(ctx.torch_stream, lambda: assemble_springs(
            mesh, x, v, m, L["fixed"], k, L["l0"], h, 0.0, grav, form=0))
        asm_ms.append(ms)
        oA, of = oracle.springs_assemble(0, xo, vo, m, L["fixed"], ep, k, L["l0"], h, 0.0, grav,
                                         orp, oci)
        vals_err = max(vals_err, float(np.abs(vals.cpu().numpy() - oA).max() /
                                       np.abs(oA).max()))
        S = Solver(ctx, n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, vals, mesh.nnzb,
                   solve_opts(precision=_lib.SOLVE_F64, precond=_lib.PRECOND_NONE, tol=1e-8,
                              maxiters=10000))
        ms, r = _ev_ms(ctx.torch_stream, lambda: S.solve(f, v))
        S.close()
        cg_ms.append(ms)
        iters.append(r.iters)
        with ctx.stream():
            x.add_(h * v)
        t0 = time.perf_counter()
        bb = float(of @ of)
        it = oracle.cg_normr2(n, 3, orp, oci, oA, of, vo, 1e-16 * bb, 10000)
        vo = it[0] if isinstance(it, tuple) else vo
        xo = xo + h * vo
    xg = x.cpu().numpy()
    # the CPU oracle step (1 core), assembly + CG, for the baseline column
    t0 = time.perf_counter()
    xc, vc = L["x"].copy(), np.zeros(n * 3)
    for _ in range(steps):
        oracle.springs_step(0, xc, vc, m, L["fixed"], ep, k, L["l0"], h, 0.0, grav, orp, oci,
                            1e-16, 10000)  # r.r <= 1e-16
    cpu_step_ms = (time.perf_counter() - t0) * 1e3 / steps
    return {
        "workload": "springs createBox 10^3 (1000 vertices, 2700 springs, nnzb %d), 10 implicit "
                    "steps, FP64, CG to 1e-8" % mesh.nnzb,
        "pattern_ms": pattern_ms, "assembly_ms_median": float(np.median(asm_ms)),
        "cg_ms_median": float(np.median(cg_ms)), "cg_iters": iters,
        "parity": {"pattern_bit_exact_vs_oracle": pattern_exact,
                   "slots_bit_exact_vs_oracle": slots_exact,
                   "assembled_values_max_rel_diff": vals_err,
                   "positions_rel_diff_after_10_steps":
                       float(np.linalg.norm(xg - xo) / np.linalg.norm(xo))},
        "cpu_oracle_step_ms": cpu_step_ms, "cpu_cores": 1}


def run_heat(args):
    """P1 heat on the 128^3 lattice (2,146,689 DOF): kappa log-uniform
    [1e-2, 1e2] per tet, T0 uniform [0, 1], dt = 1e-2; A = M + dt K,
    b = M T0.  1,000 scalar SpMVs FP32 vs FP64, then CG to 1e-8: FP64
    Jacobi-CG against the FP32 matrix with FP64 reductions (mixed)."""
    import numpy as np
    import torch
    from simit_gb300 import _lib, meshgen
    from simit_gb300.runtime import (Context, Mesh, Solver, assemble_heat, bspmv, solve_opts,
                                     tet_precompute, tune_spmv)
    size = args.size
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    st = ctx.torch_stream
    mg = meshgen.tet_grid(size)
    nT = len(mg["tets"]) // 4
    g = meshgen.rng(31)
    kappa = 10 ** g.uniform(-2, 2, nT)
    T0 = g.uniform(0, 1, mg["n"])
    if not args.no_reorder:
        mg, vo, eo = _reorder_grid(mg, with_orders=True)
        kappa = kappa[eo]
        T0n = np.empty_like(T0)
        T0n[vo] = T0
        T0 = T0n
    mesh = Mesh(ctx, mg["n"], mg["tets"], 4)
    d = ctx.device
    out = {"workload": "P1 heat %d^3 (%d DOF, nnz %d)" % (size, mg["n"], mesh.nnzb)}
    for name, dt, prec in (("fp64", torch.float64, _lib.SOLVE_F64),
                           ("fp32_matrix", torch.float32, _lib.SOLVE_MIXED)):
        B, W, _ = tet_precompute(mesh, torch.tensor(mg["x"], dtype=dt, device=d), 1.0, dtype=dt)
        kap = torch.tensor(kappa, dtype=dt, device=d)
        T = torch.tensor(T0, dtype=dt, device=d)
        ms_asm, (A, b) = _ev_ms(st, lambda: assemble_heat(mesh, B, W, kap, 1e-2, T, dtype=dt,
                                                          exact=False))
        xv = torch.rand(mesh.n, dtype=dt, device=d)
        y = torch.empty_like(xv)
        # the SpMV schedule picked by the autotuner on this matrix (cached
        # per pattern), timed beside the default one
        tu = tune_spmv(ctx, mesh.n, 1, mesh.pattern.rowptr, mesh.pattern.colidx, A,
                       mesh.nnzb, xdt=dt)
        times = {}
        for g in sorted({0, tu["g"]}):
            bspmv(ctx, mesh.n, 1, mesh.pattern.rowptr, mesh.pattern.colidx, A, xv, y, g)
            times[g], _ = _ev_ms(st, lambda: bspmv(ctx, mesh.n, 1, mesh.pattern.rowptr,
                                                  mesh.pattern.colidx, A, xv, y, g), reps=1000)
        ms_spmv = times[tu["g"]]
        es = A.element_size()
        nbytes = mesh.nnzb * (es + 4) + (mesh.n + 1) * 4 + mesh.n * 2 * es
        S = Solver(ctx, mesh.n, 1, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
                   solve_opts(precision=prec, precond=_lib.PRECOND_JACOBI, tol=1e-8,
                              maxiters=100000, lanes=_lib.LANES_AUTOTUNE))
        b64 = b.double()
        xs = torch.zeros_like(b64)
        ms_solve, r = _ev_ms(st, lambda: S.solve(b64, xs.zero_()))
        S.close()
        out[name] = {"assembly_ms": ms_asm, "spmv_ms": ms_spmv, "spmv_GBps": nbytes / ms_spmv / 1e6,
                     "spmv_frac": nbytes / ms_spmv / 1e6 / peaks()[0],
                     "spmv_schedule": {"tuned_g": tu["g"], "tuned_ms": times[tu["g"]],
                                       "default_ms": times[0]},
                     "spmv_1000_ms": ms_spmv * 1000, "solve_ms": ms_solve, "iters": r.iters,
                     "relres": (r.true_normr2 / r.bnorm2) ** 0.5}
    return out


def run_cloth(args, rank=0, world=1, local=0):
    """256 triangulated sheets (sides U{32..256}), implicit springs, PCG to
    1e-6: one CUDA-graph replay (assembly of all sheets + the persistent
    batched PCG) against the same sheets assembled and solved one at a time
    by the general solver (meshes and solvers built outside the timed
    region).  Under torchrun the sheets are sharded across ranks by
    vertex count (size-balanced, no exchange); times are maxima over ranks."""
    import numpy as np
    import torch
    from simit_gb300 import _lib, problems
    from simit_gb300 import dist as sgd
    from simit_gb300.runtime import (Context, Mesh, Solver, assemble_springs, call, dtype_code,
                                     ptr, solve_opts)
    ctx = Context(local)
    torch.cuda.set_device(local)
    torch.cuda.set_stream(ctx.torch_stream)
    st = ctx.torch_stream
    sides = problems.cloth_sides(args.sheets)
    shard = sgd.shard_by_cost(sides.astype(np.float64) ** 2, world)[rank]
    h = problems.cloth_batch(nsheets=args.sheets, select=shard)
    cb = problems.ClothBatch(ctx, h)
    cb.capture()
    for _ in range(2):
        cb.replay()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        cb.replay()
    e1.record(st)
    e1.synchronize()
    batched_ms = sgd.max_over_ranks(e0.elapsed_time(e1) / args.steps, "cuda")
    ok = sgd.sum_over_ranks(float(not bool((cb.status == 1).all().item())), "cuda") == 0
    iters = cb.iters.cpu().numpy()
    # one at a time
    c = problems.CLOTH
    sp = h["sys_ptr"]
    ep = h["ep"].reshape(-1, 2)
    seq = []
    for s in range(cb.nsys):
        v0, v1 = int(sp[s]), int(sp[s + 1])
        sel = (ep[:, 0] >= v0) & (ep[:, 0] < v1)
        mesh = Mesh(ctx, v1 - v0, (ep[sel] - v0).reshape(-1), 2)
        args_s = [torch.tensor(a, device=ctx.device) for a in (
            h["x"][v0 * 3:v1 * 3].astype(np.float32), np.zeros((v1 - v0) * 3, np.float32),
            np.full(v1 - v0, c["mass"], np.float32), h["fixed"][v0:v1],
            h["k"][sel].astype(np.float32), h["l0"][sel].astype(np.float32))]
        A, f = assemble_springs(mesh, *args_s, c["dt"], c["viscous"], c["grav"], form=0,
                                dtype=torch.float32, exact=False)
        S = Solver(ctx, mesh.n, 3, mesh.pattern.rowptr, mesh.pattern.colidx, A, mesh.nnzb,
                   solve_opts(precision=_lib.SOLVE_MIXED, precond=_lib.PRECOND_BLOCK_JACOBI,
                              tol=c["tol"], maxiters=10000))
        seq.append((mesh, args_s, A, f, f.double(), torch.zeros(mesh.n * 3, dtype=torch.float64,
                                                                  device=ctx.device), S))
    import ctypes
    g3 = (ctypes.c_double * 3)(*c["grav"])

    def one_at_a_time():
        for mesh, a_s, A, f, f64, x, S in seq:
            call("sg_assemble_springs", ctx.h, mesh.ref(), dtype_code(A), 0, *[ptr(t) for t in a_s],
                 c["dt"], c["viscous"], g3, ptr(A), ptr(f), 0)
            S.refresh()
            f64.copy_(f)
            x.zero_()
            S.solve(f64, x)

    one_at_a_time()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    one_at_a_time()
    torch.cuda.synchronize()
    seq_ms = sgd.max_over_ranks((time.perf_counter() - t0) * 1e3, "cuda")
    for item in seq:
        item[-1].close()
    n_all = sgd.sum_over_ranks(h["n"], "cuda")
    if rank != 0:
        return None
    return {"workload": "batched cloth: %d sheets, sides U{32..256}, %d vertices, "
                                  "implicit springs (stretch 5e3, bend 50), PCG to 1e-6"
                                  % (args.sheets, n_all), "n_gpus": world,
                      "scaling": "strong" if world > 1 else None,
                      "batched_graph_ms": batched_ms, "one_at_a_time_ms": seq_ms,
                      "speedup": seq_ms / batched_ms, "all_converged": ok,
                      "iters_max": int(iters.max()), "iters_mean": float(iters.mean()),
                      "autotuned_config": cb.config, "dofs": int(n_all) * 3,
                      "DOF_per_s_batched": n_all * 3 / (batched_ms / 1e3)}


def run_solve_only(args):
    """Profiling driver: the --size heterogeneous-elasticity step as the
    headline runs it (FP32 assembly with the element-blocks plan + flexible
    mixed PCG with the learned preconditioner; --block-jacobi for mixed
    block-Jacobi PCG) with the solver capped at --iters iterations; the
    second step is event-timed."""
    import torch
    from simit_gb300 import _lib, problems
    from simit_gb300 import learned as lrn
    from simit_gb300.runtime import Context
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    h = problems.hetero_mesh(args.size)
    if not args.no_reorder:
        h = problems.reorder_hetero(h)
    if args.block_jacobi:
        p = problems.HeteroElasticity(ctx, h, dtype=torch.float32,
                                      precond=_lib.PRECOND_BLOCK_JACOBI, maxiters=args.iters)
    else:
        with ctx.stream():
            prm = torch.tensor(lrn.load_weights("sym"), device=ctx.device)
        p = problems.HeteroElasticity(ctx, h, dtype=torch.float32,
                                      precond=_lib.PRECOND_LEARNED, learned_params=prm,
                                      maxiters=args.iters)
    p.step()
    ms, r = _ev_ms(ctx.torch_stream, p.step)
    print(json.dumps({"size": args.size, "iters": r.iters, "status": r.status, "step_ms": ms,
                      "kernels": r.kernels}), flush=True)


def run_learned_solve(args):
    """Profiling driver: the --size heterogeneous-elasticity system solved
    with the learned (symmetric form) preconditioner, capped at --iters
    iterations; the second solve is event-timed."""
    import torch
    from simit_gb300 import _lib, problems
    from simit_gb300 import learned as lrn
    from simit_gb300.runtime import Context, Solver, solve_opts
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    h = problems.hetero_mesh(args.size)
    if not args.no_reorder:
        h = problems.reorder_hetero(h)
    p = problems.HeteroElasticity(ctx, h, dtype=torch.float32,
                                  precond=_lib.PRECOND_BLOCK_JACOBI)
    m = p.mesh
    with ctx.stream():
        prm = torch.tensor(lrn.load_weights("sym"), device=ctx.device)
        xs = torch.zeros_like(p.b)
    S = Solver(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, p.A, m.nnzb,
               solve_opts(precision=_lib.SOLVE_MIXED, precond=_lib.PRECOND_LEARNED, tol=1e-8,
                          maxiters=args.iters, learned_params=prm, learned_form=_lib.MPNN_SYM,
                          learned_exec=_lib.MPNN_EXEC_LAYERED if args.layered
                          else _lib.MPNN_EXEC_FOLDED),
               learned_params_keep=prm)

    def one():
        with ctx.stream():
            xs.zero_()
        return S.solve(p.b, xs)
    one()
    ms, r = _ev_ms(ctx.torch_stream, one)
    # one application of the preconditioner alone (sg_mpnn_forward), the
    # same evaluation mode, event-timed over 10 calls
    g = lrn.Graph(ctx, m, p.A, form="sym")
    g.set_exec(_lib.MPNN_EXEC_LAYERED if args.layered else _lib.MPNN_EXEC_FOLDED)
    with ctx.stream():
        rr = torch.rand_like(p.b, dtype=torch.float32)
        zz = torch.empty_like(rr)
    g.forward(prm, rr, zz)
    fwd_ms, _ = _ev_ms(ctx.torch_stream, lambda: g.forward(prm, rr, zz), reps=10)
    print(json.dumps({"size": args.size, "iters": r.iters, "status": r.status, "solve_ms": ms,
                      "ms_per_iter": ms / max(1, r.iters), "apply_ms": fwd_ms,
                      "exec": "layered" if args.layered else "folded"}), flush=True)
    g.close()
    S.close()


def run_assembly_only(args):
    """Profiling driver: the --size heterogeneous-elasticity step's assembly
    (stiffness map in place + force map, FP32) with the element-blocks +
    gather plan, the coloured plan and the row owners, each event-timed over
    --reps calls; also each plan's set-up time."""
    import torch
    from simit_gb300 import _lib, problems
    from simit_gb300.runtime import Context
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    h = problems.hetero_mesh(args.size)
    if not args.no_reorder:
        h = problems.reorder_hetero(h)
    out = {"size": args.size}
    for name, plan in (("gather", "gather"), ("colored", "colored"), ("row_owner", None)):
        p = problems.HeteroElasticity(ctx, h, dtype=torch.float32,
                                      precond=_lib.PRECOND_BLOCK_JACOBI, plan=plan)
        if plan is not None:
            ctx.sync()
            t0 = time.perf_counter()
            p.mesh.color_plan() if plan == "colored" else p.mesh.gather_plan()
            ctx.sync()
            out[name + "_plan_s"] = time.perf_counter() - t0
            if plan == "colored":
                out["ncolors"] = p.mesh.ncolors
        p.assemble_in_place()
        ms, _ = _ev_ms(ctx.torch_stream, p.assemble_in_place, reps=args.reps)
        out[name + "_ms"] = ms
        out[name + "_tets_per_s"] = p.mesh.nE / (ms / 1e3)
        p.close()
        del p
        torch.cuda.empty_cache()
    print(json.dumps(out), flush=True)


def run_spmv_only(args):
    """Profiling driver: the --size heterogeneous-elasticity matrix, --reps
    SpMV launches with sg_bspmv(g = --lanes), event-timed."""
    import torch
    from simit_gb300 import _lib, problems
    from simit_gb300.runtime import Context, bspmv, bsr_add_diag
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    dt = torch.float64 if args.f64 else torch.float32
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if args.scalar:
        # the P1 heat matrix of the same lattice (one value per pattern entry)
        import numpy as np
        from simit_gb300 import meshgen
        from simit_gb300.runtime import Mesh, assemble_heat, tet_precompute
        mg = meshgen.tet_grid(args.size)
        g = meshgen.rng(31)
        kappa = 10 ** g.uniform(-2, 2, len(mg["tets"]) // 4)
        if not args.no_reorder:
            mg, vo, eo = _reorder_grid(mg, with_orders=True)
            kappa = kappa[eo]
        m = Mesh(ctx, mg["n"], mg["tets"], 4)
        d = ctx.device
        B, W, _ = tet_precompute(m, torch.tensor(mg["x"], dtype=dt, device=d), 1.0, dtype=dt)
        A, _ = assemble_heat(m, B, W, torch.tensor(kappa, dtype=dt, device=d), 1e-2,
                             torch.zeros(m.n, dtype=dt, device=d), dtype=dt, exact=False)
        x = torch.rand(m.n, dtype=dt, device=d)
        y = torch.empty_like(x)
        s = x.element_size()
        spmv = lambda: bspmv(ctx, m.n, 1, m.pattern.rowptr, m.pattern.colidx, A, x, y,  # noqa
                             g=args.lanes)
        nbytes = m.nnzb * (s + 4) + (m.n + 1) * 4 + m.n * 2 * s
        spmv()
        e0.record(ctx.torch_stream)
        for _ in range(args.reps):
            spmv()
        e1.record(ctx.torch_stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.reps
        print(json.dumps({"size": args.size, "scalar": True, "lanes": args.lanes,
                          "dtype": str(dt), "nnz": m.nnzb, "ms": ms, "GBps": nbytes / ms / 1e6,
                          "bytes": nbytes}), flush=True)
        return
    h = problems.hetero_mesh(args.size)
    if not args.no_reorder:
        h = problems.reorder_hetero(h)
    p = problems.HeteroElasticity(ctx, h, dtype=dt, precond=_lib.PRECOND_JACOBI)
    m = p.mesh
    x = torch.rand(m.n * 3, dtype=dt, device=ctx.device)
    y = torch.empty_like(x)
    s = x.element_size()
    if args.sym:  # the symmetric-storage kernel (k_sbsr3_wtma)
        from simit_gb300.runtime import SymBsr
        sb = SymBsr(ctx, m.n, m.pattern.rowptr, m.pattern.colidx, m.nnzb, stages=args.stages)
        sb.fill(p.A)
        spmv = lambda: sb.spmv(x, y)  # noqa: E731
        nl = (m.nnzb - m.n) // 2
        nbytes = (m.nnzb - nl) * (9 * s + 4) + nl * 8 + 2 * (m.n + 1) * 4 + m.n * 3 * 2 * s
    else:
        spmv = lambda: bspmv(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, p.A, x, y,  # noqa
                             g=args.lanes)
        nbytes = m.nnzb * (9 * s + 4) + (m.n + 1) * 4 + m.n * 3 * 2 * s
    tuned = None
    if args.tune_spmv:
        from simit_gb300.runtime import tune_spmv
        tuned = tune_spmv(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, p.A, m.nnzb, xdt=dt)
    spmv()
    e0.record(ctx.torch_stream)
    for _ in range(args.reps):
        spmv()
    e1.record(ctx.torch_stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.reps
    # the matrix expression MD + K (sg_bsr_add_diag) on the same pattern:
    # K read and the result written once, D and the row pointers once
    D = torch.rand(m.n * 9, dtype=dt, device=ctx.device)
    out = torch.empty_like(p.A)
    bsr_add_diag(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, p.A, diag=D, out=out)
    e0.record(ctx.torch_stream)
    for _ in range(args.reps):
        bsr_add_diag(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, p.A, diag=D, out=out)
    e1.record(ctx.torch_stream)
    e1.synchronize()
    ctx.sync()
    ad_ms = e0.elapsed_time(e1) / args.reps
    ad_bytes = m.nnzb * 2 * 9 * s + (m.n + 1) * 4 + m.n * 9 * s
    print(json.dumps({"size": args.size, "lanes": args.lanes, "sym": args.sym,
                      "stages": args.stages, "dtype": str(dt),
                      "nnzb": m.nnzb, "ms": ms, "GBps": nbytes / ms / 1e6, "bytes": nbytes,
                      "add_diag_ms": ad_ms, "add_diag_GBps": ad_bytes / ad_ms / 1e6,
                      "add_diag_bytes": ad_bytes, "tuned": tuned}), flush=True)


def workload_name(size, reorder=True):
    return ("heterogeneous linear elasticity %d^3 five-tet lattice (fem_linear form, E log-uniform "
            "[1e3,1e6], nu U[0.35,0.45], bottom face fixed)%s, solve to 1e-8 FP64 relative "
            "residual" % (size, ", vertices in Morton order, elements sorted (simit::reorder with a "
                              "Z-curve)" if reorder else ""))


def dist_setup(args):
    from simit_gb300 import dist as sgd
    rank, world, local = sgd.env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return rank, world, local


# ---------------------------------------------------------------------------
# CPU reference arm (the oracle restatement of the reference's lowered loops)
# ---------------------------------------------------------------------------
# Iterations of plain FP64 Jacobi-PCG to a 1e-8 relative residual on the
# 128^3 workload (Morton order), as the GPU arm's FP64 run counts them; the
# CPU time per step is extrapolated with it (the CPU sample times the
# assembly and a few iterations: the full solve takes about half an hour on
# one core).
FP64_JACOBI_ITERS = {128: 3195}


def cpu_host():
    """nproc and the CPU model of this host."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                k = ln.split(":")[0].strip().lower()
                if k in ("model name", "cpu model", "hardware"):
                    model = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
            for ln in out.splitlines():
                if ln.lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"nproc": os.cpu_count(), "cpu_model": model}


def cpu_config_sample(size, reorder=True, kmax=4):
    """The oracle (one thread) on the size^3 workload itself: pattern
    (ordered sets, as the reference's PathIndexBuilder; its init, untimed in
    the step), FP64 assembly of the step (precompute + stiffness + force, in
    element order with the loc slot search), and Jacobi-PCG iterations, the
    per-iteration time from 1 and kmax iterations (the set-up cancels)."""
    import numpy as np
    from oracle import oracle
    from simit_gb300 import problems
    oracle.build()
    h = problems.hetero_mesh(size)
    if reorder:
        h = problems.reorder_hetero(h)
    t0 = time.perf_counter()
    rp, ci = oracle.pattern(h["n"], h["tets"], 4)
    t_pattern = time.perf_counter() - t0
    t0 = time.perf_counter()
    B, W, _ = oracle.tet_precompute(h["X0"], h["tets"], problems.RHO)
    A = oracle.tet_stiffness(0, h["x"], h["c"], h["tets"], B, W, h["mu"], h["lam"], problems.H,
                             problems.RHO, rp, ci)
    b = oracle.tet_force(0, h["x"], np.zeros(h["n"] * 3), h["c"], h["tets"], B, W, h["mu"],
                         h["lam"], problems.H, problems.RHO, problems.GRAV)
    t_asm = time.perf_counter() - t0
    x0 = np.zeros(h["n"] * 3)
    ts = {}
    for k in (1, kmax):
        t0 = time.perf_counter()
        oracle.jacobi_pcg(h["n"], 3, rp, ci, A, b, x0, 1e-8, k, refresh=0)
        ts[k] = time.perf_counter() - t0
    return {"dofs": h["n"] * 3, "pattern_s": t_pattern, "assembly_s": t_asm,
            "iter_s": (ts[kmax] - ts[1]) / (kmax - 1), "kmax": kmax}


def cpu_solution(ncell, tol=1e-12):
    """The oracle's FP64 Jacobi-PCG solution of the ncell^3 workload (lattice
    order) to tol: the reference solution the GPU solutions are compared to."""
    import numpy as np
    from oracle import oracle
    from simit_gb300 import problems
    oracle.build()
    h = problems.hetero_mesh(ncell)
    rp, ci = oracle.pattern(h["n"], h["tets"], 4)
    B, W, _ = oracle.tet_precompute(h["X0"], h["tets"], problems.RHO)
    A = oracle.tet_stiffness(0, h["x"], h["c"], h["tets"], B, W, h["mu"], h["lam"], problems.H,
                             problems.RHO, rp, ci)
    b = oracle.tet_force(0, h["x"], np.zeros(h["n"] * 3), h["c"], h["tets"], B, W, h["mu"],
                         h["lam"], problems.H, problems.RHO, problems.GRAV)
    x, it, rr = oracle.jacobi_pcg(h["n"], 3, rp, ci, A, b, np.zeros(h["n"] * 3), tol, 400000,
                                  refresh=0)
    return {"x": x, "iters": it, "relres": rr}


def _cpu_child(q, size, reorder, sol_cells):
    """Spawned before the GPU arm touches the GPU: the CPU work of the bench
    line, run beside the GPU measurements (one core each)."""
    try:
        out = {"config": cpu_config_sample(size, reorder)}
        out["solution"] = cpu_solution(sol_cells)
        q.put(out)
    except Exception as e:  # reported, not fatal for the GPU arm
        q.put({"error": repr(e)})


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle's restatement of its lowered
    loops; its own CPU backend needs LLVM and cannot be built) on the
    workload itself, one thread: the pattern once (init), the FP64 assembly
    once, and per step a bounded sample of Jacobi-PCG iterations; the step
    time is assembly + the FP64 iteration count x the time per iteration."""
    if rank != 0:
        return
    from oracle import oracle
    import numpy as np
    from simit_gb300 import problems
    oracle.build()
    iters = FP64_JACOBI_ITERS.get(args.size)
    h = problems.hetero_mesh(args.size)
    if not args.no_reorder:
        h = problems.reorder_hetero(h)
    rp, ci = oracle.pattern(h["n"], h["tets"], 4)
    t0 = time.perf_counter()
    B, W, _ = oracle.tet_precompute(h["X0"], h["tets"], problems.RHO)
    A = oracle.tet_stiffness(0, h["x"], h["c"], h["tets"], B, W, h["mu"], h["lam"], problems.H,
                             problems.RHO, rp, ci)
    b = oracle.tet_force(0, h["x"], np.zeros(h["n"] * 3), h["c"], h["tets"], B, W, h["mu"],
                         h["lam"], problems.H, problems.RHO, problems.GRAV)
    t_asm = time.perf_counter() - t0
    x0 = np.zeros(h["n"] * 3)

    def sample():
        ts = []
        for k in (1, 4):
            t1 = time.perf_counter()
            oracle.jacobi_pcg(h["n"], 3, rp, ci, A, b, x0, 1e-8, k, refresh=0)
            ts.append(time.perf_counter() - t1)
        return (ts[1] - ts[0]) / 3
    for _ in range(args.warmup):
        sample()
    per = [sample() for _ in range(args.steps)]
    t_iter = statistics.median(per)
    dofs = h["n"] * 3
    if iters is None:  # no recorded count: the sample's own iterations only
        step_s = t_asm + t_iter
        note = "no FP64 iteration count recorded for this size: assembly + one iteration"
    else:
        step_s = t_asm + iters * t_iter
        note = ("assembly %.2f s + %d FP64 Jacobi-PCG iterations (the GPU arm's FP64 count) x "
                "%.4f s per iteration (median of %d samples of 1 and 4 iterations)"
                % (t_asm, iters, t_iter, args.steps))
    v = dofs / step_s
    host = cpu_host()
    sample_txt = ("the %d^3 workload itself (%d DOF), oracle restatement of the reference's CPU "
                  "loops, 1 thread: %s" % (args.size, dofs, note))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "DOF/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded Philox)",
           "config": {"workload": workload_name(args.size, not args.no_reorder), "dofs": dofs,
                      "method": "FP64 assembly + plain FP64 Jacobi-PCG (the reference's CPU "
                                "loops, restated)", "extrapolated": iters is not None},
           "cpu_baseline": {"value": v, "unit": "DOF/s", "cores": 1, "kind": "port",
                            "sample": sample_txt, **host},
           "e2e": {"value": v, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "assembly_s": t_asm, "iter_s": t_iter, "iters": iters}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index),
                                       "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for ln in self.p.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def spmv_bytes_f64(mesh):
    """Algorithmic bytes of one FP64 3x3 SpMV: blocks and columns, row
    pointers, x read and y written."""
    return mesh.nnzb * (72 + 4) + (mesh.n + 1) * 4 + mesh.n * 3 * 16


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def horner_traffic(size):
    """DRAM bytes per Horner-pass launch from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "horner_pass_bfp_128cube_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get("bytes_per_launch", {}).get(str(size))


def horner_roofline(ctx, mesh, A, prm, st, reps=50):
    """Event-timed Horner pass of the learned preconditioner (the kernel with
    the largest share of the step: six launches per iteration) on the
    step's own matrix: a folded FP16 graph, one forward to fill its
    buffers, then `reps` launches of step 4.  Algorithmic bytes per pass:
    each pattern entry's column and FP16 weight once (6 B), each vertex's
    slice-row index (4 B), its gathered vector, its own x and the written
    sum once each (block floating point, 8 B each)."""
    import torch
    from simit_gb300 import _lib
    from simit_gb300 import learned as lrn
    g = lrn.Graph(ctx, mesh, A, form="sym")
    g.set_exec(_lib.MPNN_EXEC_FOLDED)
    n3 = mesh.n * 3
    with ctx.stream():
        r = torch.rand(n3, dtype=torch.float32, device=ctx.device)
        z = torch.empty_like(r)
    g.forward(prm, r, z)
    for _ in range(3):
        g.fold_step(4)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        g.fold_step(4)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = mesh.nnzb * 6 + mesh.n * (4 + 8 + 8 + 8)
    g.close()
    return ms, nbytes


def spmv_traffic(size, sym=False):
    """DRAM bytes per SpMV launch from a committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "spmv_sbsr3_wtma_f32_traffic.json" if sym
                     else "spmv_bsr3_wtma_f32_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get("bytes_per_launch_scaled", {}).get(str(size))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def _step_timing(prob, st, steps, warmup, barrier):
    """Event-timed steps (assembly + refresh + solve) of a problem."""
    import torch
    for _ in range(warmup):
        prob.step()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    results = [prob.step() for _ in range(steps)]
    e1.record(st)
    barrier()
    return e0.elapsed_time(e1) / steps, results


def _tuned_summary(t):
    """The autotuners' choices for the bench line."""
    if not t:
        return None
    a, sp = t["assembly"], t["spmv"]
    return {"spmv": {"g": sp["g"], "ms": sp["ms"], "default_ms": sp["default_ms"],
                     "meaning": "g < 0: TMA variant -g-1 of sg_bspmv's table; g > 0: lanes "
                                "per block row of the streaming kernel; 0: default"},
            "assembly": {"plan": a["plan"], "tile": a["tile"], "ms": a["ms"],
                         "default_ms": a["default_ms"], "times": a["times"]}}


def run_ours(args, rank, world, local):
    # the CPU half of the line runs in a process spawned before any GPU call
    cpu_q = cpu_p = None
    if rank == 0 and not args.no_cpu:
        import multiprocessing as mp
        mpc = mp.get_context("spawn")
        cpu_q = mpc.Queue()
        cpu_p = mpc.Process(target=_cpu_child,
                            args=(cpu_q, args.size, not args.no_reorder, args.cpu_sample),
                            daemon=True)
        cpu_p.start()
    import numpy as np
    import torch
    from simit_gb300 import _lib, problems
    from simit_gb300 import learned as lrn
    from simit_gb300.runtime import Context, Solver, bspmv, solve_opts

    ctx = Context(local)
    torch.cuda.set_device(local)
    torch.cuda.set_stream(ctx.torch_stream)
    host = problems.hetero_mesh(args.size)
    if not args.no_reorder:
        host = problems.reorder_hetero(host)
    with ctx.stream():
        prm = torch.tensor(lrn.load_weights("sym"), device=ctx.device)
    # the metric's method: FP32 assembly + learned-preconditioned mixed PCG
    # tune: the assembly plan / element tile and the SpMV schedule from
    # timings on this mesh (set-up, outside the timed steps)
    prob = problems.HeteroElasticity(ctx, host, dtype=torch.float32,
                                     precond=_lib.PRECOND_LEARNED, learned_params=prm,
                                     storage=_lib.STORAGE_SYMMETRIC if args.sym
                                     else _lib.STORAGE_FULL, pdl=int(args.pdl),
                                     tune=not args.no_tune,
                                     reliable_delta=args.reliable_delta)
    st = ctx.torch_stream

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        res = prob.step()
    barrier()
    clocks = Clocks(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    results = []
    for _ in range(args.steps):
        results.append(prob.step())
    e1.record(st)
    barrier()
    clk = clocks.stop()
    from simit_gb300 import dist as sgd
    ms = sgd.max_over_ranks(e0.elapsed_time(e1) / args.steps, "cuda")
    dofs = prob.dofs
    value = dofs * world / (ms / 1e3)
    relres = max((r.true_normr2 / r.bnorm2) ** 0.5 for r in results)
    iters = results[-1].iters
    # kernels per step: stiffness + force assembly (the gather plan: element
    # blocks, slot gather; element vectors, vertex gather), the solver's
    # refresh and its own count (graph kernel nodes included)
    launches = sum(int(r.kernels) + 4 + 6 for r in results)

    # --- end to end through host buffers (pinned) -------------------------
    n3 = prob.dofs
    x_h = torch.tensor(host["x"], dtype=torch.float32).pin_memory()
    mu_h = torch.tensor(host["mu"], dtype=torch.float32).pin_memory()
    lam_h = torch.tensor(host["lam"], dtype=torch.float32).pin_memory()
    u_h = torch.empty(n3, dtype=torch.float64).pin_memory()
    prob.step_host(x_h, mu_h, lam_h, u_h)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        prob.step_host(x_h, mu_h, lam_h, u_h)
    barrier()
    e2e_s = sgd.max_over_ranks((time.perf_counter() - t0) / args.steps, "cuda")
    h2d = (x_h.numel() + mu_h.numel() + lam_h.numel()) * 4
    d2h = u_h.numel() * 8

    # --- the iteration's FP32 SpMV, event-timed ---------------------------
    m = prob.mesh
    p = torch.rand(n3, dtype=torch.float32, device=ctx.device)
    q = torch.empty_like(p)
    sym = prob.opts.storage == _lib.STORAGE_SYMMETRIC
    full_fn = lambda: bspmv(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, prob.A, p, q, g=0)  # noqa: E731
    full_bytes = m.nnzb * (9 * 4 + 4) + (m.n + 1) * 4 + m.n * 3 * (4 + 4)
    if sym:
        from simit_gb300.runtime import SymBsr
        sb = SymBsr(ctx, m.n, m.pattern.rowptr, m.pattern.colidx, m.nnzb)
        sb.fill(prob.A)
        nl = (m.nnzb - m.n) // 2
        nu = m.nnzb - nl
        fn = lambda: sb.spmv(p, q)  # noqa: E731
        spmv_bytes = nu * (9 * 4 + 4) + nl * 8 + 2 * (m.n + 1) * 4 + m.n * 3 * (4 + 4)
        kernel = ("k_sbsr3_wtma (FP32 3x3 blocked SpMV on symmetric storage: upper blocks "
                  "and the lower-block index streamed by per-warp TMA pipelines)")
    else:
        fn, spmv_bytes = full_fn, full_bytes
        kernel = "k_bsr3_wtma (FP32 3x3 blocked SpMV, per-warp TMA pipeline)"
    reps = 50
    spmv_ms = full_ms = None
    for which in ("kernel", "full"):
        f = fn if which == "kernel" else full_fn
        for _ in range(3):
            f()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(st)
        for _ in range(reps):
            f()
        s1.record(st)
        s1.synchronize()
        if which == "kernel":
            spmv_ms = s0.elapsed_time(s1) / reps
        else:
            full_ms = s0.elapsed_time(s1) / reps
    ctx.sync()
    spmv_gbs = spmv_bytes / (spmv_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    # --- roofline of the dominant kernel: the learned preconditioner's
    # Horner pass (six launches per iteration, the largest share of the step)
    horner_ms, horner_bytes = horner_roofline(ctx, m, prob.A, prm, st)
    achieved = horner_bytes / (horner_ms / 1e3) / 1e9

    # --- the step's assembly alone (stiffness map in place + force map) ----
    # algorithmic bytes: element ids and parameters (B 9, W, mu, lam) once,
    # vertex positions once, the matrix values and the force written once;
    # the gather plan also writes and reads its element blocks and vectors
    # and reads the inverse slot map (implementation bytes)
    nE = m.nE
    for _ in range(2):
        prob.assemble_in_place()
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record(st)
    for _ in range(3):
        prob.assemble_in_place()
    a1.record(st)
    a1.synchronize()
    asm_ms = a0.elapsed_time(a1) / 3
    asm_bytes = nE * (4 * 4 + 12 * 4) + m.n * 3 * 4 + m.nnzb * 36 + m.n * 3 * 4
    impl_bytes = asm_bytes + 2 * nE * 16 * 36 + nE * 16 * 4 + (m.nnzb + 1) * 4 + 2 * nE * 4 * 12
    assembly = {"ms": asm_ms, "elements_per_s": nE / (asm_ms / 1e3),
                "algorithmic_bytes": asm_bytes, "GBps": asm_bytes / (asm_ms / 1e3) / 1e9,
                "implementation_bytes": impl_bytes,
                "implementation_GBps": impl_bytes / (asm_ms / 1e3) / 1e9,
                "plan": m.plan, "tile": int(m.s.asm_tile) or 256,
                "kernels": {"gather": "element-blocks plan: k_elem_blocks<LinTetElem> + "
                                      "k_slot_gather (stiffness), k_elem_blocks<TetForceElem> "
                                      "+ k_vert_gather (force)",
                            "colored": "coloured plan: k_colored<LinTetElem>, "
                                       "k_colored<TetForceElem> per colour",
                            None: "row owners: k_rows<LinTetElem>, k_rows<TetForceElem>"}[m.plan]}
    if not args.no_jit:
        assembly["jit_stiffness"] = time_jit_stiffness(ctx, prob)

    # --- the same step with block Jacobi (the method without the network) --
    bj = None
    if not args.no_block_jacobi:
        pb = problems.HeteroElasticity(ctx, host, dtype=torch.float32,
                                       precond=_lib.PRECOND_BLOCK_JACOBI)
        bms, bres = _step_timing(pb, st, max(2, args.steps // 4), 2, barrier)
        bj = {"ms": bms, "DOF_per_s": dofs / (bms / 1e3), "iters": bres[-1].iters,
              "relres": (bres[-1].true_normr2 / bres[-1].bnorm2) ** 0.5,
              "method": "FP32 assembly + mixed-precision block-Jacobi PCG"}
        pb.close()
        del pb
        torch.cuda.empty_cache()

    # --- plain FP64 Jacobi-CG on the same GPU (FP64 assembly + solve) -----
    fp64 = None
    if not args.no_fp64:
        # the same autotuner as the headline picks its SpMV schedule and
        # assembly plan
        p64 = problems.HeteroElasticity(ctx, host, dtype=torch.float64,
                                        precond=_lib.PRECOND_JACOBI, tune=True)
        ms64, r64s = _step_timing(p64, st, 1, 1, barrier)
        r64 = r64s[-1]
        fp64 = {"ms": ms64, "DOF_per_s": dofs / (ms64 / 1e3), "iters": r64.iters,
                "relres": (r64.true_normr2 / r64.bnorm2) ** 0.5,
                "method": "FP64 assembly + FP64 point-Jacobi CG (FP64 SpMV, FP64 vectors)",
                "tuned": _tuned_summary(p64.tuned)}
        # its SpMV against the FP64 FMA rate (18 flops per 3x3 block): what
        # the FP64 step would take with the SpMV at that bound
        from simit_gb300.runtime import fp64_fma_rate
        s64 = p64.tuned["spmv"]["ms"]
        fma = fp64_fma_rate(ctx)
        nb = p64.mesh.nnzb
        bound_ms = 18.0 * nb / (fma * 1e12) * 1e3
        at_bound = ms64 - r64.iters * max(0.0, s64 - bound_ms)
        fp64["spmv"] = {"ms": s64, "fp64_tflops": 18.0 * nb / (s64 * 1e-3) / 1e12,
                        "fp64_fma_peak_tflops": fma, "frac_fp64_peak": bound_ms / s64,
                        "GBps": spmv_bytes_f64(p64.mesh) / (s64 * 1e-3) / 1e9}
        fp64["step_ms_with_spmv_at_fp64_bound"] = at_bound
        fp64["speedup_if_spmv_at_fp64_bound"] = at_bound / ms
        p64.close()
        del p64
        torch.cuda.empty_cache()

    # --- solutions against the oracle's FP64 solution (cpu_sample^3) -------
    cpu = None
    if cpu_p is not None:
        cpu = cpu_q.get()
        cpu_p.join(timeout=60)
    parity = None
    if cpu is not None and "solution" in cpu:
        hs = problems.hetero_mesh(args.cpu_sample)
        xo = np.asarray(cpu["solution"]["x"])
        parity = {"cells": args.cpu_sample, "dofs": int(len(xo)),
                  "oracle": "FP64 Jacobi-PCG to a %.0e relative residual (%d iterations)"
                            % (1e-12, cpu["solution"]["iters"])}
        cases = [("learned_mixed", _lib.PRECOND_LEARNED, torch.float32),
                 ("block_jacobi_mixed", _lib.PRECOND_BLOCK_JACOBI, torch.float32),
                 ("fp64_jacobi", _lib.PRECOND_JACOBI, torch.float64)]
        for name, pc, dt in cases:
            ps = problems.HeteroElasticity(ctx, hs, dtype=dt, precond=pc,
                                           learned_params=prm if pc == _lib.PRECOND_LEARNED
                                           else None)
            r = ps.step()
            u = ps.u.cpu().numpy()
            parity[name] = {"relerr": float(np.linalg.norm(u - xo) / np.linalg.norm(xo)),
                            "relres": (r.true_normr2 / r.bnorm2) ** 0.5, "iters": r.iters}
            ps.close()
    if rank != 0:
        return
    host_cpu = cpu_host()
    cpu_base = None
    if cpu is not None and "config" in cpu:
        c = cpu["config"]
        it = fp64["iters"] if fp64 else FP64_JACOBI_ITERS.get(args.size, 0)
        step_s = c["assembly_s"] + it * c["iter_s"]
        cpu_base = {"value": c["dofs"] / step_s, "unit": "DOF/s", "cores": 1, "kind": "port",
                    "sample": "the %d^3 workload itself (%d DOF), oracle restatement of the "
                              "reference's CPU loops, 1 thread: FP64 assembly %.2f s + %d FP64 "
                              "Jacobi-PCG iterations (this run's FP64 count) x %.4f s per "
                              "iteration (timed over 1 and %d iterations); pattern %.2f s "
                              "(init, not in the step)"
                              % (args.size, c["dofs"], c["assembly_s"], it, c["iter_s"],
                                 c["kmax"], c["pattern_s"]), **host_cpu}
    elif cpu is not None:
        cpu_base = {"value": None, "unit": "DOF/s", "cores": 1, "kind": "port",
                    "sample": "failed: " + cpu.get("error", "?"), **host_cpu}
    out = {
        "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 matrix+SpMV+network, f64 dots/residual",
        "data": "synthetic (seeded Philox mesh, parameters and displacements)",
        "config": {"workload": workload_name(args.size, not args.no_reorder), "dofs": dofs,
                   "nnzb": m.nnzb,
                   "method": "FP32 assembly (element-blocks plan) + learned-preconditioned "
                             "flexible mixed-precision PCG (symmetric form of the 3-layer "
                             "hidden-64 message-passing network, evaluated as its degree-6 "
                             "matrix polynomial; FP32 matrix/vectors, FP64 dots, FP64 reliable "
                             "updates; block-Jacobi fallback), verified FP64 residual"
                             + ("; the iteration's SpMV on symmetric storage" if sym else ""),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (FP32 matrix 1.0 GB), no flush"},
        "iters": iters, "checks": int(results[-1].checks),
        "fallbacks": int(results[-1].fallbacks), "relres_max": relres,
        "learned_dof_per_s": value,
        "e2e": {"value": dofs * world / e2e_s, "unit": "DOF/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": horner_traffic(args.size),
                     "kernel": "k_horner<__half> (one Horner step of the learned "
                               "preconditioner: sliced-ELLPACK gather, FP16 weights, "
                               "block-floating-point vectors; 6 launches per iteration)",
                     "peak_kind": peak_kind, "ms_per_launch": horner_ms,
                     "algorithmic_bytes": horner_bytes},
        "spmv": {"kernel": kernel, "ms_per_launch": spmv_ms, "algorithmic_bytes": spmv_bytes,
                 "GBps": spmv_gbs, "frac": spmv_gbs / peak,
                 "traffic": spmv_traffic(args.size, sym),
                 "full_storage_spmv": {"ms_per_launch": full_ms,
                                       "algorithmic_bytes": full_bytes,
                                       "GBps": full_bytes / (full_ms / 1e3) / 1e9}},
        "cpu_baseline": cpu_base,
        "clocks": clk,
        "assembly": assembly,
        "block_jacobi_mixed": bj,
        "fp64_jacobi_cg": fp64,
        "speedup_vs_fp64_cg": (fp64["ms"] / ms) if fp64 else None,
        "target_3x_fp64_cg_met": (fp64["ms"] / ms >= 3.0) if fp64 else None,
        "learned_vs_block_jacobi": ({"iteration_gain": bj["iters"] / max(1, iters),
                                     "time_ratio": bj["ms"] / ms} if bj else None),
        "solution_relerr_vs_fp64_oracle": parity,
        "tuned": _tuned_summary(prob.tuned),
    }
    if rank == 0 and world == 1 and not args.no_secondary:
        out["secondary"] = run_secondary(args)
    print(json.dumps(out), flush=True)


def run_secondary(args):
    """The other workloads of the path, measured after the headline and
    outside its timed region, each in its own process (`bench.py --heat`,
    `--neo`, `--springs`, `--cloth`): P1 heat 128^3 (SpMVs and CG), one
    neo-Hookean Newton step at 64^3, the springs createBox 10^3 steps and the
    batched cloth sheets.  Each entry carries its wall time and exit code; a
    run that fails records its error instead of its numbers."""
    out = {}
    for name, extra in (("heat", ["--size", "128"]), ("neo", ["--size", "64"]),
                        ("springs", []), ("cloth", ["--sheets", str(args.sheets)])):
        cmd = [sys.executable, os.path.abspath(__file__), "--" + name,
               "--steps", str(args.steps), "--warmup", str(args.warmup)] + extra
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            res = json.loads(lines[-1]) if lines else {
                "error": (r.stderr or r.stdout)[-400:]}
            res["exit_code"] = r.returncode
        except Exception as e:  # a secondary workload must not cost the headline line
            res = {"error": "%s: %s" % (type(e).__name__, e)}
        res["wall_s"] = time.perf_counter() - t0
        out[name] = res
    return out


def time_jit_stiffness(ctx, prob):
    """The linear-tet stiffness map of the step from its element function
    compiled at run time (sg_jit_assembly_create), timed beside the
    precompiled k_rows<LinTetElem>; both write the same matrix, bit for bit."""
    import torch
    from simit_gb300 import _lib, jit_elements, problems
    from simit_gb300.runtime import JitAssembly, call, dtype_code, ptr
    m, st = prob.mesh, ctx.torch_stream
    t0 = time.perf_counter()
    jit = JitAssembly(ctx, jit_elements.linear_tet(problems.H, problems.RHO), 4, 3,
                      dtype=prob.dtype, exact=False)
    compile_s = time.perf_counter() - t0
    fields = [prob.B, prob.W, prob.mu, prob.lam, prob.c]
    with ctx.stream():
        out = torch.empty_like(prob.A)

    # the precompiled row-owner kernel (the same sg_mesh without its plan)
    import ctypes
    plain = _lib.Mesh.from_buffer_copy(m.s)
    plain.slots = plain.color_order = plain.color_ptr = None
    plain.slot_src_ptr = plain.slot_src = None
    plain.ncolors = 0

    def builtin():
        call("sg_assemble_tet_stiffness", ctx.h, ctypes.byref(plain), dtype_code(prob.A),
             _lib.MODEL_LINEAR,
             ptr(prob.x), ptr(prob.c), ptr(prob.B), ptr(prob.W), ptr(prob.mu), ptr(prob.lam),
             problems.H, problems.RHO, ptr(prob.A), 0)

    res = {"compile_s": compile_s}
    for name, f in (("jit_ms", lambda: jit.assemble(m, fields, out=out)), ("builtin_ms", builtin)):
        for _ in range(2):
            f()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(3):
            f()
        e1.record(st)
        e1.synchronize()
        res[name] = e0.elapsed_time(e1) / 3
    ctx.sync()
    res["bitwise_equal"] = bool(torch.equal(out, prob.A))
    jit.close()
    return res


def main():
    args = parse()
    if args.solve_only:
        run_solve_only(args)
        return
    if args.learned_solve:
        run_learned_solve(args)
        return
    if args.spmv_only:
        run_spmv_only(args)
        return
    if args.assembly_only:
        run_assembly_only(args)
        return
    if args.cloth:
        rank, world, local = dist_setup(args)
        res = run_cloth(args, rank, world, local)
        if res is not None:
            print(json.dumps(res), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    for flag, fn in (("neo", run_neo), ("heat", run_heat), ("springs", run_springs)):
        if getattr(args, flag):
            print(json.dumps(fn(args)), flush=True)
            return
    rank, world, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
