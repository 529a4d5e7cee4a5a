"""Learned preconditioner: data, training and evaluation on the C ABI.

The network (3 message-passing layers, hidden 64, bf16 tensor-core weights,
FP32 accumulation) is defined in simit_gb300/csrc/sg_mpnn.cuh; its forward,
backward, A-norm loss and Adam step are CUDA kernels behind sg_mpnn_*.

Training pairs come from the solver itself: on seeded heterogeneous-elasticity
meshes of 16^3 .. 48^3 cells, for random right-hand sides b, the
mixed-precision block-Jacobi PCG is stopped after k iterations (k in KS); the
pair is (r_k = b - A x_k, e_k = x* - x_k) with x* the converged solution, so
e_k = A^-1 r_k.  The loss is the A-norm error (z - e)'A(z - e) / e'Ae of the
network's output z = M(r) — zero for the exact inverse, one for z = 0.
"""
import ctypes
import os

import numpy as np
import torch

from . import _lib, meshgen, problems
from ._lib import call
from .runtime import Solver, bspmv, dtype_code, ptr, solve_opts

HERE = os.path.dirname(os.path.abspath(__file__))
FORMS = {"relu": _lib.MPNN_RELU, "linear": _lib.MPNN_LINEAR, "sym": _lib.MPNN_SYM}
WEIGHTS = {f: os.path.join(HERE, "data", "mpnn_elasticity_%s.npy" % f) for f in FORMS}
KS = (1, 3, 8, 16, 32, 64, 128, 256, 512, 1024)
H, K = 64, 8
SHAPES = [("W1s", (H, 3)), ("W1m", (H, 3)), ("P2", (K, H)), ("W2h", (H, H)), ("W2m", (H, K)),
          ("P3", (K, H)), ("W3h", (H, H)), ("W3m", (H, K)), ("Wout", (3, H))]


def nparams():
    return _lib.load().sg_mpnn_nparams()


def init_params(seed=0, out_scale=0.0):
    """He-style initial weights; Wout scaled by out_scale (0 = block Jacobi)."""
    rng = meshgen.rng(seed)
    parts = []
    for name, (a, b) in SHAPES:
        w = rng.normal(0, np.sqrt(2.0 / b), size=(a, b))
        if name == "Wout":
            w *= out_scale
        parts.append(w.reshape(-1))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == nparams()
    return p


def load_weights(form="sym"):
    return np.load(WEIGHTS[form]).astype(np.float32)


def _unpack(params):
    out, o = {}, 0
    for name, (a, b) in SHAPES:
        out[name] = np.asarray(params[o:o + a * b], np.float64).reshape(a, b)
        o += a * b
    return out


def _bf16(x):
    """Values rounded to bfloat16 (nearest even), as the tensor-core layers
    and the folding kernel round the 64x64 weights."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def poly_of_params(params):
    """The symmetric form's network as a polynomial in the edge-weight
    aggregation Aw: N = sum_{k=0..3} Aw^k (x) B_k.  Returns B (4 x 3 x 3,
    float64) as the folding kernel forms it (bf16-rounded W2h, W3h):
    q2 = C2 [x; m1], q3 = C3 [x; m1; m2], N x = C4 [x; m1; m2; m3] and
    B_0 = C4x, B_1 = C4m1 + C4m2 C2x + C4m3 C3x,
    B_2 = C4m2 C2m1 + C4m3 (C3m1 + C3m2 C2x), B_3 = C4m3 C3m2 C2m1."""
    p = _unpack(params)
    E1 = np.concatenate([p["W1s"], p["W1m"]], axis=1)
    F2 = np.concatenate([_bf16(p["W2h"]) @ E1, p["W2m"]], axis=1)
    F3 = np.concatenate([_bf16(p["W3h"]) @ F2, p["W3m"]], axis=1)
    C2, C3, C4 = p["P2"] @ E1, p["P3"] @ F2, p["Wout"] @ F3
    C2x, C2m1 = C2[:, 0:3], C2[:, 3:6]
    C3x, C3m1, C3m2 = C3[:, 0:3], C3[:, 3:6], C3[:, 6:14]
    C4x, C4m1, C4m2, C4m3 = C4[:, 0:3], C4[:, 3:6], C4[:, 6:14], C4[:, 14:22]
    return np.stack([C4x,
                     C4m1 + C4m2 @ C2x + C4m3 @ C3x,
                     C4m2 @ C2m1 + C4m3 @ (C3m1 + C3m2 @ C2x),
                     C4m3 @ C3m2 @ C2m1])


def params_of_poly(B):
    """Network weights (FP32[nparams]) whose polynomial is N = sum_k Aw^k (x)
    B_k for given B (4 x 3 x 3).  The hidden layers carry their inputs and
    messages unchanged -- h1 = [x; m1], h2 = [h1; m2], h3 = [h2; m3] through
    0/1 weights, which bf16 holds exactly -- the message maps pass x's first
    aggregation on (q2 = m1, q3 = m2 in their first three channels) and the
    output layer holds the coefficients: Wout's column blocks [x | m1 | m2 |
    m3] = [B_0 | B_1 | B_2 | B_3]."""
    B = np.asarray(B, np.float64).reshape(4, 3, 3)
    p = {name: np.zeros((a, b)) for name, (a, b) in SHAPES}
    for c in range(3):
        p["W1s"][c, c] = 1.0
        p["W1m"][3 + c, c] = 1.0
    for r in range(6):
        p["W2h"][r, r] = 1.0
    for j in range(K):
        p["W2m"][6 + j, j] = 1.0
    for r in range(14):
        p["W3h"][r, r] = 1.0
    for j in range(K):
        p["W3m"][14 + j, j] = 1.0
    for c in range(3):
        p["P2"][c, 3 + c] = 1.0      # q2 = m1 (C2m1 = [I; 0], C2x = 0)
        p["P3"][c, 6 + c] = 1.0      # q3 = m2 (C3m2 = [[I, 0], [0, 0]])
    p["Wout"][:, 0:3] = B[0]
    p["Wout"][:, 3:6] = B[1]
    p["Wout"][:, 6:9] = B[2]
    p["Wout"][:, 14:17] = B[3]
    return np.concatenate([p[name].reshape(-1) for name, _ in SHAPES]).astype(np.float32)


class Graph:
    """sg_mpnn_graph of a 3x3-blocked matrix."""

    def __init__(self, ctx, mesh, A, form="relu"):
        self.ctx = ctx
        self.A = A
        self.m = _lib.Matrix(mesh.n, 3, mesh.nnzb, mesh.pattern.rowptr.data_ptr(),
                             mesh.pattern.colidx.data_ptr(), dtype_code(A), A.data_ptr())
        h = ctypes.c_void_p()
        call("sg_mpnn_graph_create", ctx.h, ctypes.byref(self.m), ctypes.byref(h))
        self.h = h
        self.n = mesh.n
        call("sg_mpnn_graph_set_form", h, FORMS[form])

    def set_exec(self, mode):
        """_lib.MPNN_EXEC_*: how forward() evaluates the symmetric form."""
        call("sg_mpnn_graph_set_exec", self.h, int(mode))

    def fold_step(self, d):
        """One Horner step of the folded evaluation on the graph's own
        buffers (sg_mpnn_fold_step; for timing a pass)."""
        call("sg_mpnn_fold_step", self.h, d)

    def forward(self, params, r, z, train=False):
        call("sg_mpnn_forward", self.h, ptr(params), ptr(r), ptr(z), int(train))

    def backward(self, params, dz, grad):
        call("sg_mpnn_backward", self.h, ptr(params), ptr(dz), ptr(grad))

    def loss(self, z, e, eAe, dz):
        out = ctypes.c_double()
        call("sg_mpnn_loss", self.h, ptr(z), ptr(e), float(eAe), ptr(dz), ctypes.byref(out))
        return out.value

    def close(self):
        if self.h:
            _lib.load().sg_mpnn_graph_destroy(self.h)
            self.h = None


def make_pairs(ctx, ncell, seed, n_rhs, ks=KS):
    """Residual/correction pairs of one seeded mesh (FP32 device tensors)."""
    host = problems.hetero_mesh(ncell, seed=seed)
    prob = problems.HeteroElasticity(ctx, host, dtype=torch.float32,
                                     precond=_lib.PRECOND_BLOCK_JACOBI, tol=1e-11)
    m = prob.mesh
    d = ctx.device
    g = meshgen.rng(seed + 1000)
    cons = torch.tensor(np.repeat(host["c"], 3) > 0, device=d)
    pairs = []
    with ctx.stream():
        for _ in range(n_rhs):
            b = torch.tensor(g.normal(size=m.n * 3), device=d)
            b[cons] = 0.0
            xs = torch.zeros_like(b)
            prob.solver.solve(b, xs)
            for k in ks:
                S = Solver(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, prob.A, m.nnzb,
                           solve_opts(precision=_lib.SOLVE_MIXED,
                                      precond=_lib.PRECOND_BLOCK_JACOBI, tol=1e-14,
                                      maxiters=k, verify=0))
                xk = torch.zeros_like(b)
                S.solve(b, xk)
                S.close()
                e = (xs - xk).float()
                # r_k = b - A x_k with FP64 accumulation (FP32 matrix, FP64
                # x): an FP32 SpMV's rounding would swamp late residuals
                Ax = bspmv(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, prob.A, xk)
                r64 = b - Ax
                rel = float(r64.norm() / b.norm())
                r = r64.float().contiguous()
                Ae = bspmv(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, prob.A, e)
                eAe = float((e.double() * Ae.double()).sum())
                if eAe > 0 and rel > 1e-5:
                    pairs.append((r, e, eAe))
    return prob, pairs


class Trainer:
    def __init__(self, ctx, params=None, lr=1e-3, seed=0):
        self.ctx = ctx
        d = ctx.device
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        with ctx.stream():
            self.params = torch.tensor(p, device=d)
            self.grad = torch.zeros_like(self.params)
            self.m = torch.zeros_like(self.params)
            self.v = torch.zeros_like(self.params)
        self.step_n = 0
        self.lr = lr

    def step(self, graph, r, e, eAe):
        with self.ctx.stream():
            z = torch.empty_like(r)
            dz = torch.empty_like(r)
        graph.forward(self.params, r, z, train=True)
        L = graph.loss(z, e, eAe, dz)
        graph.backward(self.params, dz, self.grad)
        self.step_n += 1
        call("sg_mpnn_adam", self.ctx.h, ptr(self.params), ptr(self.grad), ptr(self.m), ptr(self.v),
             self.step_n, self.lr, 0.9, 0.999, 1e-8)
        return L

    def eval_loss(self, graph, pairs):
        tot = 0.0
        for r, e, eAe in pairs:
            with self.ctx.stream():
                z = torch.empty_like(r)
                dz = torch.empty_like(r)
            graph.forward(self.params, r, z, train=True)
            tot += graph.loss(z, e, eAe, dz)
        return tot / max(1, len(pairs))


class Validator:
    """PCG iterations with the current weights on a held-out mesh (the
    quantity the preconditioner exists to reduce; the training loss is a
    one-step proxy for it)."""

    def __init__(self, ctx, ncell=16, seed=555, form="sym", maxiters=5000):
        host = problems.hetero_mesh(ncell, seed=seed)
        self.ctx = ctx
        self.prob = problems.HeteroElasticity(ctx, host, dtype=torch.float32,
                                              precond=_lib.PRECOND_BLOCK_JACOBI)
        m = self.prob.mesh
        with ctx.stream():
            self.prm = torch.zeros(nparams(), dtype=torch.float32, device=ctx.device)
        self.S = Solver(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, self.prob.A, m.nnzb,
                        solve_opts(precision=_lib.SOLVE_MIXED, precond=_lib.PRECOND_LEARNED,
                                   tol=1e-8, maxiters=maxiters, learned_params=self.prm,
                                   learned_form=FORMS[form]),
                        learned_params_keep=self.prm)

    def iters(self, params):
        with self.ctx.stream():
            self.prm.copy_(params)
            x = torch.zeros_like(self.prob.b)
        r = self.S.solve(self.prob.b, x)
        ok = r.status == 1 and r.fallbacks == 0
        return r.iters if ok else None

    def close(self):
        self.S.close()
        self.prob.close()


def train(ctx, sizes=(16, 24, 32, 40, 48), n_pairs=2000, epochs=6, lr=1e-3, seed=0,
          log=print, form="sym", val_every=100):
    """Train on n_pairs pairs spread over the meshes.  Every val_every steps
    the weights are scored by PCG iterations on a held-out mesh and the best
    scoring weights are kept.  Returns (params, history)."""
    per_mesh = max(1, n_pairs // (len(sizes) * len(KS)))
    data = []
    for i, nc in enumerate(sizes):
        prob, pairs = make_pairs(ctx, nc, seed=100 + i, n_rhs=per_mesh)
        data.append((prob, Graph(ctx, prob.mesh, prob.A, form=form), pairs))
        log("mesh %d^3: %d pairs" % (nc, len(pairs)))
    tr = Trainer(ctx, lr=lr, seed=seed)
    val = Validator(ctx, form=form)
    hist = {"loss": [], "val_iters": []}
    best = (val.iters(tr.params), 0, tr.params.detach().clone())
    hist["val_iters"].append((0, best[0]))
    L0 = np.mean([tr.eval_loss(g, p) for _, g, p in data])
    hist["loss"].append(L0)
    log("epoch 0 loss %.5f val iters %s" % (L0, best[0]))
    rng = meshgen.rng(seed + 7)
    for ep in range(epochs):
        order = [(i, j) for i, (_, _, p) in enumerate(data) for j in range(len(p))]
        rng.shuffle(order)
        for i, j in order:
            prob, g, pairs = data[i]
            r, e, eAe = pairs[j]
            tr.step(g, r, e, eAe)
            if tr.step_n % val_every == 0:
                it = val.iters(tr.params)
                hist["val_iters"].append((tr.step_n, it))
                if it is not None and (best[0] is None or it < best[0]):
                    best = (it, tr.step_n, tr.params.detach().clone())
        L = np.mean([tr.eval_loss(g, p) for _, g, p in data])
        hist["loss"].append(L)
        log("epoch %d loss %.5f best val iters %s (step %d)" % (ep + 1, L, best[0], best[1]))
    hist["best_step"] = best[1]
    params = best[2].cpu().numpy()
    val.close()
    for prob, g, _ in data:
        g.close()
        prob.close()
    return params, hist


class _PcgScore:
    """PCG iterations to tol with the symmetric form's polynomial B on one
    seeded heterogeneous-elasticity mesh (flexible mixed PCG, folded FP16
    evaluation) -- the quantity fit_poly minimises.  A solve that does not
    converge within maxiters or falls back to block Jacobi scores maxiters."""

    def __init__(self, ctx, ncell, seed, tol=1e-8, maxiters=20000):
        host = problems.hetero_mesh(ncell, seed=seed)
        self.ctx = ctx
        self.prob = problems.HeteroElasticity(ctx, host, dtype=torch.float32,
                                              precond=_lib.PRECOND_BLOCK_JACOBI)
        m = self.prob.mesh
        self.maxiters = maxiters
        with ctx.stream():
            self.prm = torch.zeros(nparams(), dtype=torch.float32, device=ctx.device)
            self.x = torch.zeros_like(self.prob.b)
        self.S = Solver(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, self.prob.A, m.nnzb,
                        solve_opts(precision=_lib.SOLVE_MIXED, precond=_lib.PRECOND_LEARNED,
                                   tol=tol, maxiters=maxiters, learned_params=self.prm,
                                   learned_form=_lib.MPNN_SYM,
                                   learned_exec=_lib.MPNN_EXEC_FOLDED),
                        learned_params_keep=self.prm)

    def __call__(self, B):
        with self.ctx.stream():
            self.prm.copy_(torch.from_numpy(params_of_poly(B)))
            self.x.zero_()
        r = self.S.solve(self.prob.b, self.x)
        if r.status != 1 or r.fallbacks:
            return self.maxiters
        return r.iters

    def close(self):
        self.S.close()
        self.prob.close()


def fit_poly(ctx, B0=None, ncell=64, seed=321, generations=40, popsize=12, sigma=0.05,
             rng_seed=0, log=print):
    """Fits the symmetric form's polynomial coefficients B_0..B_3 (36
    numbers; the network is their carrier through params_of_poly) to the
    PCG iteration count on a seeded mesh with CMA-ES (Hansen's
    (mu/mu_w, lambda) evolution strategy with rank-one and rank-mu updates
    of the covariance and cumulative step-size adaptation).  B0: start
    (default: the shipped weights' polynomial).  Returns (B, iterations,
    history)."""
    score = _PcgScore(ctx, ncell, seed)
    m = (poly_of_params(load_weights("sym")) if B0 is None else np.asarray(B0)).reshape(-1)
    n = m.size
    lam = popsize
    mu = lam // 2
    w = np.log(mu + 0.5) - np.log(np.arange(1, mu + 1))
    w /= w.sum()
    mueff = 1.0 / np.sum(w ** 2)
    cc = (4 + mueff / n) / (n + 4 + 2 * mueff / n)
    cs = (mueff + 2) / (n + mueff + 5)
    c1 = 2 / ((n + 1.3) ** 2 + mueff)
    cmu = min(1 - c1, 2 * (mueff - 2 + 1 / mueff) / ((n + 2) ** 2 + mueff))
    damps = 1 + 2 * max(0.0, np.sqrt((mueff - 1) / (n + 1)) - 1) + cs
    chin = np.sqrt(n) * (1 - 1 / (4 * n) + 1 / (21 * n * n))
    pc, ps = np.zeros(n), np.zeros(n)
    Bm, D, C = np.eye(n), np.ones(n), np.eye(n)
    invsqrt = np.eye(n)
    rng = meshgen.rng(rng_seed)
    best = (score(m.reshape(4, 3, 3)), m.copy())
    hist = [best[0]]
    log("start: %d iterations" % best[0])
    for gen in range(generations):
        z = rng.normal(size=(lam, n))
        y = (z * D) @ Bm.T
        xs = m + sigma * y
        f = np.array([score(x.reshape(4, 3, 3)) for x in xs], np.float64)
        order = np.argsort(f, kind="stable")
        if f[order[0]] < best[0]:
            best = (int(f[order[0]]), xs[order[0]].copy())
        ysel = y[order[:mu]]
        yw = w @ ysel
        m = m + sigma * yw
        ps = (1 - cs) * ps + np.sqrt(cs * (2 - cs) * mueff) * (invsqrt @ yw)
        hsig = np.linalg.norm(ps) / np.sqrt(1 - (1 - cs) ** (2 * (gen + 1))) < (1.4 + 2 / (n + 1)) * chin
        pc = (1 - cc) * pc + hsig * np.sqrt(cc * (2 - cc) * mueff) * yw
        C = ((1 - c1 - cmu) * C + c1 * (np.outer(pc, pc) + (1 - hsig) * cc * (2 - cc) * C)
             + cmu * (ysel.T * w) @ ysel)
        sigma *= np.exp((cs / damps) * (np.linalg.norm(ps) / chin - 1))
        C = (C + C.T) / 2
        evals, Bm = np.linalg.eigh(C)
        D = np.sqrt(np.maximum(evals, 1e-20))
        invsqrt = Bm @ np.diag(1 / D) @ Bm.T
        hist.append(int(f[order[0]]))
        log("generation %d: best %d, generation best %d, median %d, sigma %.4f"
            % (gen + 1, best[0], int(f[order[0]]), int(np.median(f)), sigma))
    score.close()
    return best[1].reshape(4, 3, 3), best[0], hist


def compare(ctx, params, ncell, seed=999, tol=1e-8, form="sym", exec_mode=_lib.MPNN_EXEC_FOLDED):
    """Flexible PCG with the network vs block-Jacobi PCG on a held-out mesh.
    exec_mode: how the symmetric form is evaluated (_lib.MPNN_EXEC_*)."""
    host = problems.hetero_mesh(ncell, seed=seed)
    out = {}
    d = ctx.device
    with ctx.stream():
        prm = torch.tensor(np.asarray(params, np.float32), device=d)
    for name, pc in (("block_jacobi", _lib.PRECOND_BLOCK_JACOBI),
                     ("learned", _lib.PRECOND_LEARNED)):
        prob = problems.HeteroElasticity(ctx, host, dtype=torch.float32,
                                         precond=_lib.PRECOND_BLOCK_JACOBI)
        m = prob.mesh
        S = Solver(ctx, m.n, 3, m.pattern.rowptr, m.pattern.colidx, prob.A, m.nnzb,
                   solve_opts(precision=_lib.SOLVE_MIXED, precond=pc, tol=tol, maxiters=100000,
                              learned_params=prm if pc == _lib.PRECOND_LEARNED else None,
                              learned_form=FORMS[form], learned_exec=exec_mode),
                   learned_params_keep=prm)
        x = torch.zeros_like(prob.b)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ctx.torch_stream)
        r = S.solve(prob.b, x)
        e1.record(ctx.torch_stream)
        e1.synchronize()
        out[name] = {"iters": r.iters, "status": r.status, "fallbacks": r.fallbacks,
                     "relres": (r.true_normr2 / r.bnorm2) ** 0.5, "ms": e0.elapsed_time(e1)}
        S.close()
        prob.close()
    return out


def main():
    import argparse
    import json
    import time
    from .runtime import Context
    ap = argparse.ArgumentParser(description="train the learned preconditioner")
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=None, help="weights file (default: the package's)")
    ap.add_argument("--eval-size", type=int, default=32)
    ap.add_argument("--form", default="sym", choices=sorted(FORMS))
    a = ap.parse_args()
    ctx = Context(0)
    torch.cuda.set_stream(ctx.torch_stream)
    t0 = time.time()
    params, hist = train(ctx, n_pairs=a.pairs, epochs=a.epochs, lr=a.lr, form=a.form)
    out = a.out or WEIGHTS[a.form]
    os.makedirs(os.path.dirname(out) or ".", exist_ok=True)
    np.save(out, params)
    res = compare(ctx, params, a.eval_size, form=a.form)
    print(json.dumps({"train_seconds": time.time() - t0, "loss_history": hist,
                      "eval": res, "weights": a.out}))


if __name__ == "__main__":
    main()
