"""ORACLE (test infrastructure): numpy restatement of the message-passing
preconditioner network, forward and backward, used only by tests to check the
GPU kernels (simit_gb300/csrc/sg_mpnn.cu).  The network has no counterpart in
the reference; this file states its definition:

  s_v  = D_v^-1 r_v                       (3x3 block-Jacobi of A)
  m1_v = sum_{u in N(v), u != v} a_vu s_u
  g1_v = W1s s_v + W1m m1_v,  h1 = relu(g1)          (64)
  q2_v = P2 h1_v                                     (8)
  m2_v = sum a_vu q2_u
  g2_v = W2h bf(h1_v) + W2m m2_v,  h2 = relu(g2)     (64)
  q3_v = P3 h2_v
  m3_v = sum a_vu q3_u
  g3_v = W3h bf(h2_v) + W3m m3_v,  h3 = relu(g3)     (64)
  z_v  = s_v + Wout h3_v

with a_vu = ||A_vu||_F / sqrt(||A_vv||_F ||A_uu||_F) for the off-diagonal
blocks of the pattern, bf() rounding to bfloat16 (round to nearest even), and
W2h, W3h rounded to bfloat16 (the tensor-core operands).  No biases: the map
r -> z is positively homogeneous.

Forms: relu (above), linear (identity activations, so z = M r with a fixed
matrix M), and the symmetric factorized form (forward_sym): with the linear
network N (s -> Wout h3), D_v = L_v L_v^T the Cholesky factors of the
diagonal blocks,

  M = L^-T (I + N)^T (I + N) L^-1,

symmetric positive definite by construction and equal to block Jacobi when
Wout = 0.  The hidden activations enter the tensor-core products as two bf16 terms
(bf16_split) in this form, so the operator is linear and symmetric to about
2^-16.  (I + N)^T is applied as the same network with transposed weights
(transpose_params) plus one extra aggregation: N^T y = W1s^T h3' +
sum_u a_vu W1m^T h3'_u, h3' the transposed network's last hidden layer.
"""
import numpy as np

H, K = 64, 8
SHAPES = [("W1s", (H, 3)), ("W1m", (H, 3)), ("P2", (K, H)), ("W2h", (H, H)), ("W2m", (H, K)),
          ("P3", (K, H)), ("W3h", (H, H)), ("W3m", (H, K)), ("Wout", (3, H))]
NPARAM = sum(a * b for _, (a, b) in SHAPES)


def unpack(flat):
    out, o = {}, 0
    for name, (a, b) in SHAPES:
        out[name] = np.asarray(flat[o:o + a * b], np.float64).reshape(a, b)
        o += a * b
    return out


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def edge_weights(n, rowptr, colidx, vals):
    """a per nonzero block (0 on the diagonal blocks)."""
    A = np.asarray(vals, np.float64).reshape(-1, 9)
    nrm = np.sqrt((A * A).sum(1))
    rows = np.repeat(np.arange(n), np.diff(rowptr.astype(np.int64)))
    cols = colidx.astype(np.int64)
    dn = np.zeros(n)
    diag = rows == cols
    dn[rows[diag]] = nrm[diag]
    a = nrm / np.sqrt(dn[rows] * dn[cols])
    a[diag] = 0.0
    return a, rows, cols


def block_jacobi(n, rowptr, colidx, vals):
    A = np.asarray(vals, np.float64).reshape(-1, 3, 3)
    rows = np.repeat(np.arange(n), np.diff(rowptr.astype(np.int64)))
    d = rows == colidx.astype(np.int64)
    Dinv = np.zeros((n, 3, 3))
    Dinv[rows[d]] = np.linalg.inv(A[d])
    return Dinv


def chol_inv(n, rowptr, colidx, vals):
    """Per vertex L_v^-1 with D_v = L_v L_v^T (lower Cholesky factor)."""
    A = np.asarray(vals, np.float64).reshape(-1, 3, 3)
    rows = np.repeat(np.arange(n), np.diff(rowptr.astype(np.int64)))
    d = rows == colidx.astype(np.int64)
    D = np.zeros((n, 3, 3))
    D[rows[d]] = A[d]
    return np.linalg.inv(np.linalg.cholesky(D))


def transpose_params(params):
    """Parameters of the transposed network (same layout): layer 1 <- Wout^T
    (no message), layer 2 <- layer 3 transposed, layer 3 <- layer 2
    transposed, output <- W1s^T.  W1m^T is the extra output projection."""
    p = unpack(params)
    q = {"W1s": p["Wout"].T, "W1m": np.zeros((H, 3)), "P2": p["W3m"].T, "W2h": p["W3h"].T,
         "W2m": p["P3"].T, "P3": p["W2m"].T, "W3h": p["W2h"].T, "W3m": p["P2"].T,
         "Wout": p["W1s"].T}
    return np.concatenate([q[name].reshape(-1) for name, _ in SHAPES])


def _agg(a, rows, cols, x, n):
    out = np.zeros((n,) + x.shape[1:])
    np.add.at(out, rows, a[:, None] * x[cols])
    return out


def bf16_split(x):
    """bf16(x) + bf16(x - bf16(x)): the two-term bf16 operand of the split
    activations."""
    hi = bf16(x)
    return hi + bf16(np.asarray(x, np.float64) - hi)


def forward(params, n, rowptr, colidx, vals, r, linear=False, stage="dinv", split=False):
    """linear=True: identity activations instead of relu.  stage: the input
    map s = D^-1 r ("dinv"), L^-1 r ("linv") or r ("id").  split: the hidden
    activations enter the tensor-core products as two bf16 terms."""
    act = (lambda g: g) if linear else (lambda g: np.maximum(g, 0))
    rnd = bf16_split if split else bf16
    p = unpack(params)
    W2h, W3h = bf16(p["W2h"]), bf16(p["W3h"])
    a, rows, cols = edge_weights(n, rowptr, colidx, vals)
    rv = np.asarray(r, np.float64).reshape(n, 3)
    if stage == "id":
        s = rv.copy()
    else:
        St = (block_jacobi if stage == "dinv" else chol_inv)(n, rowptr, colidx, vals)
        s = np.einsum("vij,vj->vi", St, rv)
    m1 = _agg(a, rows, cols, s, n)
    g1 = s @ p["W1s"].T + m1 @ p["W1m"].T
    h1 = act(g1)
    q2 = h1 @ p["P2"].T
    m2 = _agg(a, rows, cols, q2, n)
    h1b = rnd(h1)
    g2 = h1b @ W2h.T + m2 @ p["W2m"].T
    h2 = act(g2)
    q3 = h2 @ p["P3"].T
    m3 = _agg(a, rows, cols, q3, n)
    h2b = rnd(h2)
    g3 = h2b @ W3h.T + m3 @ p["W3m"].T
    h3 = act(g3)
    z = s + h3 @ p["Wout"].T
    cache = dict(a=a, rows=rows, cols=cols, s=s, m1=m1, g1=g1, h1=h1, h1b=h1b, q2=q2, m2=m2,
                 g2=g2, h2=h2, h2b=h2b, q3=q3, m3=m3, g3=g3, h3=h3, W2h=W2h, W3h=W3h, p=p, n=n,
                 linear=linear)
    return z.reshape(-1), cache


def forward_sym(params, n, rowptr, colidx, vals, r):
    """z = L^-T (I + N)^T (I + N) L^-1 r (linear network N)."""
    y, cu = forward(params, n, rowptr, colidx, vals, r, linear=True, stage="linv", split=True)
    wp, ca = forward(transpose_params(params), n, rowptr, colidx, vals, y, linear=True,
                     stage="id", split=True)
    p = unpack(params)
    a, rows, cols = ca["a"], ca["rows"], ca["cols"]
    t = ca["h3"] @ p["W1m"]
    w = wp.reshape(n, 3) + _agg(a, rows, cols, t, n)
    Li = chol_inv(n, rowptr, colidx, vals)
    z = np.einsum("vji,vj->vi", Li, w)
    return z.reshape(-1), dict(cu=cu, y=y, Li=Li, args=(params, n, rowptr, colidx, vals))


def fold(params):
    """The symmetric form's linear network folded into three matrices
    (float64, from the bf16-rounded W2h/W3h): q2 = C2 [x; m1],
    q3 = C3 [x; m1; m2], N x = C4 [x; m1; m2; m3] with m1 = Aw x,
    m2 = Aw q2, m3 = Aw q3.  With identity activations each hidden layer is
    a fixed linear map of the inputs and messages before it."""
    p = unpack(params)
    E1 = np.concatenate([p["W1s"], p["W1m"]], axis=1)               # 64 x 6
    F2 = np.concatenate([bf16(p["W2h"]) @ E1, p["W2m"]], axis=1)     # 64 x 14
    F3 = np.concatenate([bf16(p["W3h"]) @ F2, p["W3m"]], axis=1)     # 64 x 22
    return p["P2"] @ E1, p["P3"] @ F2, p["Wout"] @ F3


def forward_sym_folded(params, n, rowptr, colidx, vals, r, a=None):
    """z = L^-T (I + N)^T (I + N) L^-1 r through the folded matrices: three
    aggregations forward, three for the adjoint (I + N)^T (Aw symmetric).
    a: edge weights to use (default edge_weights(); the FP16 variant passes
    its rounded copy)."""
    C2, C3, C4 = fold(params)
    a0, rows, cols = edge_weights(n, rowptr, colidx, vals)
    if a is None:
        a = a0
    agg = lambda x: _agg(a, rows, cols, x, n)  # noqa: E731
    Li = chol_inv(n, rowptr, colidx, vals)
    x = np.einsum("vij,vj->vi", Li, np.asarray(r, np.float64).reshape(n, 3))
    m1 = agg(x)
    q2 = np.concatenate([x, m1], 1) @ C2.T
    m2 = agg(q2)
    q3 = np.concatenate([x, m1, m2], 1) @ C3.T
    m3 = agg(q3)
    y = x + np.concatenate([x, m1, m2, m3], 1) @ C4.T
    # adjoint: the transposed column blocks of C4, C3, C2 in reverse order
    g3 = agg(y @ C4[:, 14:22])
    u2 = y @ C4[:, 6:14] + g3 @ C3[:, 6:14]
    g2 = agg(u2)
    m1b = y @ C4[:, 3:6] + g3 @ C3[:, 3:6] + g2 @ C2[:, 3:6]
    w = y + y @ C4[:, 0:3] + g3 @ C3[:, 0:3] + g2 @ C2[:, 0:3] + agg(m1b)
    z = np.einsum("vji,vj->vi", Li, w)
    return z.reshape(-1)


def poly_coeffs(params):
    """The symmetric form as a matrix polynomial: with N = sum_k Aw^k (x) B_k
    (the per-vertex maps commute with the aggregation),
    (I + N)^T (I + N) = sum_{d=0..6} Aw^d (x) G_d, G_d = sum_{j+k=d} B'_j^T B'_k,
    B'_0 = I + B_0.  Returns G (7 x 3 x 3), float64."""
    C2, C3, C4 = fold(params)
    C2x, C2m1 = C2[:, 0:3], C2[:, 3:6]
    C3x, C3m1, C3m2 = C3[:, 0:3], C3[:, 3:6], C3[:, 6:14]
    C4x, C4m1, C4m2, C4m3 = C4[:, 0:3], C4[:, 3:6], C4[:, 6:14], C4[:, 14:22]
    Bp = [np.eye(3) + C4x,
          C4m1 + C4m2 @ C2x + C4m3 @ C3x,
          C4m2 @ C2m1 + C4m3 @ (C3m1 + C3m2 @ C2x),
          C4m3 @ C3m2 @ C2m1]
    G = np.zeros((7, 3, 3))
    for j in range(4):
        for k in range(4):
            G[j + k] += Bp[j].T @ Bp[k]
    return G


def bfp_round(v):
    """Per-vertex block floating point, the storage of the GPU's FP16
    evaluation: each row of v (n x 3) as FP16 mantissas (round to nearest
    even) times a shared power of two that brings the row's largest |value|
    into [0.5, 1)."""
    v = np.asarray(v, np.float64)
    m = np.abs(v).max(axis=1)
    _, e = np.frexp(m)                      # m = f 2^e, f in [0.5, 1)
    s = np.ldexp(1.0, -e)[:, None]
    out = (v * s).astype(np.float16).astype(np.float64) / s
    out[m == 0] = 0.0
    return out


def forward_sym_poly(params, n, rowptr, colidx, vals, r, a=None, bfp=False):
    """z = L^-T [sum_d Aw^d (x) G_d] L^-1 r by Horner's scheme
    (w_6 = G_6 x, w_d = G_d x + Aw w_{d+1}, z = L^-T w_0).  bfp: the GPU's
    FP16 evaluation -- L^-1 rounded to BF16 (both sides), x and every stored
    w_d (d = 5..0) rounded with bfp_round (its first step aggregates x and
    applies G_6 after the sum, Aw (G_6 x) = G_6 (Aw x))."""
    G = poly_coeffs(params)
    a0, rows, cols = edge_weights(n, rowptr, colidx, vals)
    if a is None:
        a = a0
    Li = chol_inv(n, rowptr, colidx, vals)
    if bfp:
        Li = bf16(Li)
    x = np.einsum("vij,vj->vi", Li, np.asarray(r, np.float64).reshape(n, 3))
    if bfp:
        x = bfp_round(x)
        w = bfp_round(x @ G[5].T + _agg(a, rows, cols, x, n) @ G[6].T)
        for d in range(4, -1, -1):
            w = bfp_round(x @ G[d].T + _agg(a, rows, cols, w, n))
        return np.einsum("vji,vj->vi", Li, w).reshape(-1)
    w = x @ G[6].T
    for d in range(5, -1, -1):
        w = x @ G[d].T + _agg(a, rows, cols, w, n)
    return np.einsum("vji,vj->vi", Li, w).reshape(-1)


def backward_sym(cache, dz):
    """Weight gradient of <dz, M r> for the symmetric form:
    grad_N(input L^-1 r, cotangent (I + N) L^-1 dz) + grad_N(input L^-1 dz,
    cotangent (I + N) L^-1 r)."""
    params, n, rowptr, colidx, vals = cache["args"]
    yt, cg = forward(params, n, rowptr, colidx, vals, dz, linear=True, stage="linv", split=True)
    return backward(cache["cu"], yt) + backward(cg, cache["y"])


def backward(cache, dz):
    """Weight gradients (flat, in SHAPES order) for dL/dz = dz.  The bf16
    roundings pass gradients straight through."""
    c = cache
    p, n = c["p"], c["n"]
    a, rows, cols = c["a"], c["rows"], c["cols"]
    dz = np.asarray(dz, np.float64).reshape(n, 3)
    g = {}
    g["Wout"] = dz.T @ c["h3"]
    dh3 = dz @ p["Wout"]
    mask = (lambda g: np.ones_like(g)) if c["linear"] else (lambda g: (g > 0))
    dg3 = dh3 * mask(c["g3"])
    g["W3h"] = dg3.T @ c["h2b"]
    g["W3m"] = dg3.T @ c["m3"]
    dh2 = dg3 @ c["W3h"]
    dm3 = dg3 @ p["W3m"]
    dq3 = _agg(a, rows, cols, dm3, n)  # a is symmetric: the transpose aggregation
    g["P3"] = dq3.T @ c["h2"]
    dh2 = dh2 + dq3 @ p["P3"]
    dg2 = dh2 * mask(c["g2"])
    g["W2h"] = dg2.T @ c["h1b"]
    g["W2m"] = dg2.T @ c["m2"]
    dh1 = dg2 @ c["W2h"]
    dm2 = dg2 @ p["W2m"]
    dq2 = _agg(a, rows, cols, dm2, n)
    g["P2"] = dq2.T @ c["h1"]
    dh1 = dh1 + dq2 @ p["P2"]
    dg1 = dh1 * mask(c["g1"])
    g["W1s"] = dg1.T @ c["s"]
    g["W1m"] = dg1.T @ c["m1"]
    return np.concatenate([g[name].reshape(-1) for name, _ in SHAPES])


def init_params(seed=0, out_scale=0.0):
    """He-style initialisation; Wout scaled by out_scale (0 = start exactly at
    block-Jacobi)."""
    rng = np.random.Generator(np.random.Philox(seed))
    parts = []
    for name, (a, b) in SHAPES:
        w = rng.normal(0, np.sqrt(2.0 / b), size=(a, b))
        if name == "Wout":
            w *= out_scale
        parts.append(w.reshape(-1))
    return np.concatenate(parts).astype(np.float32)
