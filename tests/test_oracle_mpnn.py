"""CPU checks of the learned-preconditioner oracle (oracle/mpnn_oracle.py):
its weight gradients against central finite differences for the three
forms, and the symmetric form's defining properties (symmetric, positive
definite, block Jacobi when the output weights are zero).  The GPU kernels
are checked against this oracle in test_gpu_learned.py."""
import numpy as np
import pytest

from oracle import mpnn_oracle as mo
from oracle import oracle
from simit_gb300 import problems


@pytest.fixture(scope="module")
def system():
    oracle.build()
    h = problems.hetero_mesh(3, seed=3)
    rp, ci = oracle.pattern(h["n"], h["tets"], 4)
    B, W, _ = oracle.tet_precompute(h["X0"], h["tets"], problems.RHO)
    A = oracle.tet_stiffness(0, h["x"], h["c"], h["tets"], B, W, h["mu"], h["lam"], problems.H,
                             problems.RHO, rp, ci)
    return h["n"], rp, ci, np.asarray(A)


@pytest.fixture
def exact(monkeypatch):
    # exact arithmetic: the bf16 roundings pass gradients straight through and
    # would make the map non-differentiable at rounding boundaries
    monkeypatch.setattr(mo, "bf16", lambda x: np.asarray(x, np.float64))


def _apply(form, p, n, rp, ci, A, r):
    if form == "sym":
        return mo.forward_sym(p, n, rp, ci, A, r)
    return mo.forward(p, n, rp, ci, A, r, linear=form == "linear")


def _grad(form, cache, w):
    return mo.backward_sym(cache, w) if form == "sym" else mo.backward(cache, w)


@pytest.mark.parametrize("form", ["relu", "linear", "sym"])
def test_gradient_matches_finite_differences(system, exact, form):
    n, rp, ci, A = system
    rng = np.random.default_rng(0)
    p = mo.init_params(1, out_scale=0.5).astype(np.float64) * 0.5
    r = rng.normal(size=n * 3)
    w = rng.normal(size=n * 3)
    _, cache = _apply(form, p, n, rp, ci, A, r)
    g = _grad(form, cache, w)
    f = lambda q: float(np.dot(_apply(form, q, n, rp, ci, A, r)[0], w))  # noqa: E731
    errs = []
    for i in rng.choice(len(p), 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6 * max(1.0, abs(p[i]))
        fd = (f(p + e) - f(p - e)) / (2 * e[i])
        errs.append(abs(fd - g[i]) / (abs(fd) + abs(g[i]) + 1e-9))
    # relu kinks can sit inside a difference interval: median for relu
    assert (np.median(errs) if form == "relu" else max(errs)) < 1e-3, errs


def test_symmetric_form_properties(system, exact):
    n, rp, ci, A = system
    rng = np.random.default_rng(1)
    p = mo.init_params(2, out_scale=1.0).astype(np.float64)
    u, v = rng.normal(size=n * 3), rng.normal(size=n * 3)
    Mu = mo.forward_sym(p, n, rp, ci, A, u)[0]
    Mv = mo.forward_sym(p, n, rp, ci, A, v)[0]
    assert abs(v @ Mu - u @ Mv) <= 1e-10 * abs(v @ Mu)
    assert u @ Mu > 0 and v @ Mv > 0
    p[-3 * mo.H:] = 0.0  # Wout = 0
    z0 = mo.forward_sym(p, n, rp, ci, A, u)[0]
    bj = np.einsum("vij,vj->vi", mo.block_jacobi(n, rp, ci, A), u.reshape(n, 3)).reshape(-1)
    assert np.allclose(z0, bj, rtol=1e-12, atol=1e-14 * np.abs(bj).max())


def test_transpose_params_is_the_adjoint(system, exact):
    """<v, N u> = <N^T v, u> with N^T run as the transposed network plus the
    extra aggregation of W1m^T h3'."""
    n, rp, ci, A = system
    rng = np.random.default_rng(2)
    p = mo.init_params(3, out_scale=1.0).astype(np.float64)
    u, v = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    Nu = mo.forward(p, n, rp, ci, A, u, linear=True, stage="id")[0].reshape(n, 3) - u
    wp, c = mo.forward(mo.transpose_params(p), n, rp, ci, A, v, linear=True, stage="id")
    NTv = wp.reshape(n, 3) - v + mo._agg(c["a"], c["rows"], c["cols"],
                                         c["h3"] @ mo.unpack(p)["W1m"], n)
    assert abs((v * Nu).sum() - (NTv * u).sum()) <= 1e-10 * abs((v * Nu).sum())


def test_folded_operator_equals_the_layered_network(system):
    """The folded evaluation (three small matrices, six aggregations) is the
    same operator as the layered symmetric form: equal to its split-bf16
    activations' accuracy (about 2^-16 of the correction), exactly in exact
    arithmetic."""
    n, rp, ci, A = system
    rng = np.random.default_rng(4)
    from simit_gb300 import learned
    p = learned.load_weights("sym").astype(np.float64)  # the trained symmetric-form weights
    r = rng.normal(size=n * 3)
    zl = mo.forward_sym(p, n, rp, ci, A, r)[0]
    zf = mo.forward_sym_folded(p, n, rp, ci, A, r)
    bj = np.einsum("vij,vj->vi", mo.block_jacobi(n, rp, ci, A), r.reshape(n, 3)).reshape(-1)
    corr = np.linalg.norm(zl - bj)
    assert corr > 0
    assert np.linalg.norm(zf - zl) <= 1e-4 * corr


def test_folded_operator_is_exact_in_exact_arithmetic(system, exact):
    n, rp, ci, A = system
    rng = np.random.default_rng(5)
    p = mo.init_params(6, out_scale=1.0).astype(np.float64)
    r = rng.normal(size=n * 3)
    zl = mo.forward_sym(p, n, rp, ci, A, r)[0]
    zf = mo.forward_sym_folded(p, n, rp, ci, A, r)
    assert np.allclose(zf, zl, rtol=1e-11, atol=1e-12 * np.abs(zl).max())


def test_polynomial_form_equals_the_folded_operator(system, exact):
    """The degree-6 matrix polynomial in the edge-weight aggregation (the
    evaluation the GPU runs) equals the folded network and the layered
    network in exact arithmetic, and its coefficients are symmetric."""
    n, rp, ci, A = system
    rng = np.random.default_rng(7)
    p = mo.init_params(8, out_scale=1.0).astype(np.float64)
    r = rng.normal(size=n * 3)
    zl = mo.forward_sym(p, n, rp, ci, A, r)[0]
    zp = mo.forward_sym_poly(p, n, rp, ci, A, r)
    assert np.allclose(zp, zl, rtol=1e-11, atol=1e-12 * np.abs(zl).max())
    G = mo.poly_coeffs(p)
    assert np.allclose(G, np.transpose(G, (0, 2, 1)), rtol=1e-12, atol=1e-14 * np.abs(G).max())


def test_bfp_round_block_floating_point():
    """The FP16 evaluation's vector storage as the oracle states it: each
    row keeps 11 significant bits of its largest value, any magnitude."""
    from oracle import mpnn_oracle as mo
    rng = np.random.Generator(np.random.Philox(3))
    v = rng.normal(size=(500, 3)) * np.exp(rng.uniform(-60, 60, size=(500, 1)))
    v[7] = 0.0
    v[9] = [1.0, 0.5, -0.25]          # exactly representable
    out = mo.bfp_round(v)
    m = np.abs(v).max(axis=1)
    assert np.all(np.abs(out - v) <= 2.0 ** -11 * m[:, None] * (1 + 1e-12))
    assert np.all(out[7] == 0.0) and np.array_equal(out[9], v[9])
    # rounding is relative to the row's largest value, not to each entry
    row = np.array([[1.0, 1e-9, 3e-4]])
    assert mo.bfp_round(row)[0, 1] == 0.0
    assert mo.bfp_round(row)[0, 0] == 1.0


def test_network_weights_of_a_polynomial():
    """learned.params_of_poly builds network weights whose folded polynomial
    has the given coefficients (the oracle's poly_coeffs reproduces
    G_d = sum_{j+k=d} B'_j^T B'_k); learned.poly_of_params recovers B from
    weights, also for the shipped ones."""
    from oracle import mpnn_oracle as mo
    from simit_gb300 import learned
    rng = np.random.Generator(np.random.Philox(5))
    B = rng.normal(0, 0.3, size=(4, 3, 3))
    p = learned.params_of_poly(B)
    assert p.dtype == np.float32 and p.size == mo.NPARAM
    assert np.abs(learned.poly_of_params(p) - B).max() <= 1e-7
    Bp = [np.eye(3) + B[0], B[1], B[2], B[3]]
    G = np.zeros((7, 3, 3))
    for j in range(4):
        for k in range(4):
            G[j + k] += Bp[j].T @ Bp[k]
    assert np.abs(mo.poly_coeffs(p) - G).max() <= 1e-6
    w = learned.load_weights("sym")
    Gw = mo.poly_coeffs(w)
    assert np.abs(mo.poly_coeffs(learned.params_of_poly(learned.poly_of_params(w))) - Gw).max() \
        <= 1e-6 * np.abs(Gw).max()


def test_elasticity_coupling_is_mostly_anisotropic(oracle):
    """Why scalar edge weights limit the network on elasticity: after the
    block-Jacobi scaling L_i^-1 A_ij L_j^-T, the isotropic part (tr/3 I) of
    the off-diagonal blocks holds well under half of their Frobenius energy
    (about 27 % on an 8^3 lattice with E log-uniform 1e3..1e6)."""
    from simit_gb300 import meshgen
    mg = meshgen.tet_grid(6)
    n, tets = mg["n"], mg["tets"]
    nT = len(tets) // 4
    g = np.random.default_rng(3)
    E = 10 ** g.uniform(3, 6, nT)
    nu = g.uniform(0.35, 0.45, nT)
    mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
    B, W, _ = oracle.tet_precompute(mg["X0"], tets, 1e3)
    rp, ci = oracle.pattern(n, tets, 4)
    A = oracle.tet_stiffness(0, mg["x"], np.zeros(n, np.int32), tets, B, W, mu, lam, 0.01,
                             1e3, rp, ci).reshape(-1, 3, 3)
    Linv = np.zeros((n, 3, 3))
    for i in range(n):
        k = rp[i] + list(ci[rp[i]:rp[i + 1]]).index(i)
        Linv[i] = np.linalg.inv(np.linalg.cholesky(A[k]))
    iso = tot = 0.0
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            j = ci[k]
            if j != i:
                N = Linv[i] @ A[k] @ Linv[j].T
                iso += 3 * (np.trace(N) / 3) ** 2
                tot += float((N * N).sum())
    assert 0.0 < iso / tot < 0.4
