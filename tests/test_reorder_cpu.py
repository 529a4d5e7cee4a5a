"""Locality reordering (sg_hilbert_order / sg_element_order, the host side of
simit::reorder): curve properties and the invariance of the assembled system
under the renumbering (CPU: the library's host functions and the oracle)."""
import numpy as np
import pytest

from simit_gb300 import _lib, problems
from simit_gb300.runtime import element_order, hilbert_order, reorder_mesh


def test_hilbert_index_is_a_bijection_with_unit_steps():
    bits = 3
    side = 1 << bits
    pts = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    idx = []
    for p in pts:
        import ctypes
        out = ctypes.c_uint64()
        _lib.call("sg_hilbert_index", int(p[0]), int(p[1]), int(p[2]), bits, ctypes.byref(out))
        idx.append(out.value)
    idx = np.array(idx)
    assert sorted(idx) == list(range(side ** 3))
    walk = pts[np.argsort(idx)]
    assert np.all(np.abs(np.diff(walk, axis=0)).sum(1) == 1)  # each step to a neighbour


def test_hilbert_order_of_a_lattice_walks_neighbours():
    """A lattice of 2^3 + 1 points per axis: the 8^3 interior cells come
    first along the curve in unit steps, then the upper faces."""
    side = 9
    pts = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    vo = hilbert_order(pts.astype(np.float64) * 0.125 + 0.3, bits=3)
    assert sorted(vo) == list(range(side ** 3))
    walk = np.empty_like(pts)
    walk[vo] = pts
    inner = walk[:512]
    assert np.all(inner < 8)
    assert np.all(np.abs(np.diff(inner, axis=0)).sum(1) == 1)
    assert np.all((walk[512:] == 8).any(1))


def test_element_order_sorts_sorted_tuples():
    g = np.random.default_rng(3)
    ep = g.integers(0, 50, size=200 * 4).astype(np.int32)
    eo = element_order(ep, 4)
    s = np.sort(ep.reshape(-1, 4), axis=1)
    ref = np.lexsort(s.T[::-1])  # lexicographic, stable
    assert np.array_equal(eo, ref)


def test_reordered_system_is_the_permuted_system(oracle):
    """Pattern of the renumbered mesh = renumbered pattern (bit-exact);
    assembled values equal up to the element-order rounding (1e-12)."""
    h = problems.hetero_mesh(5)
    r = problems.reorder_hetero(h)
    vo = r["vertex_ordering"]
    n = h["n"]
    rp0, ci0 = oracle.pattern(n, h["tets"], 4)
    rp1, ci1 = oracle.pattern(n, r["tets"], 4)
    rows0 = np.repeat(np.arange(n), np.diff(rp0.astype(np.int64)))
    for v_old in range(n):
        v_new = vo[v_old]
        cols_old = ci0[rp0[v_old]:rp0[v_old + 1]]
        assert np.array_equal(np.sort(vo[cols_old]), ci1[rp1[v_new]:rp1[v_new + 1]])
    args = lambda H: oracle.tet_precompute(H["X0"], H["tets"], problems.RHO)  # noqa: E731
    B0, W0, _ = args(h)
    B1, W1, _ = args(r)
    A0 = oracle.tet_stiffness(0, h["x"], h["c"], h["tets"], B0, W0, h["mu"], h["lam"],
                              problems.H, problems.RHO, rp0, ci0).reshape(-1, 9)
    A1 = oracle.tet_stiffness(0, r["x"], r["c"], r["tets"], B1, W1, r["mu"], r["lam"],
                              problems.H, problems.RHO, rp1, ci1).reshape(-1, 9)
    # map every old block (row, col) to its slot in the new pattern
    for q in range(len(ci0)):
        a, b = vo[rows0[q]], vo[ci0[q]]
        lo, hi = rp1[a], rp1[a + 1]
        s = lo + np.searchsorted(ci1[lo:hi], b)
        assert np.allclose(A1[s], A0[q], rtol=1e-12, atol=1e-12 * np.abs(A0).max())


def test_morton_order_groups_aligned_cubes():
    side = 9
    pts = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    vo = hilbert_order(pts.astype(np.float64), bits=3, curve="morton")
    walk = np.empty_like(pts)
    walk[vo] = pts
    # every run of 8 consecutive interior vertices is one aligned 2x2x2 cube
    cubes = walk[:512].reshape(-1, 8, 3) // 2
    assert np.all(cubes == cubes[:, :1, :])
    assert sorted(vo) == list(range(side ** 3))


def test_cpp_facade_set_reordering(tmp_path):
    """tests/cpp/test_reorder.cpp: the facade's reorderVertexSet /
    reorderEdgeSet / reorder on simit_gb300::Set, restating the reference's
    reorderInt and reorderDouble tests (test/reorder-tests.cpp:177-404), with
    the orderings' properties and error cases.  Host code only."""
    import os
    import subprocess
    from simit_gb300 import _lib
    _lib.load()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "test_reorder")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", root, "-I",
                           os.path.join(cuda, "include"),
                           os.path.join(root, "tests", "cpp", "test_reorder.cpp"),
                           "-L", os.path.join(root, "simit_gb300"), "-lsimit_gb300",
                           "-L", os.path.join(cuda, "lib64"), "-lcudart",
                           "-Wl,-rpath," + os.path.join(root, "simit_gb300"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all passed" in r.stdout
