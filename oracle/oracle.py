"""ORACLE (test infrastructure): ctypes wrapper over oracle/liboracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker.  The product package never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_pattern.so")

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double


def build(force=False):
    """Compile the restatement (g++, -ffp-contract=off) into liboracle.so."""
    src = os.path.join(HERE, "sg_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(src) > os.path.getmtime(LIB):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                               "-fPIC", "-shared", src, "-o", LIB])


def build_ref():
    """Compile the reference's own pattern builder when its sources exist."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.or_pattern.restype = _I64
        L.or_pattern.argtypes = [_I32, _P, _I64, _I32, _P, _P, _I64]
        L.or_slots.argtypes = [_P, _I64, _I32, _P, _P, _P]
        L.or_spmv_f64.argtypes = [_I32, _I32, _P, _P, _P, _P, _P]
        L.or_spmv_f32.argtypes = [_I32, _I32, _P, _P, _P, _P, _P]
        L.or_dot_f64.restype = _D
        L.or_dot_f64.argtypes = [_I32, _I32, _P, _P]
        L.or_cg_normr2_f64.restype = ctypes.c_int
        L.or_cg_normr2_f64.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, _D, ctypes.c_int, _P]
        L.or_jacobi_pcg_f64.restype = ctypes.c_int
        L.or_jacobi_pcg_f64.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, _D, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, _P]
        L.or_springs_assemble.argtypes = [ctypes.c_int, _I32, _P, _P, _P, _P, _I64, _P, _P, _P,
                                          _D, _D, _P, _P, _P, _P, _P]
        L.or_springs_step.restype = ctypes.c_int
        L.or_springs_step.argtypes = [ctypes.c_int, _I32, _P, _P, _P, _P, _I64, _P, _P, _P,
                                      _D, _D, _P, _P, _P, _D, ctypes.c_int]
        L.or_scalar_springs_assemble.argtypes = [_I32, _I64, _P, _P, _D, _D, _P, _P, _P]
        L.or_cg_norm_f64.restype = ctypes.c_int
        L.or_cg_norm_f64.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, _D, ctypes.c_int]
        L.or_tet_precompute.argtypes = [_I32, _P, _I64, _P, _D, _P, _P, _P]
        L.or_tet_force.argtypes = [ctypes.c_int, _I32, _P, _P, _P, _I64, _P, _P, _P, _P, _P,
                                   _D, _D, _P, _P]
        L.or_tet_stiffness.argtypes = [ctypes.c_int, _I32, _P, _P, _I64, _P, _P, _P, _P, _P,
                                       _D, _D, _P, _P, _P]
        L.or_tet_step.restype = ctypes.c_int
        L.or_tet_step.argtypes = [ctypes.c_int, _I32, _P, _P, _P, _I64, _P, _P, _P, _P, _P,
                                  _D, _D, _P, _P, _P, _D, ctypes.c_int]
        L.or_heat_assemble.argtypes = [_I32, _I64, _P, _P, _P, _P, _D, _P, _P, _P, _P, _P]
        L.or_add_diag_f64.argtypes = [_I32, _I32, _P, _P, _P, _D, ctypes.c_int, _D, _P, _P]
        L.or_add_diag_f32.argtypes = [_I32, _I32, _P, _P, _P, ctypes.c_float, ctypes.c_int,
                                      ctypes.c_float, _P, _P]
        L.or_cloth_faces.argtypes = [_P, _I64, _P, _P, _P]
        L.or_cloth_hinges.argtypes = [_P, _I64, _P, _P, _P, _P]
        L.or_cloth_stretch.argtypes = [_I32, _P, _I64, _P, _P, _P, _P]
        L.or_cloth_bend.argtypes = [_I32, _P, _I64, _P, _P, _P, _P, _P]
        L.or_cloth_step.argtypes = [_I32, _P, _P, _P, _P, _I64, _P, _P, _P, _I64, _P, _P, _P,
                                    _P, _D, _D, _D, _D]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_P)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def pattern(n, ep, card):
    ep = _c(ep, np.int32)
    nE = ep.size // card
    cap = max(1, nE * card * card + n)
    rowptr = np.zeros(n + 1, np.uint32)
    colidx = np.zeros(cap, np.uint32)
    nnz = lib().or_pattern(n, _p(ep), nE, card, _p(rowptr), _p(colidx), cap)
    assert nnz >= 0
    return rowptr, colidx[:nnz].copy()


def ref_pattern(n, ep, card):
    """The reference's own PathIndexBuilder (None when not built here)."""
    if not os.path.exists(REF_LIB):
        return None
    L = ctypes.CDLL(REF_LIB)
    L.ref_pattern.restype = _I64
    L.ref_pattern.argtypes = [_I32, _P, _I64, _I32, _P, _P, _I64]
    ep = _c(ep, np.int32)
    nE = ep.size // card
    cap = max(1, nE * card * card + n)
    rowptr = np.zeros(n + 1, np.uint32)
    colidx = np.zeros(cap, np.uint32)
    nnz = L.ref_pattern(n, _p(ep), nE, card, _p(rowptr), _p(colidx), cap)
    assert nnz >= 0
    return rowptr, colidx[:nnz].copy()


def ref_incidence(kind, n0, n1, set_of, ep, xr=1, xc=1):
    """The reference's own Link::ev (kind 0) / Link::ve (1) index or the And
    of the two between vertex sets xr, xc (2), for an edge set whose endpoint
    k lies in V0 or V1 per set_of[k] (None when not built here)."""
    if not os.path.exists(REF_LIB):
        return None
    L = ctypes.CDLL(REF_LIB)
    L.ref_incidence.restype = _I64
    L.ref_incidence.argtypes = [ctypes.c_int, _I32, _I32, _I32, _P, _P, _I64, _I32, _I32, _P,
                                _P, _I64]
    card = len(set_of)
    ep = _c(ep, np.int32)
    so = _c(set_of, np.int32)
    nE = ep.size // card
    rows = nE if kind == 0 else (n1 if xr else n0)
    cap = max(1, nE * card * card + n0 + n1)
    rowptr = np.zeros(rows + 1, np.uint32)
    colidx = np.zeros(cap, np.uint32)
    nnz = L.ref_incidence(kind, n0, n1, card, _p(so), _p(ep), nE, xr, xc, _p(rowptr),
                          _p(colidx), cap)
    assert nnz >= 0, nnz
    return rowptr, colidx[:nnz].copy()


def ref_slots(ep, card, rowptr, colidx):
    if not os.path.exists(REF_LIB):
        return None
    L = ctypes.CDLL(REF_LIB)
    L.ref_slots.argtypes = [_P, _I64, _I32, _P, _P, _P]
    ep = _c(ep, np.int32)
    nE = ep.size // card
    out = np.zeros(nE * card * card, np.uint32)
    L.ref_slots(_p(ep), nE, card, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)), _p(out))
    return out


def slots(ep, card, rowptr, colidx):
    ep = _c(ep, np.int32)
    nE = ep.size // card
    out = np.zeros(nE * card * card, np.uint32)
    lib().or_slots(_p(ep), nE, card, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
                   _p(out))
    return out


def assemble_blocks(ep, card, bs, eb, rowptr, colidx):
    """`map f to E reduce +` (src/lower/lower_maps.cpp:54-128): for elements
    in order, for (i, j), += block (i, j) into the slot loc(ep[i], ep[j])
    (src/runtime.cpp:19-23), FP64."""
    sl = slots(ep, card, rowptr, colidx).astype(np.int64)
    eb = np.asarray(eb, np.float64).reshape(-1, card * card, bs * bs)
    vals = np.zeros((len(colidx), bs * bs))
    for e in range(eb.shape[0]):
        for ij in range(card * card):
            vals[sl[e * card * card + ij]] += eb[e, ij]
    return vals.reshape(-1)


def spmv(n, bs, rowptr, colidx, vals, x):
    if vals.dtype == np.float32:
        y = np.zeros(n * bs, np.float32)
        lib().or_spmv_f32(n, bs, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
                          _p(_c(vals, np.float32)), _p(_c(x, np.float32)), _p(y))
    else:
        y = np.zeros(n * bs, np.float64)
        lib().or_spmv_f64(n, bs, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
                          _p(_c(vals, np.float64)), _p(_c(x, np.float64)), _p(y))
    return y


def add_diag(n, bs, rowptr, colidx, K, diag=None, ident=0.0, scale=1.0):
    """out = D + scale*K on K's pattern, the lowered `MDK = MD + K` of
    apps/springs/isprings.sim:74 (MDK = 0; MDK[loc(l,l)] = D[l];
    MDK[lm] = MDK[lm] + scale*K[lm]) in K's dtype; diag None: D = ident*I."""
    dt = np.float32 if K.dtype == np.float32 else np.float64
    out = np.zeros(len(K), dt)
    has_d = int(diag is not None or ident != 0.0)
    d = None if diag is None else _c(diag, dt)
    f = lib().or_add_diag_f32 if dt == np.float32 else lib().or_add_diag_f64
    f(n, bs, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
      None if d is None else _p(d), ident, has_d, scale, _p(_c(K, dt)), _p(out))
    return out


def incidence_pattern(kind, n, sel, npos):
    """Link::ev (kind 0, src/path_indices.cpp:207-246: row e = its endpoints
    in endpoint order) or Link::ve (kind 1, :248-276: per vertex the edges
    that list it, pushed back in edge order, then packed)."""
    sel = np.asarray(sel, np.int64).reshape(-1, npos)
    nE = sel.shape[0]
    if kind == 0:
        return (np.arange(nE + 1, dtype=np.uint32) * npos).astype(np.uint32), \
            sel.reshape(-1).astype(np.uint32)
    nbrs = [[] for _ in range(n)]
    for e in range(nE):
        for k in range(npos):
            nbrs[sel[e, k]].append(e)
    rowptr = np.zeros(n + 1, np.uint32)
    rowptr[1:] = np.cumsum([len(x) for x in nbrs])
    colidx = np.array([e for x in nbrs for e in x], np.uint32)
    return rowptr, colidx


def assemble_incidence(kind, sel, npos, bs, eb, rowptr, colidx):
    """`map` into an incidence matrix: for elements in order, for each write
    (endpoint k, in order) `+=` into loc(row, col) (src/runtime.cpp:19-23:
    the first slot of that column in the row), FP64, zero-initialised."""
    sel = np.asarray(sel, np.int64).reshape(-1, npos)
    bb = bs * bs
    eb = np.asarray(eb, np.float64).reshape(sel.shape[0], npos, bb)
    vals = np.zeros((len(colidx), bb))

    def loc(r, c):
        q = int(rowptr[r])
        while int(colidx[q]) != c:
            q += 1
        return q
    for e in range(sel.shape[0]):
        for k in range(npos):
            v = int(sel[e, k])
            q = loc(e, v) if kind == 0 else loc(v, e)
            vals[q] += eb[e, k]
    return vals.reshape(-1)


def rect_pattern(nr, sel_r, npos_r, sel_c, npos_c):
    """∃e.(v-e ∧ e-u) with v and u in different vertex sets
    (src/path_indices.cpp:359-429, And of Link::ve over the row set's
    endpoints and Link::ev over the column set's): sorted unique columns."""
    sr = np.asarray(sel_r, np.int64).reshape(-1, npos_r)
    sc = np.asarray(sel_c, np.int64).reshape(-1, npos_c)
    rows = [set() for _ in range(nr)]
    for e in range(sr.shape[0]):
        for v in sr[e]:
            rows[v].update(int(u) for u in sc[e])
    rowptr = np.zeros(nr + 1, np.uint32)
    rowptr[1:] = np.cumsum([len(r) for r in rows])
    colidx = np.array([u for r in rows for u in sorted(r)], np.uint32)
    return rowptr, colidx


def assemble_rect(sel_r, npos_r, sel_c, npos_c, bs, eb, rowptr, colidx):
    """`map` into it: elements in order, writes (k, j) in order, `+=` into
    loc(row endpoint k, column endpoint j), FP64."""
    sr = np.asarray(sel_r, np.int64).reshape(-1, npos_r)
    sc = np.asarray(sel_c, np.int64).reshape(-1, npos_c)
    bb = bs * bs
    eb = np.asarray(eb, np.float64).reshape(sr.shape[0], npos_r, npos_c, bb)
    vals = np.zeros((len(colidx), bb))
    for e in range(sr.shape[0]):
        for k in range(npos_r):
            for j in range(npos_c):
                q = int(rowptr[sr[e, k]])
                while int(colidx[q]) != sc[e, j]:
                    q += 1
                vals[q] += eb[e, k, j]
    return vals.reshape(-1)


def cg_normr2(n, bs, rowptr, colidx, A, b, x0, tol2, maxiters):
    x = _c(x0, np.float64).copy()
    nr = np.zeros(1)
    it = lib().or_cg_normr2_f64(n, bs, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
                                _p(_c(A, np.float64)), _p(_c(b, np.float64)), _p(x), tol2,
                                maxiters, _p(nr))
    return x, it, float(nr[0])


def jacobi_pcg(n, bs, rowptr, colidx, A, b, x0, tol, maxiters, refresh=50, zr_stop=False):
    x = _c(x0, np.float64).copy()
    rr = np.zeros(1)
    it = lib().or_jacobi_pcg_f64(n, bs, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
                                 _p(_c(A, np.float64)), _p(_c(b, np.float64)), _p(x), tol,
                                 maxiters, refresh, int(zr_stop), _p(rr))
    return x, it, float(rr[0])


def relres(n, bs, rowptr, colidx, A, b, x):
    """||b - A x|| / ||b|| in FP64 with the lowered SpMV."""
    r = np.asarray(b, np.float64) - spmv(n, bs, rowptr, colidx, np.asarray(A, np.float64),
                                         np.asarray(x, np.float64))
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def springs_assemble(form, x, v, m, fixed, ep, k, l0, h, viscous, grav, rowptr, colidx):
    n = len(m)
    nS = len(k)
    MDK = np.zeros(int(rowptr[n]) * 9)
    f = np.zeros(n * 3)
    lib().or_springs_assemble(form, n, _p(_c(x, np.float64)), _p(_c(v, np.float64)),
                              _p(_c(m, np.float64)), _p(_c(fixed, np.uint8)), nS,
                              _p(_c(ep, np.int32)), _p(_c(k, np.float64)),
                              _p(_c(l0, np.float64)), h, viscous, _p(_c(grav, np.float64)),
                              _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)), _p(MDK),
                              _p(f))
    return MDK, f


def springs_step(form, x, v, m, fixed, ep, k, l0, h, viscous, grav, rowptr, colidx, tol2,
                 maxiters):
    """Advances x, v (float64 arrays, modified in place); returns CG iterations."""
    assert x.dtype == np.float64 and v.dtype == np.float64
    n = len(m)
    return lib().or_springs_step(form, n, _p(x), _p(v), _p(_c(m, np.float64)),
                                 _p(_c(fixed, np.uint8)), len(k), _p(_c(ep, np.int32)),
                                 _p(_c(k, np.float64)), _p(_c(l0, np.float64)), h, viscous,
                                 _p(_c(grav, np.float64)), _p(_c(rowptr, np.uint32)),
                                 _p(_c(colidx, np.uint32)), tol2, maxiters)


def scalar_springs_assemble(n, ep, a, diag, scale, rowptr, colidx):
    A = np.zeros(int(rowptr[n]))
    lib().or_scalar_springs_assemble(n, len(a), _p(_c(ep, np.int32)), _p(_c(a, np.float64)),
                                     diag, scale, _p(_c(rowptr, np.uint32)),
                                     _p(_c(colidx, np.uint32)), _p(A))
    return A


def cg_norm(n, bs, rowptr, colidx, A, b, tol, maxiters):
    x = np.zeros(n * bs)
    it = lib().or_cg_norm_f64(n, bs, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)),
                              _p(_c(A, np.float64)), _p(_c(b, np.float64)), _p(x), tol,
                              maxiters)
    return x, it


def tet_precompute(x, tets, rho):
    n = len(x) // 3
    nT = len(tets) // 4
    B = np.zeros(nT * 9)
    W = np.zeros(nT)
    m = np.zeros(n)
    lib().or_tet_precompute(n, _p(_c(x, np.float64)), nT, _p(_c(tets, np.int32)), rho, _p(B),
                            _p(W), _p(m))
    return B, W, m


def tet_force(neo, x, v, c, tets, B, W, u, l, h, rho, grav):
    n = len(x) // 3
    f = np.zeros(n * 3)
    lib().or_tet_force(int(neo), n, _p(_c(x, np.float64)), _p(_c(v, np.float64)),
                       _p(_c(c, np.int32)), len(tets) // 4, _p(_c(tets, np.int32)),
                       _p(_c(B, np.float64)), _p(_c(W, np.float64)), _p(_c(u, np.float64)),
                       _p(_c(l, np.float64)), h, rho, _p(_c(grav, np.float64)), _p(f))
    return f


def tet_stiffness(neo, x, c, tets, B, W, u, l, h, rho, rowptr, colidx):
    n = len(x) // 3
    A = np.zeros(int(rowptr[n]) * 9)
    lib().or_tet_stiffness(int(neo), n, _p(_c(x, np.float64)), _p(_c(c, np.int32)),
                           len(tets) // 4, _p(_c(tets, np.int32)), _p(_c(B, np.float64)),
                           _p(_c(W, np.float64)), _p(_c(u, np.float64)), _p(_c(l, np.float64)),
                           h, rho, _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)), _p(A))
    return A


def tet_step(neo, x, v, c, tets, B, W, u, l, h, rho, grav, rowptr, colidx, tol2, maxiters):
    """Advances x, v (float64, in place); returns CG iterations."""
    assert x.dtype == np.float64 and v.dtype == np.float64
    return lib().or_tet_step(int(neo), len(x) // 3, _p(x), _p(v), _p(_c(c, np.int32)),
                             len(tets) // 4, _p(_c(tets, np.int32)), _p(_c(B, np.float64)),
                             _p(_c(W, np.float64)), _p(_c(u, np.float64)),
                             _p(_c(l, np.float64)), h, rho, _p(_c(grav, np.float64)),
                             _p(_c(rowptr, np.uint32)), _p(_c(colidx, np.uint32)), tol2,
                             maxiters)


def heat_assemble(n, tets, B, W, kappa, dt, T0, rowptr, colidx):
    A = np.zeros(int(rowptr[n]))
    b = np.zeros(n)
    lib().or_heat_assemble(n, len(tets) // 4, _p(_c(tets, np.int32)), _p(_c(B, np.float64)),
                           _p(_c(W, np.float64)), _p(_c(kappa, np.float64)), dt,
                           _p(_c(T0, np.float64)), _p(_c(rowptr, np.uint32)),
                           _p(_c(colidx, np.uint32)), _p(A), _p(b))
    return A, b


def cloth_faces(x, faces):
    """Per face (apps/cloth/cloth.sim:66-102): the stretching matrix (nF, 3, 3)
    and the rest squared edge lengths (nF, 3)."""
    faces = _c(faces, np.int32)
    nF = faces.size // 3
    K = np.zeros((nF, 3, 3))
    rest = np.zeros((nF, 3))
    lib().or_cloth_faces(_p(_c(x, np.float64)), nF, _p(faces), _p(K), _p(rest))
    return K, rest


def cloth_hinges(x, hinges):
    """Per hinge (cloth.sim:105-113): rest angle, rest length, perpendicular
    length."""
    hinges = _c(hinges, np.int32)
    nH = hinges.size // 4
    ang, ln, perp = np.zeros(nH), np.zeros(nH), np.zeros(nH)
    lib().or_cloth_hinges(_p(_c(x, np.float64)), nH, _p(hinges), _p(ang), _p(ln), _p(perp))
    return ang, ln, perp


def cloth_stretch(n, x, faces, K, rest):
    """`map stretchingForce to faces reduce +` (cloth.sim:142-164), 3 per vertex."""
    faces = _c(faces, np.int32)
    f = np.zeros(n * 3)
    lib().or_cloth_stretch(n, _p(_c(x, np.float64)), faces.size // 3, _p(faces),
                           _p(_c(K, np.float64)), _p(_c(rest, np.float64)), _p(f))
    return f


def cloth_bend(n, x, hinges, ang, ln, perp):
    """`map bendingForce to hinges reduce +` (cloth.sim:166-173), 3 per vertex."""
    hinges = _c(hinges, np.int32)
    f = np.zeros(n * 3)
    lib().or_cloth_bend(n, _p(_c(x, np.float64)), hinges.size // 4, _p(hinges),
                        _p(_c(ang, np.float64)), _p(_c(ln, np.float64)),
                        _p(_c(perp, np.float64)), _p(f))
    return f


def cloth_step(x, v, m, fixed, faces, K, rest, hinges, ang, ln, perp, dt, ks, kb, damping):
    """One step of cloth.sim's `main` (cloth.sim:201-222); returns (x, v)."""
    x = np.array(x, np.float64).reshape(-1)
    v = np.array(v, np.float64).reshape(-1)
    n = x.size // 3
    faces = _c(faces, np.int32)
    hinges = _c(hinges, np.int32)
    lib().or_cloth_step(n, _p(x), _p(v), _p(_c(m, np.float64)), _p(_c(fixed, np.int32)),
                        faces.size // 3, _p(faces), _p(_c(K, np.float64)),
                        _p(_c(rest, np.float64)), hinges.size // 4, _p(hinges),
                        _p(_c(ang, np.float64)), _p(_c(ln, np.float64)),
                        _p(_c(perp, np.float64)), dt, ks, kb, damping)
    return x, v
