"""Seeded synthetic meshes for the sparse-system path (host setup, not timed).

All random values come from numpy's Philox counter-based generator, which
gives the same stream on x86-64 and aarch64, so the CPU oracle and the GPU
path see identical inputs.

* box_springs   -- simit::createBox lattice + axis springs
                   (reference: src/graph.cpp:66-115, same vertex and edge order)
* tet_grid      -- unit cube of n^3 cells, 5 tets per cell, split parity
                   alternating so that face diagonals match between cells
* cloth_sheet   -- triangulated square sheet: stretch springs on triangle edges,
                   bending springs across each shared edge
"""
import numpy as np


def rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def box_springs(nx, ny, nz):
    """Endpoints (int32[2E]) and vertex count of createBox(nx, ny, nz).

    Vertex (x,y,z) has index x*ny*nz + y*nz + z; the x edges come first, then
    y, then z, each in x-, y-, z-major loop order, as src/graph.cpp:77-113.
    """
    idx = np.arange(nx * ny * nz, dtype=np.int64).reshape(nx, ny, nz)
    eps = []
    if nx > 1:
        eps.append(np.stack([idx[:-1, :, :], idx[1:, :, :]], -1).reshape(-1, 2))
    if ny > 1:
        eps.append(np.stack([idx[:, :-1, :], idx[:, 1:, :]], -1).reshape(-1, 2))
    if nz > 1:
        eps.append(np.stack([idx[:, :, :-1], idx[:, :, 1:]], -1).reshape(-1, 2))
    ep = np.concatenate(eps, 0) if eps else np.zeros((0, 2), np.int64)
    return ep.reshape(-1).astype(np.int32), nx * ny * nz


def springs_lattice(nx, ny, nz, spacing, jitter, seed):
    """Config-style spring lattice: positions on a jittered grid, rest lengths
    equal to the initial lengths, bottom (z = 0) layer pinned."""
    ep, n = box_springs(nx, ny, nz)
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    x = g.reshape(-1, 3).astype(np.float64) * spacing
    x += rng(seed).uniform(-jitter, jitter, size=x.shape)
    e = ep.reshape(-1, 2)
    l0 = np.linalg.norm(x[e[:, 1]] - x[e[:, 0]], axis=1)
    fixed = (g.reshape(-1, 3)[:, 2] == 0).astype(np.uint8)
    return {"n": n, "x": x.reshape(-1), "ep": ep, "l0": l0, "fixed": fixed}


# Corner labels of a cell: bit 0 -> +x, bit 1 -> +y, bit 2 -> +z.
_EVEN = (0, 3, 5, 6)   # (0,0,0) (1,1,0) (1,0,1) (0,1,1)
_ODD = (1, 2, 4, 7)    # (1,0,0) (0,1,0) (0,0,1) (1,1,1)


def _five_tets(corner_class, center_class):
    tets = [tuple(center_class)]
    for c in corner_class:
        nb = [c ^ 1, c ^ 2, c ^ 4]
        tets.append((c, nb[0], nb[1], nb[2]))
    return np.array(tets, np.int64)


_SPLIT_A = _five_tets(_EVEN, _ODD)
_SPLIT_B = _five_tets(_ODD, _EVEN)


def tet_grid(nx, ny=None, nz=None, disp=0.0, seed=0):
    """Unit-cube lattice of nx*ny*nz cells, 5 tets per cell.

    Vertex (i,j,k) has index (i*(ny+1) + j)*(nz+1) + k and rest position
    (i/nx, j/ny, k/nz).  Tets are listed cell by cell (i-, j-, k-major), and
    every tet is ordered so that det([x0-x3, x1-x3, x2-x3]) < 0, i.e. the rest
    volume W = -det/6 of the reference's precomputeTetMat is positive.
    `disp` adds a seeded uniform displacement in [-disp, disp] to every
    coordinate (the deformed state).
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    V = (nx + 1) * (ny + 1) * (nz + 1)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    corners = np.empty((i.size, 8), np.int64)
    for c in range(8):
        ci, cj, ck = i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1)
        corners[:, c] = (ci * (ny + 1) + cj) * (nz + 1) + ck
    par = ((i + j + k) & 1).astype(bool)
    split = np.where(par[:, None, None], _SPLIT_B[None], _SPLIT_A[None])  # cells x 5 x 4
    tets = np.take_along_axis(corners[:, None, :].repeat(5, 1), split, axis=2).reshape(-1, 4)
    gi, gj, gk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                             indexing="ij")
    X0 = np.stack([gi / nx, gj / ny, gk / nz], -1).reshape(-1, 3).astype(np.float64)
    # orientation from the rest positions
    d = X0[tets[:, :3]] - X0[tets[:, 3:4]]
    det = np.einsum("ti,ti->t", d[:, 0], np.cross(d[:, 1], d[:, 2]))
    flip = det > 0
    tets[flip, 0], tets[flip, 1] = tets[flip, 1].copy(), tets[flip, 0].copy()
    x = X0.copy()
    if disp:
        x += rng(seed).uniform(-disp, disp, size=x.shape)
    return {"n": V, "tets": tets.reshape(-1).astype(np.int32), "X0": X0.reshape(-1),
            "x": x.reshape(-1), "dims": (nx, ny, nz)}


def tet_grid_counts(nx):
    """(tets, vertices) of an nx^3 5-tet lattice."""
    return 5 * nx ** 3, (nx + 1) ** 3


def cloth_sheet(side, seed=0, spacing=None):
    """A side x side vertex sheet in the z = 0 plane.

    Each quad is split into two triangles along alternating diagonals.
    Stretch springs run along every triangle edge (each once); bending
    springs join the two opposite vertices of every pair of triangles that
    share an edge.  Returns positions, spring endpoints (stretch first, then
    bend) and a per-spring flag 1 = bending.
    """
    s = side
    h = 1.0 / (s - 1) if spacing is None else spacing
    gi, gj = np.meshgrid(np.arange(s), np.arange(s), indexing="ij")
    x = np.stack([gi * h, gj * h, np.zeros_like(gi, dtype=np.float64)], -1).reshape(-1, 3)
    vid = lambda a, b: a * s + b  # noqa: E731
    a, b = np.meshgrid(np.arange(s - 1), np.arange(s - 1), indexing="ij")
    a, b = a.reshape(-1), b.reshape(-1)
    v00, v10, v01, v11 = vid(a, b), vid(a + 1, b), vid(a, b + 1), vid(a + 1, b + 1)
    alt = ((a + b) & 1).astype(bool)
    # triangles (t0, t1) per quad
    t0 = np.where(alt[:, None], np.stack([v00, v10, v01], 1), np.stack([v00, v10, v11], 1))
    t1 = np.where(alt[:, None], np.stack([v10, v11, v01], 1), np.stack([v00, v11, v01], 1))
    tris = np.concatenate([t0, t1], 0)
    # edges with their opposite vertex
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], 0)
    opp = np.concatenate([tris[:, 2], tris[:, 0], tris[:, 1]], 0)
    lo, hi = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
    key = lo.astype(np.int64) * (s * s) + hi
    order = np.argsort(key, kind="stable")
    key_s, opp_s = key[order], opp[order]
    uniq, first, counts = np.unique(key_s, return_index=True, return_counts=True)
    stretch = np.stack([uniq // (s * s), uniq % (s * s)], 1)
    shared = counts == 2
    bend = np.stack([opp_s[first[shared]], opp_s[first[shared] + 1]], 1)
    bend = np.sort(bend, 1)
    ep = np.concatenate([stretch, bend], 0).astype(np.int32)
    is_bend = np.concatenate([np.zeros(len(stretch), np.int8), np.ones(len(bend), np.int8)])
    l0 = np.linalg.norm(x[ep[:, 1]] - x[ep[:, 0]], axis=1)
    fixed = np.zeros(s * s, np.uint8)
    fixed[vid(0, 0)] = 1
    fixed[vid(s - 1, 0)] = 1
    return {"n": s * s, "x": x.reshape(-1), "ep": ep.reshape(-1), "is_bend": is_bend,
            "l0": l0, "fixed": fixed}


def cloth_mesh(side, seed=0, height=2.0, half=1.5):
    """A side x side triangle sheet over the square [-half, half]^2 of the
    plane y = height, as the cloth program's face and hinge sets want.

    Each quad is split into two triangles along alternating diagonals, all
    wound the same way.  Each interior edge gives a hinge (a, b, c, d): the
    edge's endpoints a < b, then the vertices opposite it in its first and
    second triangle.  Returns rest positions (n*3), faces (nF*3) and hinges
    (nH*4), all row-major.
    """
    s = side
    t = np.linspace(-half, half, s)
    gi, gj = np.meshgrid(t, t, indexing="ij")
    x = np.stack([gi, np.full_like(gi, height), gj], -1).reshape(-1, 3)
    a, b = np.meshgrid(np.arange(s - 1), np.arange(s - 1), indexing="ij")
    a, b = a.reshape(-1), b.reshape(-1)
    v00, v10, v01, v11 = a * s + b, (a + 1) * s + b, a * s + b + 1, (a + 1) * s + b + 1
    alt = ((a + b) & 1).astype(bool)
    t0 = np.where(alt[:, None], np.stack([v00, v10, v01], 1), np.stack([v00, v10, v11], 1))
    t1 = np.where(alt[:, None], np.stack([v10, v11, v01], 1), np.stack([v00, v11, v01], 1))
    faces = np.concatenate([t0, t1], 0).astype(np.int32)
    # every (edge, opposite vertex) of every face, grouped by the sorted edge
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]], 0)
    opp = np.concatenate([faces[:, 2], faces[:, 0], faces[:, 1]], 0)
    lo, hi = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
    key = lo.astype(np.int64) * (s * s) + hi
    order = np.argsort(key, kind="stable")
    key_s, opp_s = key[order], opp[order]
    uniq, first, counts = np.unique(key_s, return_index=True, return_counts=True)
    inner = counts == 2
    k = uniq[inner]
    hinges = np.stack([k // (s * s), k % (s * s), opp_s[first[inner]], opp_s[first[inner] + 1]],
                      1).astype(np.int32)
    return {"n": s * s, "x": x.reshape(-1), "faces": faces.reshape(-1),
            "hinges": hinges.reshape(-1)}


def _tetgen_records(text, nhead, width):
    """Records of one TetGen file as MeshVol::loadTet / loadTetEdge read them
    (src/mesh.cpp:253-321, 341-373): the first nhead tokens are the header
    (the record count first), the rest of that line is dropped; then lines
    are read while the stream has not hit its end, so a last line without a
    newline is not read; lines shorter than 3 characters and lines starting
    with '#' are skipped; each record drops its leading index and keeps the
    next `width` integers or numbers (width from the header when None).  The
    result has exactly `count` rows, zero-filled past the records present."""
    first, _, rest = text.partition("\n")
    head = first.split()[:nhead]
    count = int(head[0])
    width = int(head[1]) if width is None else width
    segments = rest.split("\n")[:-1]  # the last segment ends at end-of-file
    rows = []
    for ln in segments:
        if len(rows) >= count:
            break
        if len(ln) < 3 or ln[0] == "#":
            continue
        rows.append(ln.split()[1:1 + width])
    return count, width, rows


def parse_tetgen_nodes(text):
    """Vertex positions [n, 3] (float64) of a TetGen .node text."""
    n, _, rows = _tetgen_records(text, 1, 3)
    x = np.zeros((n, 3), np.float64)
    for i, r in enumerate(rows):
        x[i, :len(r)] = [float(t) for t in r]
    return x


def parse_tetgen_elements(text):
    """Element endpoints [nE, per] (int32) of a TetGen .ele text (the
    header's second token is the endpoints per element)."""
    ne, per, rows = _tetgen_records(text, 2, None)
    e = np.zeros((ne, per), np.int32)
    for i, r in enumerate(rows):
        e[i, :len(r)] = [int(t) for t in r]
    return e


def parse_tetgen_edges(text):
    """Edge endpoints [nEdges, 2] (int32) of a TetGen .edge text (boundary
    markers after the two endpoints are ignored)."""
    ne, _, rows = _tetgen_records(text, 1, 2)
    e = np.zeros((ne, 2), np.int32)
    for i, r in enumerate(rows):
        e[i, :len(r)] = [int(t) for t in r]
    return e


def load_tetgen(node_path, ele_path):
    """TetGen .node/.ele files (MeshVol::loadTet): flat positions [n*3] and
    endpoints [nE*per]; indices are kept as written (no 1-based shift)."""
    with open(node_path) as f:
        x = parse_tetgen_nodes(f.read())
    with open(ele_path) as f:
        e = parse_tetgen_elements(f.read())
    return x.reshape(-1), e.reshape(-1)


def load_tetgen_edges(edge_path):
    """TetGen .edge file (MeshVol::loadTetEdge): flat endpoints [nEdges*2],
    the spring set of apps/springs/springs.cpp."""
    with open(edge_path) as f:
        return parse_tetgen_edges(f.read()).reshape(-1)
