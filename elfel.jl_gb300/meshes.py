"""Block meshes (L2, T3, T6, Q4, T4) and node selection.

The reference takes these from MeshSteward 1.1.3 (L2block, T3block, T6block,
T6toT3, Q4block, T4block, boundary/connectedv, vselect; used e.g. at Elfel.jl
test/test_heat.jl:28-33, 143-148 and test/test_stokes.jl:28-39,
examples/heat/poisson/t4.jl:24-30), which is not vendored with it.  The conventions
below follow the reference's mesh fixtures (test/qmesh-conn.dat): nodes are
numbered x-fastest, cells are visited with the x index outer and the y index
inner, and each cell (n1, n2, n3, n4) = ((i,j), (i+1,j), (i+1,j+1), (i,j+1))
is split into [n1, n2, n3] and [n1, n3, n4].

T6 meshes number their nodes on the refined (2nx+1) x (2ny+1) grid, x-fastest,
so that every element's DOFs stay close in number (the SpMV gathers and the
16-bit column compression rely on it).  Midside node k+3 sits on the edge from
vertex k to vertex k+1 (mod 3), as FEH1_T6 expects.  Node numbers are 1-based
in the public arrays, as in the reference.
"""
import numpy as np


class Mesh:
    """Connectivity (nel x nn, 1-based node numbers) plus node coordinates
    (nnodes x sdim: 1 for L2 meshes, 2 for T3/T6/Q4, 3 for T4)."""

    def __init__(self, etype, conn, xy):
        self.etype = etype
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        xy = np.asarray(xy, dtype=np.float64)
        self.xy = np.ascontiguousarray(xy.reshape(xy.shape[0], -1))

    @property
    def sdim(self):
        return self.xy.shape[1]

    @property
    def nel(self):
        return self.conn.shape[0]

    @property
    def nnodes(self):
        return self.xy.shape[0]

    @property
    def nodes_per_elem(self):
        return self.conn.shape[1]

    def __repr__(self):
        return f"Mesh({self.etype}, nel={self.nel}, nnodes={self.nnodes})"


def _cells(nx, ny, orientation):
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")  # x outer, y inner
    i = i.ravel()
    j = j.ravel()
    if orientation == "a":
        flip = np.zeros(i.shape, dtype=bool)
    elif orientation == "alternate":
        flip = ((i + j) % 2) == 1
    else:
        raise ValueError("orientation must be 'a' or 'alternate'")
    return i, j, flip


def T3block(A, B, nx, ny, orientation="a"):
    """nx x ny cells of the rectangle [0,A] x [0,B], 2 T3 per cell.

    orientation 'a': every cell cut on its (i,j)-(i+1,j+1) diagonal;
    'alternate': cells with odd i+j cut on the other diagonal.
    """
    xs = np.linspace(0.0, A, nx + 1)
    ys = np.linspace(0.0, B, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    i, j, flip = _cells(nx, ny, orientation)
    nid = lambda a, b: b * (nx + 1) + a + 1
    n1, n2, n3, n4 = nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)
    t1 = np.where(flip[:, None], np.stack([n1, n2, n4], 1), np.stack([n1, n2, n3], 1))
    t2 = np.where(flip[:, None], np.stack([n2, n3, n4], 1), np.stack([n1, n3, n4], 1))
    conn = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return Mesh("T3", conn, xy)


def T6block(A, B, nx, ny, orientation="a"):
    """T6 version of T3block; midside nodes at the edge midpoints."""
    xv = np.linspace(0.0, A, nx + 1)
    yv = np.linspace(0.0, B, ny + 1)
    xf = np.empty(2 * nx + 1)
    yf = np.empty(2 * ny + 1)
    xf[0::2] = xv
    yf[0::2] = yv
    xf[1::2] = 0.5 * (xv[:-1] + xv[1:])
    yf[1::2] = 0.5 * (yv[:-1] + yv[1:])
    X, Y = np.meshgrid(xf, yf, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    W = 2 * nx + 1
    i, j, flip = _cells(nx, ny, orientation)
    I, J = 2 * i, 2 * j
    fid = lambda a, b: b * W + a + 1
    # fine-grid coordinates of the 4 cell corners
    c1, c2, c3, c4 = (I, J), (I + 2, J), (I + 2, J + 2), (I, J + 2)

    def tri(a, b, c):
        mid = lambda p, q: ((p[0] + q[0]) // 2, (p[1] + q[1]) // 2)
        pts = [a, b, c, mid(a, b), mid(b, c), mid(c, a)]
        return np.stack([fid(*p) for p in pts], axis=1)

    t1 = np.where(flip[:, None], tri(c1, c2, c4), tri(c1, c2, c3))
    t2 = np.where(flip[:, None], tri(c2, c3, c4), tri(c1, c3, c4))
    conn = np.stack([t1, t2], axis=1).reshape(-1, 6)
    return Mesh("T6", conn, xy)


def T6toT3(mesh):
    """Vertex (T3) mesh of a T6 mesh; vertices renumbered in ascending order of
    their T6 node number.  Returns the T3 mesh; ``mesh.vertex_nodes`` holds the
    T6 node number (1-based) of each T3 node."""
    v = np.unique(mesh.conn[:, :3])
    newid = np.zeros(mesh.nnodes + 1, dtype=np.int64)
    newid[v] = np.arange(1, v.size + 1)
    m = Mesh("T3", newid[mesh.conn[:, :3]], mesh.xy[v - 1])
    m.vertex_nodes = v
    return m


def Q4block(A, B, nx, ny):
    """nx x ny bilinear quadrilaterals of [0,A] x [0,B]; cell (i,j) =
    ((i,j), (i+1,j), (i+1,j+1), (i,j+1)) counter-clockwise, cells x outer /
    y inner, nodes x-fastest (the T3block conventions without the split)."""
    xs = np.linspace(0.0, A, nx + 1)
    ys = np.linspace(0.0, B, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    i, j, _ = _cells(nx, ny, "a")
    nid = lambda a, b: b * (nx + 1) + a + 1
    conn = np.stack([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)], axis=1)
    return Mesh("Q4", conn, xy)


def L2block(A, n):
    """n two-node segments of [0, A] on the x axis (1-D coordinates)."""
    x = np.linspace(0.0, A, n + 1).reshape(-1, 1)
    k = np.arange(1, n + 1)
    return Mesh("L2", np.stack([k, k + 1], axis=1), x)


def T4block(A, B, C, nx, ny, nz):
    """nx x ny x nz hexahedral cells of [0,A] x [0,B] x [0,C], each split into
    the six tetrahedra around its (0,0,0)-(1,1,1) diagonal (Kuhn's
    subdivision; every cell split the same way, so faces match).  Nodes
    x-fastest, then y, then z; cells x outer, y, z inner; every tetrahedron
    positively oriented."""
    xs = np.linspace(0.0, A, nx + 1)
    ys = np.linspace(0.0, B, ny + 1)
    zs = np.linspace(0.0, C, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    nid = lambda a, b, c: (c * (ny + 1) + b) * (nx + 1) + a + 1
    unit = np.eye(3, dtype=np.int64)
    tets = []
    # one tetrahedron per permutation (p, q, r) of the axes: the path
    # 0 -> e_p -> e_p + e_q -> (1,1,1); odd permutations swap two vertices
    for (p, q, r), odd in (((0, 1, 2), 0), ((0, 2, 1), 1), ((1, 0, 2), 1), ((1, 2, 0), 0), ((2, 0, 1), 0),
                           ((2, 1, 0), 1)):
        o = np.zeros(3, dtype=np.int64)
        a = unit[p]
        b = unit[p] + unit[q]
        d = np.ones(3, dtype=np.int64)
        vs = [nid(i + v[0], j + v[1], k + v[2]) for v in (o, a, b, d)]
        if odd:
            vs[1], vs[2] = vs[2], vs[1]
        tets.append(np.stack(vs, axis=1))
    conn = np.stack(tets, axis=1).reshape(-1, 4)
    return Mesh("T4", conn, xyz)


# Local boundary features of each cell: edges of 2-D cells, faces of
# tetrahedra, end points of segments.  T6 edges list their midside node third.
_FACETS = {
    "L2": [[0], [1]],
    "T3": [[0, 1], [1, 2], [2, 0]],
    "T6": [[0, 1, 3], [1, 2, 4], [2, 0, 5]],
    "Q4": [[0, 1], [1, 2], [2, 3], [3, 0]],
    "T4": [[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]],
}


def _facets(mesh):
    """(facet vertex keys, all facet nodes) of every (cell, local facet), local facet outer."""
    fl = _FACETS[mesh.etype]
    c = mesh.conn
    nv = 2 if mesh.etype == "T6" else len(fl[0])
    nodes = np.concatenate([c[:, f] for f in fl], axis=0)
    return np.sort(nodes[:, :nv], axis=1), nodes


def _single(key):
    """Mask of the rows of key that occur once (lexicographic sort of the rows)."""
    if key.shape[0] == 0:
        return np.zeros(0, dtype=bool)
    order = np.lexsort(key.T[::-1])
    ks = key[order]
    start = np.concatenate([[True], np.any(ks[1:] != ks[:-1], axis=1)])
    grp = np.cumsum(start) - 1
    cnt = np.bincount(grp)
    once = np.empty(key.shape[0], dtype=bool)
    once[order] = cnt[grp] == 1
    return once


def boundary_nodes(mesh):
    """Nodes on facets used by exactly one cell (connectedv(boundary(mesh))), 1-based, ascending."""
    key, nodes = _facets(mesh)
    return np.unique(nodes[_single(key)].ravel())


def boundary_edges(mesh):
    """(element, local facet) pairs, 1-based, of the facets used by one element only."""
    key, _ = _facets(mesh)
    on = np.nonzero(_single(key))[0]
    nel = mesh.nel
    return np.stack([on % nel + 1, on // nel + 1], axis=1).astype(np.int64)


def vselect(xy, box, inflate=0.0):
    """Nodes inside box = [xmin, xmax, ymin, ymax(, zmin, zmax)] grown by inflate (1-based)."""
    b = np.asarray(box, dtype=np.float64).ravel()
    xy = np.asarray(xy).reshape(len(xy), -1)
    ok = np.ones(xy.shape[0], dtype=bool)
    for d in range(min(xy.shape[1], b.size // 2)):
        ok &= (xy[:, d] >= b[2 * d] - inflate) & (xy[:, d] <= b[2 * d + 1] + inflate)
    return np.nonzero(ok)[0] + 1


def vselect_nearest(xy, point):
    """Node nearest to point (1-based)."""
    d = np.sum((xy - np.asarray(point, dtype=np.float64)[None, :]) ** 2, axis=1)
    return int(np.argmin(d)) + 1


def jitter(mesh, amount, seed, curved=False):
    """Move interior vertex nodes by a seeded uniform offset in [-amount, amount]^sdim.

    T6 midside nodes are then put back at the midpoints of their (moved)
    edges, which keeps the elements straight-sided; curved=True jitters the
    interior midside nodes as well (isoparametric, curved elements).
    """
    rng = np.random.default_rng(seed)
    xy = mesh.xy.copy()
    bnd = np.zeros(mesh.nnodes, dtype=bool)
    bnd[boundary_nodes(mesh) - 1] = True
    nv = 3 if mesh.etype == "T6" else mesh.nodes_per_elem
    verts = np.unique(mesh.conn[:, :nv]) - 1
    inner = verts[~bnd[verts]]
    xy[inner] += rng.uniform(-amount, amount, size=(inner.size, mesh.sdim))
    if mesh.nodes_per_elem == 6:
        c = mesh.conn - 1
        for k in range(3):
            a, b, m = c[:, k], c[:, (k + 1) % 3], c[:, 3 + k]
            xy[m] = 0.5 * (xy[a] + xy[b])
        if curved:
            mids = np.unique(c[:, 3:6])
            mids = mids[~bnd[mids]]
            xy[mids] += rng.uniform(-amount, amount, size=(mids.size, 2))
    return Mesh(mesh.etype, mesh.conn, xy)
