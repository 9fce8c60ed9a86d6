"""Host-side meshes for the device path: quadrilateral meshes as
``Mesh2D::from_quads`` takes them (vertices, counter-clockwise element
corners, periodic face pairs, one tag per boundary face), their node
positions, and the seeded generators of the workloads.

The generators follow the reference's (src/mesh/core/mesh2d.rs:309-420):
``uniform_rectangle`` numbers vertices row by row from the bottom left and
tags a boundary face with the side its face number names (face 0 south,
1 east, 2 north, 3 west); ``uniform_periodic`` pairs the right face of each
row's last element with the left face of its first, and the top faces of
the top row with the bottom faces of the bottom row."""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# BoundaryTag (src/mesh/data/boundary_tags.rs:8-34) as the ABI's face tags:
# the variants in declaration order (Periodic, 3, is a face pairing here,
# not a tag), and Custom(n) as CUSTOM_TAG_BASE + n
TAG_WALL, TAG_OPEN, TAG_TIDAL, TAG_RIVER, TAG_DIRICHLET, TAG_NEUMANN = 0, 1, 2, 4, 5, 6
CUSTOM_TAG_BASE = 1000


def custom_tag(n: int) -> int:
    """The face tag of BoundaryTag::Custom(n)."""
    return CUSTOM_TAG_BASE + int(n)


@dataclass
class QuadMesh:
    vertices: np.ndarray  # (n_vertices, 2) float64
    elements: np.ndarray  # (n_elements, 4) int64, counter-clockwise
    periodic: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int64))
    face_tags: np.ndarray | None = None  # (n_elements, 4) int32

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])

    def corners(self) -> np.ndarray:
        """(n_elements, 4, 2) corner coordinates."""
        return self.vertices[self.elements]


def _legendre_pd(n: int, x: float) -> tuple[float, float]:
    # P_n and P_n' by the three-term recurrence (src/polynomial/legendre.rs:62-94)
    if n == 0:
        return 1.0, 0.0
    if n == 1:
        return x, 1.0
    pm, pc = 1.0, x
    for k in range(1, n):
        pn = (float(2 * k + 1) * x * pc - float(k) * pm) / float(k + 1)
        pm, pc = pc, pn
    if abs(x - 1.0) < 1e-14:
        dp = float(n * (n + 1)) / 2.0
    elif abs(x + 1.0) < 1e-14:
        dp = (1.0 if n % 2 else -1.0) * float(n * (n + 1)) / 2.0
    else:
        dp = float(n) * (x * pc - pm) / (x * x - 1.0)
    return pc, dp


def gll_nodes(order: int) -> np.ndarray:
    """GLL nodes by Newton from the Chebyshev–Lobatto points
    (src/polynomial/nodes.rs:17-77); the same values as the library's."""
    n = order
    x = [-math.cos(math.pi * j / n) for j in range(n + 1)]
    x[0], x[n] = -1.0, 1.0
    for j in range(1, n):
        xj = x[j]
        for _ in range(100):
            p, dp = _legendre_pd(n, xj)
            step = (1.0 - xj * xj) * dp / (float(n) * float(n + 1) * p)
            if abs(step) < 1e-15:
                break
            xj += step
        x[j] = xj
    return np.array(x)


def gll_weights(order: int) -> np.ndarray:
    n = order
    return np.array([2.0 / (float(n * (n + 1)) * _legendre_pd(n, xj)[0] ** 2)
                     for xj in gll_nodes(order)])


def reference_nodes(order: int) -> tuple[np.ndarray, np.ndarray]:
    """(r, s) of the element nodes, node i = j·(N+1) + a, r fastest."""
    x = gll_nodes(order)
    n1 = order + 1
    r = np.tile(x, n1)
    s = np.repeat(x, n1)
    return r, s


def node_positions(mesh: QuadMesh, order: int) -> tuple[np.ndarray, np.ndarray]:
    """Physical (x, y) of every node, (n_elements, (N+1)²) each, by the
    bilinear map of Mesh2D::bilinear (src/mesh/core/mesh2d.rs:644-660)."""
    r, s = reference_nodes(order)
    c = mesh.corners()
    n0 = (1.0 - r) * (1.0 - s) / 4.0
    n1 = (1.0 + r) * (1.0 - s) / 4.0
    n2 = (1.0 + r) * (1.0 + s) / 4.0
    n3 = (1.0 - r) * (1.0 + s) / 4.0
    x = (n0 * c[:, 0:1, 0] + n1 * c[:, 1:2, 0]) + n2 * c[:, 2:3, 0] + n3 * c[:, 3:4, 0]
    y = (n0 * c[:, 0:1, 1] + n1 * c[:, 1:2, 1]) + n2 * c[:, 2:3, 1] + n3 * c[:, 3:4, 1]
    return x, y


def _structured(x0, x1, y0, y1, nx, ny):
    # structured_quads (src/mesh/core/mesh2d.rs:226-254)
    dx = (x1 - x0) / nx
    dy = (y1 - y0) / ny
    i = np.arange(nx + 1, dtype=np.float64)
    j = np.arange(ny + 1, dtype=np.float64)
    vx = np.tile(x0 + i * dx, ny + 1)
    vy = np.repeat(y0 + j * dy, nx + 1)
    verts = np.stack([vx, vy], axis=1)
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    v0 = (jj * (nx + 1) + ii).ravel().astype(np.int64)
    elems = np.stack([v0, v0 + 1, v0 + nx + 2, v0 + nx + 1], axis=1)
    return verts, elems


def uniform_rectangle(x0, x1, y0, y1, nx, ny, sides=(TAG_WALL,) * 4) -> QuadMesh:
    """Mesh2D::uniform_rectangle_with_sides: ``sides`` are the tags of the
    [south, east, north, west] sides."""
    verts, elems = _structured(x0, x1, y0, y1, nx, ny)
    tags = np.tile(np.array(sides, dtype=np.int32), (nx * ny, 1))
    return QuadMesh(verts, elems, np.zeros((0, 4), np.int64), tags)


def uniform_periodic(x0, x1, y0, y1, nx, ny) -> QuadMesh:
    """Mesh2D::uniform_periodic (src/mesh/core/mesh2d.rs:398-414)."""
    verts, elems = _structured(x0, x1, y0, y1, nx, ny)
    pairs = [(j * nx + nx - 1, 1, j * nx, 3) for j in range(ny)]
    pairs += [((ny - 1) * nx + i, 2, i, 0) for i in range(nx)]
    return QuadMesh(verts, elems, np.array(pairs, np.int64).reshape(-1, 4),
                    np.zeros((nx * ny, 4), np.int32))


def channel_periodic_x(x0, x1, y0, y1, nx, ny, south=TAG_WALL, north=TAG_WALL) -> QuadMesh:
    """Mesh2D::channel_periodic_x_with_sides (src/mesh/core/mesh2d.rs:365-393)."""
    verts, elems = _structured(x0, x1, y0, y1, nx, ny)
    pairs = [(j * nx + nx - 1, 1, j * nx, 3) for j in range(ny)]
    tags = np.zeros((nx * ny, 4), np.int32)
    tags[:, 0] = south
    tags[:, 2] = north
    return QuadMesh(verts, elems, np.array(pairs, np.int64).reshape(-1, 4), tags)


def move_vertices(mesh: QuadMesh, fn) -> QuadMesh:
    """The mesh with every vertex moved to fn(x, y) (vectorised)."""
    x, y = fn(mesh.vertices[:, 0], mesh.vertices[:, 1])
    return QuadMesh(np.stack([x, y], axis=1), mesh.elements, mesh.periodic, mesh.face_tags)


def hilbert_index(x: np.ndarray, y: np.ndarray, bits: int) -> np.ndarray:
    """Position of the cells (x, y) of a 2^bits grid along the Hilbert curve
    (src/mesh/core/mesh2d.rs:112-132), vectorised."""
    x = x.astype(np.uint64).copy()
    y = y.astype(np.uint64).copy()
    d = np.zeros_like(x)
    s = np.uint64(1 << (bits - 1))
    while s > 0:
        rx = (x & s) != 0
        ry = (y & s) != 0
        d += s * s * ((np.uint64(3) * rx.astype(np.uint64)) ^ ry.astype(np.uint64))
        x &= s - np.uint64(1)
        y &= s - np.uint64(1)
        flip = (~ry) & rx
        x = np.where(flip, s - np.uint64(1) - x, x)
        y = np.where(flip, s - np.uint64(1) - y, y)
        swap = ~ry
        x, y = np.where(swap, y, x), np.where(swap, x, y)
        s = np.uint64(int(s) >> 1)
    return d


def in_hilbert_order(mesh: QuadMesh) -> tuple[QuadMesh, np.ndarray]:
    """The mesh with its elements along a Hilbert curve through their
    centroids and its vertices numbered by first use in that order
    (Mesh2D::in_hilbert_order and select_elements,
    src/mesh/core/mesh2d.rs:711-790), and for each new element its old
    index. One scale for both directions (square cells of a 2^16 grid over
    the centroids' larger extent); equal keys keep the old order. Periodic
    pairs are renumbered."""
    p = mesh.corners()
    c = 0.25 * (((p[:, 0] + p[:, 1]) + p[:, 2]) + p[:, 3])
    lo, hi = c.min(axis=0), c.max(axis=0)
    extent = float((hi - lo).max()) if c.size else 0.0
    scale = 65535.0 / extent if extent > 0.0 else 0.0
    cells = ((c - lo) * scale).astype(np.int64)  # truncation toward zero, as `as u32`
    order = np.argsort(hilbert_index(cells[:, 0], cells[:, 1], 16), kind="stable")
    new_of_old = np.empty_like(order)
    new_of_old[order] = np.arange(order.size)
    periodic = mesh.periodic.copy()
    if periodic.size:
        periodic[:, 0] = new_of_old[periodic[:, 0]]
        periodic[:, 2] = new_of_old[periodic[:, 2]]
    tags = None if mesh.face_tags is None else mesh.face_tags[order]
    elements = mesh.elements[order]
    used, first = np.unique(elements.reshape(-1), return_index=True)
    by_use = used[np.argsort(first, kind="stable")]
    new_vertex = np.full(mesh.vertices.shape[0], -1, np.int64)
    new_vertex[by_use] = np.arange(by_use.size)
    return (QuadMesh(mesh.vertices[by_use], new_vertex[elements], periodic, tags), order)


def graded_jittered_box(lx: float, ly: float, nx: int, ny: int, size_range=(100.0, 400.0),
                        jitter: float = 0.15, seed: int = 0,
                        sides=(TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN)) -> QuadMesh:
    """A synthetic unstructured-like quad paving of [0, lx]×[0, ly]: a
    tensor grid whose column widths and row heights are graded smoothly
    within ``size_range`` (so the aspect ratio stays below max/min), its
    interior vertices jittered by up to ``jitter`` × the local size with a
    seeded generator. The element corners stay counter-clockwise and the
    Jacobians positive (jitter < ¼)."""
    rng = np.random.default_rng(seed)

    def graded(length, n, phase):
        t = (np.arange(n) + 0.5) / n
        lo, hi = size_range
        w = lo + (hi - lo) * 0.5 * (1.0 + np.sin(2.0 * np.pi * (1.7 * t + phase)))
        w = w * (length / w.sum())
        edges = np.concatenate([[0.0], np.cumsum(w)])
        edges[-1] = length
        return edges, w

    ex, wx = graded(lx, nx, rng.uniform())
    ey, wy = graded(ly, ny, rng.uniform())
    vx = np.tile(ex, ny + 1)
    vy = np.repeat(ey, nx + 1)
    # local size at each vertex: the smaller neighbouring width/height
    sx = np.minimum(np.concatenate([[wx[0]], wx]), np.concatenate([wx, [wx[-1]]]))
    sy = np.minimum(np.concatenate([[wy[0]], wy]), np.concatenate([wy, [wy[-1]]]))
    lx_loc = np.tile(sx, ny + 1)
    ly_loc = np.repeat(sy, nx + 1)
    ii = np.tile(np.arange(nx + 1), ny + 1)
    jj = np.repeat(np.arange(ny + 1), nx + 1)
    interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
    dx = rng.uniform(-jitter, jitter, vx.size) * lx_loc
    dy = rng.uniform(-jitter, jitter, vy.size) * ly_loc
    vx = np.where(interior, vx + dx, vx)
    vy = np.where(interior, vy + dy, vy)
    verts = np.stack([vx, vy], axis=1)
    jg, ig = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    v0 = (jg * (nx + 1) + ig).ravel().astype(np.int64)
    elems = np.stack([v0, v0 + 1, v0 + nx + 2, v0 + nx + 1], axis=1)
    tags = np.tile(np.array(sides, dtype=np.int32), (nx * ny, 1))
    return QuadMesh(verts, elems, np.zeros((0, 4), np.int64), tags)


# -- quadtree paving -------------------------------------------------------
#
# An unstructured all-quad mesh of a box with a graded element size: a
# 2:1-balanced quadtree of square-ish cells whose leaf level follows a
# requested level field, each leaf fanned into triangles from its centre
# (one triangle per leaf edge, or two where a finer neighbour puts a hanging
# vertex at the edge's midpoint), and every triangle split into three quads
# through its centroid and edge midpoints. The mesh is conforming (every
# triangle edge's midpoint is shared by both sides), its vertices have
# valence 3 (centroids), 4 (edge midpoints) or 4–8 (cell corners and
# centres), and the quads of one triangle have equal areas. Leaves of
# level l hold quads of √area ≈ 0.289·C_l (0.204·C_l beside a finer
# neighbour), C_l the leaf's side.


def quadtree_levels(desired: np.ndarray, max_level: int) -> np.ndarray:
    """Leaf level of every finest cell of a quadtree over ``desired`` (an
    (ny, nx) field of requested levels 0..max_level on the finest grid,
    both sides multiples of 2^max_level): a block is split while any cell
    in it asks for a finer level, and then leaves are refined until edge
    neighbours differ by at most one level (2:1 balance)."""
    want = np.asarray(desired, np.int64)
    ny, nx = want.shape
    step = 1 << max_level
    if ny % step or nx % step:
        raise ValueError("the finest grid must hold whole root cells")

    def quantised(d):
        level = np.zeros_like(d)
        for lv in range(max_level):
            b = 1 << (max_level - lv)
            split = d.reshape(ny // b, b, nx // b, b).max(axis=(1, 3)) > lv
            level = np.where(np.repeat(np.repeat(split, b, axis=0), b, axis=1),
                             np.maximum(level, lv + 1), level)
        return level

    level = quantised(want)
    for _ in range(4 * max_level + 4):
        around = level.copy()
        around[1:, :] = np.maximum(around[1:, :], level[:-1, :])
        around[:-1, :] = np.maximum(around[:-1, :], level[1:, :])
        around[:, 1:] = np.maximum(around[:, 1:], level[:, :-1])
        around[:, :-1] = np.maximum(around[:, :-1], level[:, 1:])
        coarse = level < around - 1
        if not coarse.any():
            return level
        want = np.maximum(np.where(coarse, around - 1, want), level)
        level = quantised(want)
    raise RuntimeError("quadtree balance did not settle")


def _leaf_triangles(level: np.ndarray, max_level: int) -> np.ndarray:
    """(n, 6) integer triangles (centre, then two boundary points, counter-
    clockwise) of every leaf's fan, in half-finest-cell units."""
    ny, nx = level.shape
    out = []
    for lv in range(max_level + 1):
        b = 1 << (max_level - lv)
        jj, ii = np.nonzero(level[::b, ::b] == lv)
        i0, j0 = ii * b, jj * b

        def finer(i, j, inside):
            hit = np.zeros(i.size, bool)
            hit[inside] = level[j[inside], i[inside]] > lv
            return hit

        # a finer leaf across an edge puts a vertex at the edge's midpoint
        split = (finer(i0, j0 - 1, j0 > 0), finer(i0 + b, j0, i0 + b < nx),
                 finer(i0, j0 + b, j0 + b < ny), finer(i0 - 1, j0, i0 > 0))
        x0, y0, h = 2 * i0, 2 * j0, b
        ring = ((x0, y0), (x0 + h, y0), (x0 + 2 * h, y0), (x0 + 2 * h, y0 + h),
                (x0 + 2 * h, y0 + 2 * h), (x0 + h, y0 + 2 * h), (x0, y0 + 2 * h), (x0, y0 + h))
        code = split[0] * 1 + split[1] * 2 + split[2] * 4 + split[3] * 8
        for c in np.unique(code):
            sel = code == c
            seq = [k for k in range(8) if k % 2 == 0 or (c >> (k // 2)) & 1]
            for a, z in zip(seq, seq[1:] + seq[:1]):
                out.append(np.stack([x0[sel] + h, y0[sel] + h, ring[a][0][sel], ring[a][1][sel],
                                     ring[z][0][sel], ring[z][1][sel]], axis=1))
    return np.concatenate(out).astype(np.int64)


def quadtree_paving(lx: float, ly: float, desired: np.ndarray, max_level: int,
                    sides=(TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN), jitter: float = 0.1,
                    seed: int = 0, smoothing: int = 1) -> QuadMesh:
    """The quadtree paving of [0, lx]×[0, ly] for the requested level field
    ``desired`` ((ny, nx) on the finest grid; see :func:`quadtree_levels`).
    Interior vertices get ``smoothing`` Laplacian passes, then a seeded
    jitter of up to ``jitter`` × their shortest edge in each coordinate;
    boundary vertices stay on the sides. ``sides`` tag the [south, east,
    north, west] boundary faces. Raises if a Jacobian is not positive."""
    level = quadtree_levels(desired, max_level)
    ny, nx = level.shape
    tri = _leaf_triangles(level, max_level) * 6  # 1/12 of a finest cell
    a, b, c = tri[:, 0:2], tri[:, 2:4], tri[:, 4:6]
    ab, bc, ca = (a + b) // 2, (b + c) // 2, (c + a) // 2
    g = (a + b + c) // 3
    quads = np.stack([np.stack([a, ab, g, ca], 1), np.stack([b, bc, g, ab], 1),
                      np.stack([c, ca, g, bc], 1)], 1).reshape(-1, 4, 2)
    top_x, top_y = 12 * nx, 12 * ny
    key = quads[..., 0] * (top_y + 1) + quads[..., 1]
    unique, inverse = np.unique(key, return_inverse=True)
    elements = inverse.reshape(-1, 4).astype(np.int64)
    ix, iy = unique // (top_y + 1), unique % (top_y + 1)
    on_side = (iy == 0, ix == top_x, iy == top_y, ix == 0)
    boundary = on_side[0] | on_side[1] | on_side[2] | on_side[3]
    tags = np.zeros(elements.shape, np.int32)
    for f in range(4):
        p, q = elements[:, f], elements[:, (f + 1) % 4]
        for side in range(4):
            tags[on_side[side][p] & on_side[side][q], f] = sides[side]
    verts = np.stack([ix * (lx / top_x), iy * (ly / top_y)], axis=1)
    e0 = elements.reshape(-1)
    e1 = np.roll(elements, -1, axis=1).reshape(-1)
    for _ in range(smoothing):
        total = np.zeros_like(verts)
        count = np.zeros(verts.shape[0])
        np.add.at(total, e0, verts[e1])
        np.add.at(total, e1, verts[e0])
        np.add.at(count, e0, 1.0)
        np.add.at(count, e1, 1.0)
        verts = np.where(boundary[:, None], verts, total / count[:, None])
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        shortest = np.full(verts.shape[0], np.inf)
        edge = np.linalg.norm(verts[e1] - verts[e0], axis=1)
        np.minimum.at(shortest, e0, edge)
        np.minimum.at(shortest, e1, edge)
        moved = verts + rng.uniform(-jitter, jitter, verts.shape) * shortest[:, None]
        verts = np.where(boundary[:, None], verts, moved)
    mesh = QuadMesh(verts, elements, np.zeros((0, 4), np.int64), tags)
    if corner_jacobians(mesh).min() <= 0.0:
        raise RuntimeError("quadtree paving: a Jacobian is not positive")
    return mesh


def corner_jacobians(mesh: QuadMesh) -> np.ndarray:
    """(n_elements, 4) cross products of the two edges at each corner; a
    bilinear quad's Jacobian is positive everywhere when these are."""
    p = mesh.corners()
    nxt = np.roll(p, -1, axis=1) - p
    prv = np.roll(p, 1, axis=1) - p
    return nxt[..., 0] * prv[..., 1] - nxt[..., 1] * prv[..., 0]


def element_shape(mesh: QuadMesh) -> tuple[np.ndarray, np.ndarray]:
    """(√area, stretch) of every element: the stretch is the ratio of the
    singular values of the bilinear map's Jacobian at the element centre
    (1 for a square, the side ratio for a rectangle)."""
    p = mesh.corners()
    xr = 0.5 * ((p[:, 1] - p[:, 0]) + (p[:, 2] - p[:, 3]))
    xs = 0.5 * ((p[:, 3] - p[:, 0]) + (p[:, 2] - p[:, 1]))
    sv = np.linalg.svd(np.stack([xr, xs], axis=2), compute_uv=False)
    nxt = np.roll(p, -1, axis=1)
    area = 0.5 * np.abs((p[..., 0] * nxt[..., 1] - nxt[..., 0] * p[..., 1]).sum(axis=1))
    return np.sqrt(area), sv[:, 0] / sv[:, 1]


def node_mass(mesh: QuadMesh, order: int) -> np.ndarray:
    """GLL weight × J at every node, (n_elements, (N+1)²): the diagonal mass
    matrix of GeometricFactors2D::compute (src/operators/geometric.rs:160-176)."""
    r, s = reference_nodes(order)
    w = gll_weights(order)
    n1 = order + 1
    w2 = np.tile(w, n1) * np.repeat(w, n1)  # w_r · w_s at node j·n1 + a
    c = mesh.corners()
    x0, y0, x1, y1 = c[:, 0:1, 0], c[:, 0:1, 1], c[:, 1:2, 0], c[:, 1:2, 1]
    x2, y2, x3, y3 = c[:, 2:3, 0], c[:, 2:3, 1], c[:, 3:4, 0], c[:, 3:4, 1]
    x_r = 0.25 * ((1.0 - s) * (x1 - x0) + (1.0 + s) * (x2 - x3))
    y_r = 0.25 * ((1.0 - s) * (y1 - y0) + (1.0 + s) * (y2 - y3))
    x_s = 0.25 * ((1.0 - r) * (x3 - x0) + (1.0 + r) * (x2 - x1))
    y_s = 0.25 * ((1.0 - r) * (y3 - y0) + (1.0 + r) * (y2 - y1))
    return w2 * (x_r * y_s - x_s * y_r)
