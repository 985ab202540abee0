"""Deterministic synthetic meshes for the PFEM-2 workloads, plus SALOME DAT I/O.

The reference reads meshes in the SALOME DAT format (``Mesh2D::loadMeshFromFile``,
src/mesh_2d.cu:36-96): a header ``nV nE``, then ``id x y z`` per vertex (1-based ids),
then ``id type v...`` per entity, where type 203 is a triangle (3 vertex ids) and
102 a boundary edge (2 vertex ids).  The reference parser appends a spurious
triangle when the file ends with a newline (its ``while(!eof)`` loop,
src/mesh_2d.cu:56-72), so :func:`write_dat` never emits one.

Workloads (all triangles counter-clockwise, every quad split along its
lower-left/upper-right diagonal):

* ``unit_square(64)``      - 64x64 quads on [0,1]^2, 8,192 triangles, 4,225 nodes,
  no jitter (the 2D Poisson problem).
* ``channel()``            - [0,4]x[0,1], 256x64 quads, 32,768 triangles, 16,705 nodes,
  interior nodes jittered by at most 0.2h (splitmix64, seed 0).
* ``cylinder_channel()``   - [0,2.2]x[0,0.41] with a cylinder of radius 0.05 at
  (0.2,0.2): a structured O-grid ring (600 x 24 quads) inside the box
  [0.1,0.3]^2 and a quad-split Cartesian far field (hx=1/700, hy=1/800) outside it;
  994,240 triangles, 499,288 nodes, jitter <= 0.2h on interior nodes.
* ``refine_uniform(...)``  - 1:4 red refinement (edge midpoints), used for the
  3,976,960-triangle refinement of the cylinder mesh.

Jitter is drawn per interior node in final node-index order from a splitmix64
stream, two uniforms per node, each mapped to [-1, 1) and scaled by 0.2 x the local
spacing.  Coordinates are written with ``%.17g``, which round-trips IEEE doubles exactly, so a
mesh written and re-read has bit-identical coordinates.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """``count`` consecutive outputs of the splitmix64 generator started at ``seed``."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform_pm1(seed: int, count: int) -> np.ndarray:
    """Uniform doubles in [-1, 1) from the top 53 bits of splitmix64 outputs."""
    u = (splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


def _split_quads(ll, lr, ur, ul):
    """Two CCW triangles per quad (lower-left, lower-right, upper-right, upper-left)."""
    t1 = np.stack([ll, lr, ur], axis=-1)
    t2 = np.stack([ll, ur, ul], axis=-1)
    return np.concatenate([t1.reshape(-1, 3), t2.reshape(-1, 3)], axis=0)


def _orient_ccw(xy, tri):
    a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
    cr = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    neg = cr < 0
    tri = tri.copy()
    tri[neg, 1], tri[neg, 2] = tri[neg, 2].copy(), tri[neg, 1].copy()
    return tri


def _renumber(xy, tri, key_nodes, boundary_mask, jitter_scale, seed):
    """Renumber nodes by ``key_nodes`` (lexsort keys), cells by their sorted vertex ids,
    then jitter interior nodes in the new node order."""
    order = np.lexsort(key_nodes)
    inv = np.empty_like(order)
    inv[order] = np.arange(order.size)
    xy = xy[order]
    boundary_mask = boundary_mask[order]
    jitter_scale = jitter_scale[order] if np.ndim(jitter_scale) else jitter_scale
    tri = inv[tri]
    s = np.sort(tri, axis=1)
    corder = np.lexsort((s[:, 2], s[:, 1], s[:, 0]))
    tri = tri[corder]
    interior = np.nonzero(~boundary_mask)[0]
    if seed is not None and interior.size and np.any(jitter_scale):
        r = uniform_pm1(seed, 2 * interior.size).reshape(-1, 2)
        sc = jitter_scale[interior] if np.ndim(jitter_scale) else jitter_scale
        xy = xy.copy()
        xy[interior] += 0.2 * r * (sc[:, None] if np.ndim(sc) else sc)
    return xy, tri


def structured_rectangle(nx, ny, lx, ly, jitter=0.0, seed=0):
    """Quad-split structured grid on [0,lx]x[0,ly]; node order is column-major (y fastest)."""
    i, j = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    x = lx * i.astype(np.float64) / nx
    y = ly * j.astype(np.float64) / ny
    xy = np.stack([x.ravel(), y.ravel()], axis=1)
    nid = (i * (ny + 1) + j)
    ll = nid[:-1, :-1]
    lr = nid[1:, :-1]
    ur = nid[1:, 1:]
    ul = nid[:-1, 1:]
    tri = _split_quads(ll.ravel(), lr.ravel(), ur.ravel(), ul.ravel()).astype(np.int64)
    bnd = ((i == 0) | (i == nx) | (j == 0) | (j == ny)).ravel()
    h = min(lx / nx, ly / ny)
    key = (xy[:, 1], np.rint(xy[:, 0] / (lx / nx)))
    xy, tri = _renumber(xy, tri, key, bnd, h if jitter else 0.0, seed if jitter else None)
    return xy, tri.astype(np.int32)


def unit_square(n: int = 64):
    """The unit-square Poisson mesh: n x n quads, 2 triangles each, no jitter."""
    return structured_rectangle(n, n, 1.0, 1.0, jitter=0.0)


def channel(nx: int = 256, ny: int = 64, lx: float = 4.0, ly: float = 1.0, seed: int = 0):
    """The 4x1 channel: 256 x 64 quads with interior jitter <= 0.2h (seed 0)."""
    return structured_rectangle(nx, ny, lx, ly, jitter=0.2, seed=seed)


def cylinder_channel(seed: int = 0, nxh: int = 700, nyh: int = 800, nr: int = 24,
                     box=(0.1, 0.3, 0.1, 0.3), center=(0.2, 0.2), radius=0.05,
                     lx: float = 2.2, ly: float = 0.41, first_layer: float = 0.06,
                     jitter: bool = True):
    """Channel-with-cylinder mesh (about 1.0M triangles at the defaults).

    The far field is a Cartesian grid with spacing hx = 1/nxh, hy = 1/nyh (quad split);
    the box ``[bx0,bx1]x[by0,by1]`` around the cylinder holds an O-grid ring whose
    outer nodes are the Cartesian nodes on the box perimeter and whose inner nodes lie
    on the circle along the same rays.  The first radial layer takes ``first_layer`` of
    each ray (0.003-0.0055 here), so radial edge midpoints stay farther than 0.001
    from the circle, the body-edge tolerance the flow driver uses.
    """
    hx, hy = 1.0 / nxh, 1.0 / nyh
    NX = int(round(lx / hx))
    NY = int(round(ly / hy))
    bi0, bi1 = int(round(box[0] / hx)), int(round(box[1] / hx))
    bj0, bj1 = int(round(box[2] / hy)), int(round(box[3] / hy))
    # Cartesian nodes outside the open box
    i, j = np.meshgrid(np.arange(NX + 1), np.arange(NY + 1), indexing="ij")
    inside = (i > bi0) & (i < bi1) & (j > bj0) & (j < bj1)
    keep = ~inside
    cid = -np.ones((NX + 1, NY + 1), dtype=np.int64)
    cid[keep] = np.arange(int(keep.sum()))
    cx = lx * i[keep].astype(np.float64) / NX
    cy = ly * j[keep].astype(np.float64) / NY
    xy_c = np.stack([cx, cy], axis=1)
    qi, qj = np.meshgrid(np.arange(NX), np.arange(NY), indexing="ij")
    qkeep = ~((qi >= bi0) & (qi < bi1) & (qj >= bj0) & (qj < bj1))
    qi, qj = qi[qkeep], qj[qkeep]
    tri_c = _split_quads(cid[qi, qj], cid[qi + 1, qj], cid[qi + 1, qj + 1], cid[qi, qj + 1])
    bnd_c = ((i[keep] == 0) | (i[keep] == NX) | (j[keep] == 0) | (j[keep] == NY))
    sc_c = np.full(xy_c.shape[0], min(hx, hy))
    # box perimeter, counter-clockwise from the lower-left corner
    per = []
    per += [(ii, bj0) for ii in range(bi0, bi1)]
    per += [(bi1, jj) for jj in range(bj0, bj1)]
    per += [(ii, bj1) for ii in range(bi1, bi0, -1)]
    per += [(bi0, jj) for jj in range(bj1, bj0, -1)]
    per = np.array(per)
    nth = per.shape[0]
    P = xy_c[cid[per[:, 0], per[:, 1]]]
    C = np.array(center)
    d = P - C
    # inner nodes along the rays (IEEE-exact operations only, so the mesh is the same bits
    # on every platform: no libm trigonometry)
    dn = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1])
    Q = C + radius * (d / dn[:, None])
    w = np.concatenate([[0.0], first_layer + (1.0 - first_layer) * np.arange(nr) / (nr - 1)])
    # ring layers k = 0..nr-1 are new nodes; layer nr is the perimeter
    ring_xy = (1.0 - w[:nr, None, None]) * Q[None] + w[:nr, None, None] * P[None]
    nbase = xy_c.shape[0]
    rid = np.empty((nr + 1, nth), dtype=np.int64)
    rid[:nr] = nbase + np.arange(nr * nth).reshape(nr, nth)
    rid[nr] = cid[per[:, 0], per[:, 1]]
    k = np.arange(nth)
    kp = (k + 1) % nth
    ll = rid[:-1][:, k]
    lr = rid[:-1][:, kp]
    ur = rid[1:][:, kp]
    ul = rid[1:][:, k]
    tri_r = _split_quads(ll.ravel(), lr.ravel(), ur.ravel(), ul.ravel())
    xy = np.concatenate([xy_c, ring_xy.reshape(-1, 2)], axis=0)
    bnd_r = np.zeros(nr * nth, dtype=bool)
    bnd_r[:nth] = True  # nodes on the cylinder
    seg = np.linalg.norm(P - Q, axis=1)
    dw = np.diff(w)
    thick = np.minimum(np.concatenate([dw[:1], np.minimum(dw[:-1], dw[1:])]), 1.0)
    circ = np.linalg.norm(ring_xy - np.roll(ring_xy, -1, axis=1), axis=2)
    sc_r = np.minimum(thick[:nr, None] * seg[None], circ) * 0.5
    bnd = np.concatenate([bnd_c, bnd_r])
    sc = np.concatenate([sc_c, sc_r.ravel()])
    tri = np.concatenate([tri_c, tri_r], axis=0)
    tri = _orient_ccw(xy, tri)
    key = (xy[:, 1], np.floor(xy[:, 0] / hx + 0.5))
    xy, tri = _renumber(xy, tri, key, bnd, sc if jitter else 0.0, seed if jitter else None)
    tri = _orient_ccw(xy, tri)
    return xy, tri.astype(np.int32)


def _dist(dx, dy):
    """sqrt(dx^2 + dy^2) from IEEE-exact operations (same bits on every platform)."""
    return np.sqrt(np.multiply(dx, dx) + np.multiply(dy, dy))


def refine_uniform(xy: np.ndarray, tri: np.ndarray, snap_circle=None):
    """1:4 refinement: every triangle is split through its edge midpoints.

    New nodes (edge midpoints) are numbered after the old ones in order of their sorted
    (min, max) vertex pair.  With ``snap_circle=(cx, cy, r, tol)`` midpoints of edges
    whose both ends lie on the circle are projected onto it.
    """
    nv = xy.shape[0]
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]], axis=0)
    es = np.sort(e, axis=1)
    key = es[:, 0].astype(np.int64) * nv + es[:, 1]
    uk, inv = np.unique(key, return_inverse=True)
    a, b = uk // nv, uk % nv
    mid = 0.5 * (xy[a] + xy[b])
    if snap_circle is not None:
        cx, cy, r, tol = snap_circle
        da = np.abs(_dist(xy[a, 0] - cx, xy[a, 1] - cy) - r) < tol
        db = np.abs(_dist(xy[b, 0] - cx, xy[b, 1] - cy) - r) < tol
        on = da & db
        v = mid[on] - np.array([cx, cy])
        mid[on] = np.array([cx, cy]) + r * v / _dist(v[:, 0], v[:, 1])[:, None]
    nt = tri.shape[0]
    m = (nv + inv).reshape(3, nt).T  # m01, m12, m20
    v0, v1, v2 = tri[:, 0], tri[:, 1], tri[:, 2]
    t = np.concatenate([
        np.stack([v0, m[:, 0], m[:, 2]], 1),
        np.stack([m[:, 0], v1, m[:, 1]], 1),
        np.stack([m[:, 2], m[:, 1], v2], 1),
        np.stack([m[:, 0], m[:, 1], m[:, 2]], 1),
    ], axis=0)
    return np.concatenate([xy, mid], axis=0), t.astype(np.int32)


def write_dat(path: str, xy: np.ndarray, tri: np.ndarray) -> None:
    """Write a SALOME DAT mesh (triangles only, 1-based ids, no trailing newline)."""
    nv, nt = xy.shape[0], tri.shape[0]
    lines = ["%d %d" % (nv, nt)]
    ids = np.arange(1, nv + 1)
    lines += ["%d %.17g %.17g 0" % (k, x, y) for k, (x, y) in zip(ids, xy)]
    t1 = tri.astype(np.int64) + 1
    lines += ["%d 203 %d %d %d" % (nv + 1 + k, a, b, c) for k, (a, b, c) in enumerate(t1)]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def read_dat(path: str, scale: float = 1.0):
    """Read a SALOME DAT mesh as the reference does (triangles kept, other entities
    skipped, 1-based ids); a trailing newline is tolerated."""
    with open(path) as f:
        tok = f.read().split()
    nv, _ = int(tok[0]), int(tok[1])
    p = 2
    xy = np.empty((nv, 2))
    for k in range(nv):
        xy[k, 0] = scale * float(tok[p + 1])
        xy[k, 1] = scale * float(tok[p + 2])
        p += 4
    tris = []
    n = len(tok)
    while p + 1 < n:
        typ = int(tok[p + 1])
        if typ == 203:
            tris.append((int(tok[p + 2]) - 1, int(tok[p + 3]) - 1, int(tok[p + 4]) - 1))
            p += 5
        else:
            nvert = typ % 100
            p += 2 + nvert
    return xy, np.array(tris, dtype=np.int32).reshape(-1, 3)


def channel_boundary_nodes(xy: np.ndarray, lx: float, ly: float, umax: float = 1.5,
                           cylinder=None, tol: float = 2e-6, body_tol: float = 1e-3):
    """Dirichlet node lists of the flow drivers (Cylinder2D/main.cu:663-699).

    Returns (velocity_x, velocity_y, pressure) lists of (node, value) in ascending node
    order: parabolic inflow u = 4 umax y (ly - y) / ly^2 at x = 0, p = 0 at x = lx,
    no-slip on y = 0, y = ly and on the cylinder ``(cx, cy, r)``.
    """
    vx, vy, pr = [], [], []
    for i, (x, y) in enumerate(xy):
        if abs(x) < tol:
            vx.append((i, 4 * umax * y * (ly - y) / (ly * ly)))
            vy.append((i, 0.0))
        elif abs(x - lx) < tol:
            pr.append((i, 0.0))
        elif abs(y) < tol or abs(y - ly) < tol:
            vx.append((i, 0.0))
            vy.append((i, 0.0))
        elif cylinder is not None and abs(_dist(x - cylinder[0], y - cylinder[1]) - cylinder[2]) < body_tol:
            vx.append((i, 0.0))
            vy.append((i, 0.0))
    return vx, vy, pr


def square_boundary_nodes(xy: np.ndarray, tol: float = 2e-6):
    """All nodes on the boundary of [0,1]^2 with value 0 (the sin-sin Poisson problem)."""
    x, y = xy[:, 0], xy[:, 1]
    on = (np.abs(x) < tol) | (np.abs(x - 1) < tol) | (np.abs(y) < tol) | (np.abs(y - 1) < tol)
    return [(int(i), 0.0) for i in np.nonzero(on)[0]]


# ---- 3D (Mesh3D, Poisson3D) -----------------------------------------------------
def box_tets(nx: int = 40, ny: int = 20, nz: int = 10, lo=(-1.0, 0.0, -0.25), hi=(1.0, 1.0, 0.25),
             jitter: float = 0.2, seed: int = 0):
    """Structured tetrahedral mesh of a box: nx x ny x nz hexahedra, each split into the
    six tetrahedra around its (0,0,0)-(1,1,1) diagonal (conforming across hexahedra).
    The default box is the Poisson3D case's [-1,1] x [0,1] x [-0.25,0.25]; interior
    nodes move by at most ``jitter`` x the smallest spacing per axis (splitmix64 stream,
    three uniforms per interior node in node order).  Returns (xyz, tet)."""
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    h = [(hi[a] - lo[a]) / n for a, n in enumerate((nx, ny, nz))]
    xyz = np.stack([lo[0] + h[0] * i.ravel().astype(np.float64),
                    lo[1] + h[1] * j.ravel().astype(np.float64),
                    lo[2] + h[2] * k.ravel().astype(np.float64)], axis=1)
    # exact end coordinates, so that boundary tests with a 2e-6 tolerance see them
    for a, n in enumerate((nx, ny, nz)):
        idx = (i, j, k)[a].ravel()
        xyz[idx == n, a] = hi[a]
    nid = (i * (ny + 1) + j) * (nz + 1) + k

    def corner(dx, dy, dz):
        return nid[dx:nx + dx, dy:ny + dy, dz:nz + dz].ravel()

    tets = []
    for a, b in ((0, 1), (0, 2), (1, 0), (1, 2), (2, 0), (2, 1)):
        s1 = [0, 0, 0]
        s1[a] = 1
        s2 = list(s1)
        s2[b] = 1
        tets.append(np.stack([corner(0, 0, 0), corner(*s1), corner(*s2), corner(1, 1, 1)], axis=1))
    tet = np.concatenate(tets, axis=0)
    s = np.sort(tet, axis=1)
    tet = tet[np.lexsort((s[:, 3], s[:, 2], s[:, 1], s[:, 0]))]
    bnd = ((i == 0) | (i == nx) | (j == 0) | (j == ny) | (k == 0) | (k == nz)).ravel()
    interior = np.nonzero(~bnd)[0]
    if jitter and interior.size:
        r = uniform_pm1(seed, 3 * interior.size).reshape(-1, 3)
        xyz = xyz.copy()
        xyz[interior] += jitter * r * np.array(h)[None, :]
    return xyz, tet.astype(np.int32)


def write_dat3(path: str, xyz: np.ndarray, tet: np.ndarray) -> None:
    """Write a SALOME DAT mesh of tetrahedra (type 304, 1-based ids, no trailing newline)."""
    nv, nt = xyz.shape[0], tet.shape[0]
    lines = ["%d %d" % (nv, nt)]
    lines += ["%d %.17g %.17g %.17g" % (k + 1, x, y, z) for k, (x, y, z) in enumerate(xyz)]
    t1 = tet.astype(np.int64) + 1
    lines += ["%d 304 %d %d %d %d" % (nv + 1 + k, a, b, c, d) for k, (a, b, c, d) in enumerate(t1)]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def read_dat3(path: str, scale: float = 1.0):
    """Read a SALOME DAT mesh as Mesh3D::loadMeshFromFile (src/mesh_3d.cu:84-147) does:
    tetrahedra (type 304) kept, other entities skipped, 1-based ids."""
    with open(path) as f:
        tok = f.read().split()
    nv = int(tok[0])
    p = 2
    xyz = np.empty((nv, 3))
    for q in range(nv):
        for a in range(3):
            xyz[q, a] = scale * float(tok[p + 1 + a])
        p += 4
    tets = []
    n = len(tok)
    while p + 1 < n:
        typ = int(tok[p + 1])
        if typ == 304:
            tets.append(tuple(int(tok[p + 2 + a]) - 1 for a in range(4)))
        p += 2 + typ % 100
    return xyz, np.array(tets, dtype=np.int32).reshape(-1, 4)


def box_boundary_nodes(xyz: np.ndarray, tol: float = 2e-6):
    """Dirichlet nodes of the Poisson3D case (cases/Poisson3D/main.cu:111-126), tested
    in its order: x = -1 -> -1, x = 1 -> 1, y = 0 -> 0, y = 1 -> 2, z = -0.25 -> 3,
    z = 0.25 -> -2."""
    out = []
    for i, (x, y, z) in enumerate(xyz):
        if abs(x - (-1.0)) < tol:
            out.append((i, -1.0))
        elif abs(x - 1.0) < tol:
            out.append((i, 1.0))
        elif abs(y) < tol:
            out.append((i, 0.0))
        elif abs(y - 1.0) < tol:
            out.append((i, 2.0))
        elif abs(z - (-0.25)) < tol:
            out.append((i, 3.0))
        elif abs(z - 0.25) < tol:
            out.append((i, -2.0))
    return out


def cube_boundary_nodes(xyz: np.ndarray, tol: float = 2e-6):
    """All nodes on the boundary of [0,1]^3 with value 0 (the sin-sin-sin problem)."""
    on = np.zeros(xyz.shape[0], bool)
    for a in range(3):
        on |= (np.abs(xyz[:, a]) < tol) | (np.abs(xyz[:, a] - 1) < tol)
    return [(int(i), 0.0) for i in np.nonzero(on)[0]]
