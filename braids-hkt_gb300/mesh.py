"""Seeded unstructured river meshes and their finite-volume geometry records.

The solver consumes the face-based records of the reference's cut-cell
exporter: per face ``owner/neighbour/bid/normal/length/mid``, per cell
``area/xy``, a CSR cell->face incidence ``offset/faces/signs`` and the cached
least-squares stencil geometry. Triangles from a Delaunay triangulation fit
that layout unchanged.

Geometry formulas follow the reference's Fortran caches:
- ``bed_ls_delta`` = neighbour centroid - cell centroid per CSR entry
  (``src/solver/cut_cells/cutcell_solver.f90:8666-8688``);
- ``hydraulic_ls_weight`` = length / |r|^2 and the 2x2 normal matrix
  ``[a11, a12, a22, a11*a22 - a12*a12]`` accumulated in CSR order
  (``cutcell_solver.f90:8639-8662``);
- ``face_displacement`` = face midpoint - cell centroid per side
  (``cutcell_solver.f90:8693``);
- ``distance`` = |(mid - xy_owner).n| and |(xy_neighbour - mid).n|
  (``src/braids_support/gpu_fwave/resident_update.py:76-78``).

Faces are numbered in first-visit order over Morton-sorted cells, so both the
cell sweep and the face sweep walk memory with spatial locality.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import numpy as np

# Hydraulic boundary modes of the reference's exterior owner
# (src/braids_core/sediment/river_exterior_bed.h:94-156).
MODE_STAGE = 2          # prescribed water level, half-Riemann outflow
MODE_TOTAL_Q = 6        # total discharge distributed by conveyance


@dataclass
class Mesh:
    points: np.ndarray            # (np, 2) vertices
    tri: np.ndarray               # (nc, 3) CCW vertex ids
    owner: np.ndarray             # (nf,) int32
    neighbour: np.ndarray         # (nf,) int32, -1 exterior
    bid: np.ndarray               # (nf,) int32, boundary segment or -1 (wall / interior)
    normal: np.ndarray            # (2, nf) unit normal owner -> neighbour
    length: np.ndarray            # (nf,)
    mid: np.ndarray               # (2, nf)
    area: np.ndarray              # (nc,)
    xy: np.ndarray                # (2, nc) centroids
    offset: np.ndarray            # (nc+1,) int32
    faces: np.ndarray             # (nadj,) int32
    signs: np.ndarray             # (nadj,) int32 +1 owner / -1 neighbour
    boundary_offset: np.ndarray   # (nb+1,) int32
    boundary_faces: np.ndarray    # (sum,) int32, faces of each open segment in order
    records: dict = field(default_factory=dict)

    @property
    def nc(self):
        return len(self.area)

    @property
    def nf(self):
        return len(self.owner)

    @property
    def nadj(self):
        return len(self.faces)

    @property
    def nb(self):
        return len(self.boundary_offset) - 1


def morton_order(x, y):
    """Permutation sorting points along a 2-D Morton (Z-order) curve."""
    def spread(v):
        v = v.astype(np.uint64) & np.uint64(0xFFFF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
        v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
        v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
        v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
        return v
    lo = np.array([x.min(), y.min()])
    span = max(float(x.max() - lo[0]), float(y.max() - lo[1]), 1e-30)
    qx = np.floor((x - lo[0]) / span * 65535.0).astype(np.int64)
    qy = np.floor((y - lo[1]) / span * 65535.0).astype(np.int64)
    key = spread(qx) | (spread(qy) << np.uint64(1))
    return np.argsort(key, kind="stable")


def build_mesh(points, tri, segment_of_edge):
    """Face/CSR topology of a triangle mesh.

    ``segment_of_edge(a, b)`` receives the end points (arrays (m,2)) of the
    exterior edges and returns their open-boundary segment id, or -1 for a
    wall. Triangles are re-oriented counter-clockwise and Morton sorted.
    """
    points = np.ascontiguousarray(points, dtype=np.float64)
    tri = np.asarray(tri, dtype=np.int64).copy()
    p = points[tri]
    cross = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - \
            (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    flip = cross < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    cen = points[tri].mean(axis=1)
    tri = tri[morton_order(cen[:, 0], cen[:, 1])]
    nc = len(tri)
    p = points[tri]
    # Centroid and area (shoelace), FP64.
    xy = np.ascontiguousarray(((p[:, 0] + p[:, 1]) + p[:, 2]).T / 3.0)
    area = 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) -
                  (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    if np.any(area <= 0):
        raise ValueError("degenerate triangle")
    # Local edges (v0,v1), (v1,v2), (v2,v0): occurrence index 3*t + e.
    a = tri[:, [0, 1, 2]].ravel()
    b = tri[:, [1, 2, 0]].ravel()
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    key = lo * np.int64(len(points)) + hi
    order = np.argsort(key, kind="stable")          # occurrences of one edge are adjacent, ascending
    ks = key[order]
    start = np.ones(len(ks), dtype=bool)
    start[1:] = ks[1:] != ks[:-1]
    group = np.cumsum(start) - 1                      # edge id in key order
    first = order[start]                              # first (smallest) occurrence of each edge
    count = np.bincount(group)
    if np.any(count > 2):
        raise ValueError("non-manifold edge")
    second = np.full(len(first), -1, dtype=np.int64)
    two = np.flatnonzero(count == 2)
    second[two] = order[np.flatnonzero(start)[two] + 1]
    # Faces numbered by first visit over the Morton-sorted cells.
    face_order = np.argsort(first, kind="stable")
    first = first[face_order]
    second = second[face_order]
    nf = len(first)
    face_of_edge = np.empty(len(ks), dtype=np.int64)
    rank = np.empty(nf, dtype=np.int64)
    rank[face_order] = np.arange(nf)
    face_of_edge[order] = rank[group]
    owner = (first // 3).astype(np.int32)
    neighbour = np.where(second >= 0, second // 3, -1).astype(np.int32)
    va = a[first]
    vb = b[first]
    d = points[vb] - points[va]
    length = np.hypot(d[:, 0], d[:, 1])
    normal = np.ascontiguousarray(np.stack((d[:, 1] / length, -d[:, 0] / length)))
    mid = np.ascontiguousarray((0.5 * (points[va] + points[vb])).T)
    bid = np.full(nf, -1, dtype=np.int32)
    ext = np.flatnonzero(neighbour < 0)
    if len(ext):
        bid[ext] = np.asarray(segment_of_edge(points[va[ext]], points[vb[ext]]), dtype=np.int32)
    faces = face_of_edge.astype(np.int32)             # CSR entries 3c+e in local edge order
    signs = np.where(owner[faces] == np.repeat(np.arange(nc), 3), 1, -1).astype(np.int32)
    offset = (3 * np.arange(nc + 1)).astype(np.int32)
    nb = int(bid.max()) + 1 if np.any(bid >= 0) else 0
    bfaces, boff = [], [0]
    for s in range(nb):
        ids = np.flatnonzero(bid == s)
        # Order the segment along its own direction for reproducible reductions.
        mids = mid[:, ids]
        span = np.ptp(mids, axis=1)
        ids = ids[np.argsort(mids[int(np.argmax(span))], kind="stable")]
        bfaces.append(ids)
        boff.append(boff[-1] + len(ids))
    boundary_faces = (np.concatenate(bfaces) if bfaces else np.zeros(0, np.int64)).astype(np.int32)
    return Mesh(points=points, tri=tri.astype(np.int32), owner=owner, neighbour=neighbour, bid=bid,
                normal=normal, length=length, mid=mid, area=area, xy=xy,
                offset=offset, faces=faces, signs=signs,
                boundary_offset=np.asarray(boff, dtype=np.int32), boundary_faces=boundary_faces)


def cartesian_mesh(length, width, spacing):
    """Face/CSR topology of a Cartesian quadrilateral channel mesh.

    Square cells of side ``spacing`` over [0, length] x [0, width]; the left
    edge is open segment 0, the right edge open segment 1, the long sides are
    walls. Cells are Morton sorted; faces are numbered by first visit over
    the sorted cells, each cell's edges in counter-clockwise order (bottom,
    right, top, left), owner = the first visitor with its outward normal.
    The same records a cut-cell or quadtree exporter hands over for its
    uncut cells (four faces per cell instead of three).
    """
    nx, ny = int(round(length / spacing)), int(round(width / spacing))
    if nx < 1 or ny < 1:
        raise ValueError("channel smaller than one cell")
    dx, dy = length / nx, width / ny
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    I, J = I.ravel(), J.ravel()
    cx, cy = (I + 0.5) * dx, (J + 0.5) * dy
    order = morton_order(cx, cy)
    I, J, cx, cy = I[order], J[order], cx[order], cy[order]
    nc = nx * ny
    cell_of = np.full((nx, ny), -1, dtype=np.int64)
    cell_of[I, J] = np.arange(nc)
    # local edges: (di, dj) of the other cell, outward normal, midpoint offset, length
    local = [((0, -1), (0.0, -1.0), (0.0, -0.5 * dy), dx), ((1, 0), (1.0, 0.0), (0.5 * dx, 0.0), dy),
             ((0, 1), (0.0, 1.0), (0.0, 0.5 * dy), dx), ((-1, 0), (-1.0, 0.0), (-0.5 * dx, 0.0), dy)]
    face_id = {}
    owner, neighbour, normal, mid, flen, bid = [], [], [], [], [], []
    faces = np.empty(4 * nc, dtype=np.int32)
    signs = np.empty(4 * nc, dtype=np.int32)
    for c in range(nc):
        i, j = int(I[c]), int(J[c])
        for e, ((di, dj), nrm, moff, ln) in enumerate(local):
            key = (2 * i + 1 + di, 2 * j + 1 + dj)            # edge midpoint on the doubled grid
            if key not in face_id:
                oi, oj = i + di, j + dj
                other = int(cell_of[oi, oj]) if 0 <= oi < nx and 0 <= oj < ny else -1
                face_id[key] = len(owner)
                owner.append(c); neighbour.append(other); normal.append(nrm)
                mid.append((cx[c] + moff[0], cy[c] + moff[1])); flen.append(ln)
                bid.append(-1 if other >= 0 or dj != 0 else (0 if di < 0 else 1))
            f = face_id[key]
            faces[4 * c + e] = f
            signs[4 * c + e] = 1 if owner[f] == c else -1
    owner = np.asarray(owner, dtype=np.int32)
    neighbour = np.asarray(neighbour, dtype=np.int32)
    bid = np.asarray(bid, dtype=np.int32)
    mid = np.ascontiguousarray(np.asarray(mid).T)
    bfaces, boff = [], [0]
    for sgm in range(2):
        ids = np.flatnonzero(bid == sgm)
        ids = ids[np.argsort(mid[1, ids], kind="stable")]
        bfaces.append(ids)
        boff.append(boff[-1] + len(ids))
    return Mesh(points=np.zeros((0, 2)), tri=np.zeros((0, 3), np.int32), owner=owner, neighbour=neighbour, bid=bid,
                normal=np.ascontiguousarray(np.asarray(normal).T), length=np.asarray(flen, dtype=np.float64),
                mid=mid, area=np.full(nc, dx * dy), xy=np.ascontiguousarray(np.stack((cx, cy))),
                offset=(4 * np.arange(nc + 1)).astype(np.int32), faces=faces, signs=signs,
                boundary_offset=np.asarray(boff, dtype=np.int32),
                boundary_faces=np.concatenate(bfaces).astype(np.int32))


def opening_chains(mesh: Mesh, segment: int):
    """Ordered face chains of one open segment (connected runs of its faces).

    Two faces of the segment are linked when an end point of one meets an end
    point of the other (within 128 ulp of the coordinate scale, at least
    1e-10) and their owners are the same or neighbouring cells; each chain
    starts at its end face with the smallest face number and walks the links
    (the section order of river_boundary_components.connected_opening_chains,
    src/braids_core/sediment/river_boundary_components.py:11-56).
    """
    from scipy.spatial import cKDTree
    owner, neighbour = mesh.owner, mesh.neighbour
    ids = np.flatnonzero((neighbour < 0) & (mesh.bid == segment))
    if not len(ids):
        raise ValueError("segment has no open faces")
    nx, ny = mesh.normal[0, ids], mesh.normal[1, ids]
    tangent = np.stack((-ny, nx), axis=1)
    centre = mesh.mid[:, ids].T
    half = .5 * mesh.length[ids, None] * tangent
    ends = np.empty((2 * len(ids), 2))
    ends[0::2] = centre - half
    ends[1::2] = centre + half
    scale = max(1., float(np.max(np.abs(ends))))
    tol = max(1e-10, 128 * np.spacing(scale))
    inner = neighbour >= 0
    linked = set(zip(np.minimum(owner[inner], neighbour[inner]).tolist(),
                     np.maximum(owner[inner], neighbour[inner]).tolist()))
    adj = [set() for _ in ids]
    for a, b in sorted(cKDTree(ends).query_pairs(tol)):
        i, j = a // 2, b // 2
        if i == j:
            raise ValueError("degenerate open face")
        oi, oj = int(owner[ids[i]]), int(owner[ids[j]])
        if oi == oj or (min(oi, oj), max(oi, oj)) in linked:
            adj[i].add(j)
            adj[j].add(i)
    if any(len(a) > 2 for a in adj):
        raise ValueError("a branched opening needs explicit boundary sections")
    left, chains = set(range(len(ids))), []
    while left:
        seed = min(left, key=lambda i: int(ids[i]))
        stack, comp = [seed], set()
        while stack:
            i = stack.pop()
            if i not in comp:
                comp.add(i)
                stack.extend(adj[i] - comp)
        tips = [i for i in comp if len(adj[i]) <= 1]
        if not tips:
            raise ValueError("a closed opening is not a section")
        at, prev, order = min(tips, key=lambda i: int(ids[i])), -1, []
        while True:
            order.append(int(ids[at]))
            left.discard(at)
            nxt = adj[at] - {prev}
            if not nxt:
                break
            prev, at = at, next(iter(nxt))
        if len(order) != len(comp):
            raise ValueError("could not order the opening")
        chains.append(order)
    return chains


def geometry_records(mesh: Mesh):
    """Least-squares stencil geometry cached per CSR entry and face side.

    Accumulation order and expression shape follow the reference caches so
    that every consumer sees bitwise-identical FP64 weights.
    """
    nc, nf = mesh.nc, mesh.nf
    owner, neighbour, faces, signs, offset = mesh.owner, mesh.neighbour, mesh.faces, mesh.signs, mesh.offset
    xy = mesh.xy
    other = np.where(signs < 0, owner[faces], neighbour[faces])
    has = other >= 0
    cell_of = np.repeat(np.arange(nc), np.diff(offset))
    safe = np.where(has, other, 0)
    r1 = np.where(has, xy[0, safe] - xy[0, cell_of], 0.0)
    r2 = np.where(has, xy[1, safe] - xy[1, cell_of], 0.0)
    ls_delta = np.ascontiguousarray(np.stack((r1, r2)))
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(has, mesh.length[faces] / (r1 * r1 + r2 * r2), 0.0)
    a11 = np.zeros(nc)
    a12 = np.zeros(nc)
    a22 = np.zeros(nc)
    degree = np.diff(offset)
    for slot in range(int(degree.max())):
        cells = np.flatnonzero(degree > slot)
        k = offset[cells] + slot
        m = has[k]
        cells, k = cells[m], k[m]
        a11[cells] = a11[cells] + w[k] * (r1[k] * r1[k])
        a12[cells] = a12[cells] + (w[k] * r1[k]) * r2[k]
        a22[cells] = a22[cells] + w[k] * (r2[k] * r2[k])
    ls_matrix = np.ascontiguousarray(np.stack((a11, a12, a22, a11 * a22 - a12 * a12)))
    disp = np.zeros((2, 2, nf))          # [component, side, face]
    disp[0, 0] = mesh.mid[0] - xy[0, owner]
    disp[1, 0] = mesh.mid[1] - xy[1, owner]
    nb_ = neighbour >= 0
    nsafe = np.where(nb_, neighbour, 0)
    disp[0, 1] = np.where(nb_, mesh.mid[0] - xy[0, nsafe], 0.0)
    disp[1, 1] = np.where(nb_, mesh.mid[1] - xy[1, nsafe], 0.0)
    disp_len = np.hypot(disp[0], disp[1])        # (2, nf) |mid - xy| per side
    nx, ny = mesh.normal
    distance = np.zeros((2, nf))
    distance[0] = np.abs((mesh.mid[0] - xy[0, owner]) * nx + (mesh.mid[1] - xy[1, owner]) * ny)
    distance[1] = np.where(nb_, np.abs((xy[0, nsafe] - mesh.mid[0]) * nx + (xy[1, nsafe] - mesh.mid[1]) * ny), 0.0)
    rec = dict(ls_delta=ls_delta, ls_weight=np.ascontiguousarray(w), ls_matrix=ls_matrix,
               disp=np.ascontiguousarray(disp), disp_len=np.ascontiguousarray(disp_len),
               distance=np.ascontiguousarray(distance))
    mesh.records.update(rec)
    return rec


RECORD_KEYS = ("owner", "neighbour", "bid", "normal", "length", "mid", "area", "xy", "offset", "faces", "signs",
               "boundary_offset", "boundary_faces", "ls_matrix", "ls_weight", "ls_delta", "displacement", "distance")


def mesh_from_records(d, points=None, tri=None):
    """A Mesh over a reference owner's geometry records.

    ``d`` holds owner, neighbour, bid, normal (2,nf), length, mid (2,nf),
    area, xy (2,nc), the CSR offset / faces / signs, boundary_offset /
    boundary_faces (river_mesh_records.initialize), and the f-wave
    reconstruction's least-squares records in the layout the reference's
    FP64 GPU kernels take them (reconstruction.cu:43-60): ls_matrix (4,nc),
    ls_weight (nadj), ls_delta (2,nadj), distance (2,nf) (the owner-side and
    neighbour-side normal distances) and displacement, the face midpoint
    minus the cell centre, either as (2,2,nf) [component, side, face] (the
    Fortran exporter's face_displacement) or as (4,nf) side-major rows owner
    x, owner y, neighbour x, neighbour y (the geometry cache's
    ``displacement``, bend_methods_v1.py:125-128), which is converted. Every
    shape is checked; any other layout is refused. Cells may be any polygons
    (cut cells, quadtree); no geometry is recomputed, so the solver sees the
    reference's own bits. Rotor arrays need the cell polygons as triangles
    (points, tri); without them a case takes no rotors.
    """
    missing = [k for k in RECORD_KEYS if k not in d]
    if missing:
        raise ValueError(f"records lack {missing}")
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    nc, nf = len(d["area"]), len(d["owner"])
    nadj = len(d["faces"])
    shapes = dict(owner=(nf,), neighbour=(nf,), bid=(nf,), normal=(2, nf), length=(nf,), mid=(2, nf), area=(nc,),
                  xy=(2, nc), offset=(nc + 1,), faces=(nadj,), signs=(nadj,), ls_matrix=(4, nc),
                  ls_weight=(nadj,), ls_delta=(2, nadj), distance=(2, nf))
    bad = [f"{k} {np.shape(d[k])} (expected {v})" for k, v in shapes.items() if np.shape(d[k]) != v]
    if bad:
        raise ValueError("records have inconsistent shapes: " + ", ".join(bad))
    if int(np.asarray(d["offset"])[-1]) != nadj:
        raise ValueError("records: offset[-1] differs from the number of CSR entries")
    disp = f64(d["displacement"])
    if disp.shape == (4, nf):           # side-major rows: owner x, y; neighbour x, y
        disp = np.ascontiguousarray(np.stack((disp[[0, 2]], disp[[1, 3]])))
    elif disp.shape != (2, 2, nf):
        raise ValueError(f"records: displacement {disp.shape} is neither (2,2,nf) nor (4,nf)")
    mesh = Mesh(points=np.zeros((0, 2)) if points is None else f64(points),
                tri=np.zeros((0, 3), np.int64) if tri is None else np.asarray(tri, dtype=np.int64),
                owner=i32(d["owner"]), neighbour=i32(d["neighbour"]), bid=i32(d["bid"]), normal=f64(d["normal"]),
                length=f64(d["length"]), mid=f64(d["mid"]), area=f64(d["area"]), xy=f64(d["xy"]),
                offset=i32(d["offset"]), faces=i32(d["faces"]), signs=i32(d["signs"]),
                boundary_offset=i32(d["boundary_offset"]), boundary_faces=i32(d["boundary_faces"]))
    mesh.records = dict(ls_matrix=f64(d["ls_matrix"]), ls_weight=f64(d["ls_weight"]), ls_delta=f64(d["ls_delta"]),
                        disp=disp, disp_len=np.ascontiguousarray(np.hypot(disp[0], disp[1])),
                        distance=f64(d["distance"]))
    return mesh


def records_of(mesh: Mesh):
    """The records dict of a Mesh under the reference's key names (the inverse of mesh_from_records)."""
    r = mesh.records
    d = {k: getattr(mesh, k) for k in RECORD_KEYS[:13]}
    d.update(ls_matrix=r["ls_matrix"], ls_weight=r["ls_weight"], ls_delta=r["ls_delta"], displacement=r["disp"],
             distance=r["distance"])
    return d


# ---------------------------------------------------------------------------
# Synthetic channel meshes
# ---------------------------------------------------------------------------

def jittered_channel_points(length, width, spacing, jitter, rng, refine=()):
    """Grid points on [0,L]x[0,W] with uniform jitter; edge points slide only along their edge.

    ``refine`` is a sequence of boxes ``(x0, x1, y0, y1, spacing)``: coarse
    points inside a box are replaced by a finer jittered grid.
    """
    nx = int(round(length / spacing))
    ny = int(round(width / spacing))
    xs = np.linspace(0.0, length, nx + 1)
    ys = np.linspace(0.0, width, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    X = X.ravel()
    Y = Y.ravel()
    jx = rng.uniform(-jitter, jitter, X.size)
    jy = rng.uniform(-jitter, jitter, X.size)
    onx = (X == 0.0) | (X == length)
    ony = (Y == 0.0) | (Y == width)
    X = X + np.where(onx, 0.0, jx)
    Y = Y + np.where(ony, 0.0, jy)
    pts = [np.c_[X, Y]]
    keep = np.ones(len(pts[0]), dtype=bool)
    for (x0, x1, y0, y1, s) in refine:
        x0, x1 = max(0.0, x0), min(length, x1)
        y0, y1 = max(0.0, y0), min(width, y1)
        inside = (pts[0][:, 0] > x0 - spacing * 0.5) & (pts[0][:, 0] < x1 + spacing * 0.5) & \
                 (pts[0][:, 1] > y0 - spacing * 0.5) & (pts[0][:, 1] < y1 + spacing * 0.5)
        # coarse points inside the box are replaced by the fine grid; a box
        # that reaches an edge of the domain also replaces that edge's coarse
        # points (the domain corners stay)
        keep &= ~inside | (onx & ony)
        fx = np.arange(x0, x1 + 1e-9, s)
        fy = np.arange(y0, y1 + 1e-9, s)
        FX, FY = np.meshgrid(fx, fy, indexing="ij")
        FX = FX.ravel()
        FY = FY.ravel()
        fj = 0.25 * s
        jx = rng.uniform(-fj, fj, FX.size)
        jy = rng.uniform(-fj, fj, FY.size)
        # fine points on an edge of the domain slide only along that edge
        edge_x = (FX <= 0.0) | (FX >= length)
        edge_y = (FY <= 0.0) | (FY >= width)
        FX = np.where(edge_x, FX, FX + jx)
        FY = np.where(edge_y, FY, FY + jy)
        ok = (FX >= 0.0) & (FX <= length) & (FY >= 0.0) & (FY <= width) & ~(edge_x & edge_y)
        pts.append(np.c_[FX[ok], FY[ok]])
    base = pts[0][keep]
    out = np.concatenate([base] + pts[1:])
    _, unique = np.unique(np.round(out, 9), axis=0, return_index=True)
    return out[np.sort(unique)]


def gaussian_field(length, width, sigma, correlation, rng, resolution=1.0):
    """Stationary Gaussian random field by FFT filtering of white noise.

    Covariance sigma^2 exp(-r^2 / (2 l^2)); the raster is padded by 3 l on
    every side so the periodic FFT does not correlate opposite edges. Returns
    ``(x0, y0, res, raster)`` for bilinear sampling.
    """
    from scipy.fft import next_fast_len
    pad = 3.0 * correlation
    nx = next_fast_len(int(np.ceil((length + 2 * pad) / resolution)) + 1, real=True)
    ny = next_fast_len(int(np.ceil((width + 2 * pad) / resolution)) + 1, real=True)
    noise = rng.standard_normal((nx, ny))
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=resolution)
    ky = 2 * np.pi * np.fft.rfftfreq(ny, d=resolution)
    K2 = kx[:, None] ** 2 + ky[None, :] ** 2
    filt = np.exp(-K2 * correlation ** 2 / 4.0)
    field = np.fft.irfft2(np.fft.rfft2(noise) * filt, s=(nx, ny))
    field *= sigma / field.std()
    return (-pad, -pad, resolution, field)


def sample_field(grid, x, y):
    x0, y0, res, raster = grid
    fx = (x - x0) / res
    fy = (y - y0) / res
    i = np.clip(np.floor(fx).astype(np.int64), 0, raster.shape[0] - 2)
    j = np.clip(np.floor(fy).astype(np.int64), 0, raster.shape[1] - 2)
    tx = fx - i
    ty = fy - j
    return ((1 - tx) * (1 - ty) * raster[i, j] + tx * (1 - ty) * raster[i + 1, j] +
            (1 - tx) * ty * raster[i, j + 1] + tx * ty * raster[i + 1, j + 1])


def channel_mesh(length, width, spacing, jitter, seed, refine=()):
    """Delaunay mesh of a straight channel: inlet segment 0 at x=0, outlet 1 at x=L, walls elsewhere."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = jittered_channel_points(length, width, spacing, jitter, rng, refine)
    tri = Delaunay(pts).simplices

    def segment(a, b):
        tol = 1e-9 * max(length, 1.0)
        inlet = (np.abs(a[:, 0]) < tol) & (np.abs(b[:, 0]) < tol)
        outlet = (np.abs(a[:, 0] - length) < tol) & (np.abs(b[:, 0] - length) < tol)
        return np.where(inlet, 0, np.where(outlet, 1, -1))
    mesh = build_mesh(pts, tri, segment)
    geometry_records(mesh)
    return mesh


def section_neighbours(mesh: Mesh, segment: int):
    """Physical neighbour faces along one straight inlet section.

    Returns (left, right) for the segment's open faces (arrays over all faces,
    -1 elsewhere): faces sorted by their station along the section tangent
    (-ny, nx) of the first face; consecutive faces whose facing ends meet
    (gap within max(1e-10, 64 ulp of the midpoint scale)) are neighbours, a
    gap ends a bank. The section must be collinear with one consistent normal
    (NormalSection's adjacency, src/braids_core/sediment/
    river_exterior_normal.py:11-27).
    """
    nf = len(mesh.owner)
    left = np.full(nf, -1, np.int32)
    right = left.copy()
    ids = np.flatnonzero((mesh.neighbour < 0) & (mesh.bid == segment))
    if not len(ids):
        raise ValueError("normal inlet has no physical faces")
    normal = mesh.normal[:, ids[0]]
    relative = mesh.mid[:, ids] - mesh.mid[:, ids[0], None]
    tol = max(1e-10, 64 * np.spacing(max(1., float(np.max(np.abs(mesh.mid[:, ids]))))))
    if (np.any(np.abs(mesh.normal[:, ids] - normal[:, None]) > 1e-12) or
            np.any(np.abs(normal @ relative) > tol)):
        raise ValueError("a normal inlet needs one collinear, consistently oriented section")
    station = np.array([-normal[1], normal[0]]) @ relative
    order = np.argsort(station)
    ids, station = ids[order], station[order]
    widths = mesh.length[ids]
    gaps = np.diff(station) - .5 * (widths[:-1] + widths[1:])
    if np.any(gaps < -tol):
        raise ValueError("normal inlet faces overlap")
    for i in np.flatnonzero(np.abs(gaps) <= tol):
        left[ids[i + 1]] = ids[i]
        right[ids[i]] = ids[i + 1]
    return left, right
