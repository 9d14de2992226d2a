"""Host-side geometry of the HLLC / MUSCL-Hancock option.

The HLLC operator keeps its own cell incidence and least-squares inverse,
distinct from the f-wave stencil (src/braids_core/hydraulics/hllc.py:29-43):

  * incidence: every cell lists its faces in ascending face number, the
    order in which the operator's own set-up visits them; budgets and updates
    sum in this order;
  * inverse: pinv(sum over faces of d d^T / |d|^2), d the centroid offset to
    the neighbour, or for a wall the mirror offset 2 ((mid - xy) . n) n; open
    (inlet / outlet) faces take no part; numpy's pinv with rcond 1e-12 on the
    stacked 2x2 matrices (the same LAPACK call per matrix, bitwise equal to
    one call per cell), dot products through np.vecdot (the same inner
    product as np.dot on two 2-vectors).
"""
from __future__ import annotations

import numpy as np


def open_faces(mesh):
    """(nf,) int32: 1 on inlet / outlet faces (exterior faces of an open segment)."""
    return ((mesh.neighbour < 0) & (mesh.bid >= 0)).astype(np.int32)


def hllc_geometry(mesh):
    """Incidence in ascending face order, LS inverse (3, nc) and open-face flags."""
    cached = mesh.records.get("hllc")
    if cached is not None:
        return cached
    nc = mesh.nc
    owner, neighbour = mesh.owner, mesh.neighbour
    deg = np.diff(mesh.offset)
    cell_of = np.repeat(np.arange(nc), deg)
    order = np.lexsort((mesh.faces, cell_of))         # by cell, then face number
    faces = np.ascontiguousarray(mesh.faces[order], dtype=np.int32)
    signs = np.where(owner[faces] == cell_of, 1, -1).astype(np.int32)
    selected = open_faces(mesh)
    xy, mid, normal = mesh.xy, mesh.mid, mesh.normal
    other = np.where(signs > 0, neighbour[faces], owner[faces])
    matrix = np.zeros((nc, 2, 2))
    for slot in range(int(deg.max())):
        cells = np.flatnonzero(deg > slot)
        k = mesh.offset[cells] + slot
        f, j = faces[k], other[k]
        use = ~((j < 0) & (selected[f] != 0))
        cells, f, j = cells[use], f[use], j[use]
        inner = j >= 0
        d = np.empty((len(cells), 2))
        d[inner] = (xy[:, j[inner]] - xy[:, cells[inner]]).T
        w = ~inner
        if w.any():
            nrm = normal[:, f[w]].T
            dist = np.vecdot((mid[:, f[w]] - xy[:, cells[w]]).T, nrm)
            d[w] = (2 * dist)[:, None] * nrm
        norm = np.vecdot(d, d)
        pos = norm > 0
        cells, d, norm = cells[pos], d[pos], norm[pos]
        outer = d[:, :, None] * d[:, None, :]
        matrix[cells] = matrix[cells] + outer / norm[:, None, None]
    inv = np.linalg.pinv(matrix, rcond=1e-12)
    inverse = np.ascontiguousarray(np.stack((inv[:, 0, 0], inv[:, 0, 1], inv[:, 1, 1])))
    rec = dict(offset=np.ascontiguousarray(mesh.offset, dtype=np.int32), faces=faces, signs=signs,
               inverse=inverse, selected=selected)
    mesh.records["hllc"] = rec
    return rec


def entry_records(mesh):
    """Per CSR entry of the HLLC incidence: encoded face, other-cell code and
    stencil geometry (4, nadj), as brx_hllc_set takes them (local indices).

    Offsets follow the kernel's expressions exactly (IEEE subtraction and
    products, no contraction): xy[j] - xy[i] to a neighbour; for a wall
    2 * ((mid - xy) . n) * n with the dot product as (mid_x - x) n_x +
    (mid_y - y) n_y (hllc.h:25-28); mid - xy for the limiter (hllc.h:33).
    """
    g = hllc_geometry(mesh)
    nc = mesh.nc
    faces, signs = g["faces"], g["signs"]
    cell = np.repeat(np.arange(nc), np.diff(g["offset"]))
    owner, neighbour = mesh.owner, mesh.neighbour
    other = np.where(signs > 0, neighbour[faces], owner[faces]).astype(np.int32)
    wall = other < 0
    is_open = wall & (g["selected"][faces] != 0)
    other = np.where(is_open, -2, other).astype(np.int32)
    code = np.where(signs > 0, faces, ~faces).astype(np.int32)
    xy, mid, normal = mesh.xy, mesh.mid, mesh.normal
    jj = np.where(other >= 0, other, 0)
    geo = np.zeros((4, len(faces)))
    geo[0] = np.where(other >= 0, xy[0, jj] - xy[0, cell], 0.0)
    geo[1] = np.where(other >= 0, xy[1, jj] - xy[1, cell], 0.0)
    nx, ny = normal[0, faces], normal[1, faces]
    mdx, mdy = mid[0, faces] - xy[0, cell], mid[1, faces] - xy[1, cell]
    dist = mdx * nx + mdy * ny
    wl = other == -1
    geo[0, wl] = (2. * dist[wl]) * nx[wl]
    geo[1, wl] = (2. * dist[wl]) * ny[wl]
    geo[2], geo[3] = mdx, mdy
    return code, other, np.ascontiguousarray(geo), g["inverse"]


def pack(cases, cell_offset, face_offset):
    """Concatenated HLLC stencil of a scenario batch (global indices)."""
    codes, others, geos, invs = [], [], [], []
    for i, case in enumerate(cases):
        code, other, geo, inv = entry_records(case["mesh"])
        F0, C0 = int(face_offset[i]), int(cell_offset[i])
        codes.append(np.where(code >= 0, code + F0, ~(~code + F0)).astype(np.int32))
        others.append(np.where(other >= 0, other + C0, other).astype(np.int32))
        geos.append(geo)
        invs.append(inv)
    return dict(entry_face=np.ascontiguousarray(np.concatenate(codes), dtype=np.int32),
                entry_other=np.ascontiguousarray(np.concatenate(others), dtype=np.int32),
                entry_geo=np.ascontiguousarray(np.concatenate(geos, axis=1)),
                inverse=np.ascontiguousarray(np.concatenate(invs, axis=1)))
