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
