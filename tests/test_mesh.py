"""Mesh and geometry-record invariants of the synthetic river meshes."""
import numpy as np

import braids_hkt_gb300.mesh as M
import braids_hkt_gb300.scenarios as S


def test_channel_topology():
    m = M.channel_mesh(200.0, 40.0, 4.0, 1.0, seed=3)
    assert m.nc > 900 and np.all(m.area > 0)
    assert abs(m.area.sum() - 200.0 * 40.0) < 1e-8
    own = np.repeat(np.arange(m.nc), np.diff(m.offset))
    np.testing.assert_array_equal(np.where(m.signs > 0, m.owner[m.faces], m.neighbour[m.faces]), own)
    inner = m.neighbour >= 0
    d = m.xy[:, m.neighbour[inner]] - m.xy[:, m.owner[inner]]
    assert np.all((d * m.normal[:, inner]).sum(0) > 0)          # normals point owner -> neighbour
    ext = ~inner
    d = m.mid[:, ext] - m.xy[:, m.owner[ext]]
    assert np.all((d * m.normal[:, ext]).sum(0) > 0)            # and outward on the boundary
    assert set(np.unique(m.bid[ext])) == {-1, 0, 1}
    # closed surface: sum of length * normal vanishes per cell
    s = np.zeros((2, m.nc))
    for k in range(m.nadj):
        f = m.faces[k]
        s[:, own[k]] += m.signs[k] * m.length[f] * m.normal[:, f]
    assert np.abs(s).max() < 1e-10


def test_least_squares_records():
    m = M.channel_mesh(60.0, 20.0, 4.0, 1.0, seed=4)
    r = m.records
    a11, a12, a22, det = r["ls_matrix"]
    np.testing.assert_allclose(det, a11 * a22 - a12 * a12)
    full = det > 1e-12 * (a11 + a22) ** 2        # corner cells with one neighbour are rank one
    assert full.mean() > 0.95
    # a linear field is reproduced exactly by the weighted least squares
    f = 3.0 * m.xy[0] - 2.0 * m.xy[1]
    own = np.repeat(np.arange(m.nc), np.diff(m.offset))
    other = np.where(m.signs < 0, m.owner[m.faces], m.neighbour[m.faces])
    ok = other >= 0
    bx = np.zeros(m.nc)
    by = np.zeros(m.nc)
    np.add.at(bx, own[ok], (r["ls_weight"] * r["ls_delta"][0] * (f[np.where(ok, other, 0)] - f[own]))[ok])
    np.add.at(by, own[ok], (r["ls_weight"] * r["ls_delta"][1] * (f[np.where(ok, other, 0)] - f[own]))[ok])
    gx = (a22 * bx - a12 * by) / det
    gy = (a11 * by - a12 * bx) / det
    np.testing.assert_allclose(gx[full], 3.0, rtol=1e-9)
    np.testing.assert_allclose(gy[full], -2.0, rtol=1e-9)


def test_config1_size_and_boundaries():
    case = S.config1()
    m = case["mesh"]
    assert 45_000 <= m.nc <= 55_000
    assert m.nb == 2 and list(case["seg_mode"]) == [6, 2]
    assert np.all(case["q"][0] > 0)                      # lake at rest at 3 m, bed below everywhere
    assert abs(case["z"].min() - (-5.0)) < 1.0


def test_case_roundtrip():
    case = S.small_channel()
    back = S.case_from_arrays(S.case_arrays(case))
    np.testing.assert_array_equal(back["mesh"].faces, case["mesh"].faces)
    np.testing.assert_array_equal(back["mesh"].records["ls_weight"], case["mesh"].records["ls_weight"])
    assert back["controls"] == case["controls"]
