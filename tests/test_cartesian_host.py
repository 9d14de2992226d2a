"""Cartesian square cells (four faces per cell, the shape of the reference's
uncut Cartesian cut cells) in the oracle: closed geometry, a lake at rest
that stays at rest, and a flowing channel that conserves the open-channel
water budget."""
import numpy as np

import braids_hkt_gb300.scenarios as S
from oracle import Oracle


def test_cells_close():
    m = S.cartesian_channel()["mesh"]
    assert np.all(np.diff(m.offset) == 4)
    cell = np.repeat(np.arange(m.nc), 4)
    for comp in range(2):
        s = np.bincount(cell, weights=m.signs * m.length[m.faces] * m.normal[comp, m.faces], minlength=m.nc)
        assert np.abs(s).max() <= 1e-12


def test_lake_at_rest_holds():
    case = S.cartesian_channel()
    case["forcing"] = np.array([[0.0, 0.0], [0.0, 3.0]])
    q = case["q"].copy()
    st, _, _ = Oracle(case, threads=2).advance(q, 5.0, 0.0)
    assert st == 0
    wet = q[0] > 1e-6
    assert np.ptp((q[0] + case["z"])[wet]) <= 1e-12
    assert np.abs(q[1:]).max() <= 1e-12


def test_channel_water_budget():
    case = S.cartesian_channel()
    m = case["mesh"]
    q = case["q"].copy()
    v0 = float(np.sum(q[0] * m.area))
    st, water, _ = Oracle(case, threads=2).advance(q, 5.0, 0.0)
    assert st == 0
    openf = (m.neighbour < 0) & (m.bid >= 0)
    ledger = -5.0 * float(np.sum(water[openf] * m.length[openf]))
    v1 = float(np.sum(q[0] * m.area))
    assert abs((v1 - v0) - ledger) <= max(1e-10, 64 * np.finfo(float).eps * max(v0, v1))


def test_hllc_lake_at_rest_holds():
    case = S.cartesian_channel()
    case["forcing"] = np.array([[0.0, 0.0], [0.0, 3.0]])
    q = case["q"].copy()
    st, _, _ = Oracle(case, threads=2).hllc_advance(q, 3.0, 0.0)
    assert st == 0
    wet = q[0] > 1e-6
    assert np.ptp((q[0] + case["z"])[wet]) <= 1e-12
    assert np.abs(q[1:]).max() <= 1e-12
