"""Conservative wet-bank viscosity in the oracle (om_shoreline_viscosity).

Against tests/golden/viscosity (made by tests/golden/make_viscosity_golden.py
from the reference's own kernels and safe state): the momentum-rate increment
is equal bit for bit. Physics: on a closed domain the shared-face stresses
cancel in the momentum total (the term only moves momentum between cells),
dry columns and walls take no stress, and a uniform velocity field has none.
"""
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from oracle import Oracle

GOLD = Path(__file__).parent / "golden" / "viscosity"


@pytest.mark.parametrize("name", ["channel_banks", "lake_islands"])
def test_viscosity_rate_matches_reference(name):
    g = np.load(GOLD / f"{name}.npz")
    case = S.case_from_arrays({k: g[k] for k in g.files})
    case["viscosity"] = float(g["nu"])
    o = Oracle(case, threads=2)
    rate = o.viscosity_rate(g["state"])
    assert np.abs(g["rate"]).max() > 1e-3
    np.testing.assert_array_equal(rate, g["rate"])


def test_viscosity_conserves_momentum_on_a_closed_domain():
    case = S.lake_at_rest()
    case["viscosity"] = 0.3
    q = S.perturbed_state(case, 7, 0.3, 0.8, 0.1)
    rate = Oracle(case, threads=2).viscosity_rate(q)
    area = case["mesh"].area
    for row in (1, 2):
        total = float(np.sum(rate[row] * area))
        scale = float(np.sum(np.abs(rate[row]) * area))
        assert abs(total) <= 1e-12 * scale
    dry = q[0] <= case["controls"]["dry"]
    assert dry.any()
    # a dry column exchanges nothing (its faces carry no stress)
    assert np.all(rate[1:, dry] == 0.0) or np.abs(rate[1:, dry]).max() <= 1e-14


def test_uniform_velocity_has_no_viscous_stress():
    case = S.lake_at_rest(islands=False)
    case["viscosity"] = 1.0
    q = case["q"].copy()
    q[1] = 0.7 * q[0]
    q[2] = -0.2 * q[0]
    rate = Oracle(case, threads=2).viscosity_rate(q)
    assert np.abs(rate[1:]).max() <= 1e-12
