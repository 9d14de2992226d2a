"""Compensated device totals (brx_totals) against exact host sums, and what they show.

Water volume and mechanical energy per scenario are Neumaier-summed on the
device in a fixed order; against math.fsum of the same per-cell terms they
agree to 1e-14 relative. A still lake keeps both to round-off; a dry-bed dam
break in a closed box keeps its volume to 1e-12 and loses energy (the scheme
dissipates at the bore).
"""
import math

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def exact(case_q, z, area, g, dry):
    h, hu, hv = case_q
    mass = math.fsum((area * h).tolist())
    e = .5 * g * h * h + g * h * z
    wet = h > dry
    e = e + np.where(wet, .5 * (hu * hu + hv * hv) / np.where(wet, h, 1.0), 0.0)
    return mass, math.fsum((area * e).tolist())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_totals_match_exact_sums(precision):
    from braids_hkt_gb300.solver import RiverSolver
    cases = [S.small_channel(), S.dam_break(), S.lake_at_rest()]
    s = RiverSolver(cases, precision=precision)
    s.advance(0.5, 0.0)
    tot = s.totals()
    q = s.state()
    off = s.packed["cell_offset"]
    for i, c in enumerate(cases):
        a, b = off[i], off[i + 1]
        m, e = exact(q[:, a:b], np.asarray(c["z"]), c["mesh"].area, c["controls"]["grav"], c["controls"]["dry"])
        assert abs(tot[i, 0] - m) <= 1e-14 * abs(m)
        assert abs(tot[i, 1] - e) <= 1e-14 * abs(e)


def test_totals_lake_and_dam_break():
    from braids_hkt_gb300.solver import RiverSolver
    s = RiverSolver([S.lake_at_rest(), S.dam_break()], precision="mixed")
    t0 = s.totals().copy()
    for k in range(4):
        s.advance(0.5, 0.5 * k)
    t1 = s.totals()
    assert abs(t1[0, 0] - t0[0, 0]) <= 1e-12 * t0[0, 0]
    assert abs(t1[0, 1] - t0[0, 1]) <= 1e-12 * abs(t0[0, 1])
    assert abs(t1[1, 0] - t0[1, 0]) <= 1e-12 * t0[1, 0]
    assert t1[1, 1] < t0[1, 1]
