"""Device-chained intervals (brx_advance_chain) against consecutive intervals.

A chained scenario begins its next interval on the device as soon as it has
completed one, so scenarios of one batch run different intervals at the same
time. Each interval must still be exactly what consecutive advance calls give
(start times formed as t += dt): the same accepted and rejected substep
counts, controller statistics, boundary ledger and gross boundary volume, and
a bit-identical state, in both arithmetic forms and for both hydraulic
methods; an idle scenario stays untouched.
"""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu

KEYS = ("hydraulic_substeps", "hydraulic_rejections", "hydraulic_minimum_dt", "hydraulic_maximum_dt",
        "accepted_cfl_max", "hydraulic_next_substep_hint_s", "failed")


def hydrograph_channel():
    case = S.small_channel(length=120.0, width=24.0, spacing=4.0, discharge=10.0)
    times = np.array([0.0, 1.0, 3.0, 8.0])
    value = np.zeros((2, case["mesh"].nb, len(times)))
    value[0, 0] = [10.0, 18.0, 40.0, 25.0]
    value[1, 1] = case["forcing"][1, 1]
    case["table_time"], case["table_value"] = times, value
    return case


def batch():
    """Scenarios of very different substep counts in one batch, one of them
    with a hydrograph table (time-dependent forcing across the intervals)."""
    return [S.small_channel(), S.dam_break(), S.small_rotor_channel(), S.lake_at_rest(), hydrograph_channel()]


def solver(cases, precision, method="fwave"):
    """The batch with one forcing table over all its segments: every
    segment holds its scenario's constant forcing except the last
    scenario's, which follows its hydrograph."""
    from braids_hkt_gb300.solver import RiverSolver
    s = RiverSolver(cases, precision=precision, method=method)
    last = cases[-1]
    packed = s.packed["forcing"]
    nb = last["table_value"].shape[1]
    times = last["table_time"]
    value = np.repeat(packed[:, :, None], len(times), axis=2)
    value[:, packed.shape[1] - nb:, :] = last["table_value"]
    s.set_forcing_table(times, value)
    return s


def consecutive(s, dt, t0, k):
    rows = [[] for _ in range(s.nscen)]
    t = np.array(t0, dtype=float)
    for _ in range(k):
        d = s.advance(dt, t)
        led, gro = s.ledger(), s.gross_boundary_volume()
        for i in range(s.nscen):
            rows[i].append(dict(d[i], boundary_ledger_m3=float(led[i]), gross_boundary_volume_m3=float(gro[i])))
        t = t + dt
    return rows


@pytest.mark.parametrize("precision,method", [("mixed", "fwave"), ("fp64", "fwave"), ("mixed", "hllc")])
def test_chain_equals_consecutive_intervals(precision, method):
    cases = batch()
    a, b = solver(cases, precision, method), solver(cases, precision, method)
    dt = np.full(len(cases), 0.5)
    t0 = np.array([0.0, 0.0, 0.25, 1.0, 0.5])
    k = 4
    chained = a.advance_chain(dt, t0, k)
    plain = consecutive(b, dt, t0, k)
    for i in range(len(cases)):
        for j in range(k):
            for key in KEYS + ("boundary_ledger_m3", "gross_boundary_volume_m3"):
                assert chained[i][j][key] == plain[i][j][key], (i, j, key, chained[i][j][key], plain[i][j][key])
        np.testing.assert_array_equal(a.state(i), b.state(i))
    # the scenarios needed different substep counts: the chain really interleaved intervals
    totals = [sum(r["hydraulic_substeps"] for r in rows) for rows in chained]
    assert max(totals) > 2 * min(totals)
    # the ledger getters report the chain's last interval
    np.testing.assert_array_equal(a.ledger(), b.ledger())


def test_chain_leaves_idle_scenario_untouched():
    cases = batch()
    a, b = solver(cases, "mixed"), solver(cases, "mixed")
    dt = np.array([0.5, 0.5, 0.0, 0.5, 0.5])
    q_idle = a.state(2).copy()
    chained = a.advance_chain(dt, np.zeros(len(cases)), 3)
    plain = consecutive(b, dt, np.zeros(len(cases)), 3)
    np.testing.assert_array_equal(a.state(2), q_idle)
    assert all(r["hydraulic_substeps"] == 0 for r in chained[2])
    for i in (0, 1, 3, 4):
        assert [r["hydraulic_substeps"] for r in chained[i]] == [r["hydraulic_substeps"] for r in plain[i]]
        np.testing.assert_array_equal(a.state(i), b.state(i))


def test_chain_then_advance_continues_the_clock():
    """After a chain the solver carries the controller's hint like after
    consecutive intervals: the next plain interval matches too."""
    cases = batch()
    a, b = solver(cases, "mixed"), solver(cases, "mixed")
    dt = np.full(len(cases), 0.5)
    a.advance_chain(dt, np.zeros(len(cases)), 2)
    consecutive(b, dt, np.zeros(len(cases)), 2)
    da, db = a.advance(dt, np.full(len(cases), 1.0)), b.advance(dt, np.full(len(cases), 1.0))
    for i in range(len(cases)):
        assert da[i]["hydraulic_substeps"] == db[i]["hydraulic_substeps"]
        np.testing.assert_array_equal(a.state(i), b.state(i))
