"""The owner's water budget on the GPU: the device boundary ledger of an
interval equals the oracle's (-dt sum over open faces of the interval-mean
water flux x length, FP64 to 1e-10), and RiverSolver.step passes the
reference's budget test (volume change = ledger within
max(1e-10, 64 eps x inventory)) for inflow / outflow channels, the
exact-discharge inlet, outlet section owners, rotors and the HLLC method, in
both forms."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def oracle_ledger(case, dt):
    from oracle import Oracle
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    st, water, _ = o.advance(q, dt, 0.0)
    assert st == 0
    m = case["mesh"]
    openf = (m.neighbour < 0) & (m.bid >= 0)
    return -dt * float(np.sum(water[openf] * m.length[openf]))


@pytest.mark.parametrize("make", [S.small_channel, S.stage_discharge_channel, S.rating_channel],
                         ids=["channel", "inlet", "rating"])
def test_ledger_matches_oracle(make):
    from braids_hkt_gb300.solver import RiverSolver
    case = make()
    s = RiverSolver(case, precision="fp64")
    s.advance(1.0, 0.0)
    ref = oracle_ledger(case, 1.0)
    got = float(s.ledger()[0])
    assert abs(got - ref) <= 1e-10 * max(1.0, abs(ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_passes_the_water_budget(precision):
    from braids_hkt_gb300.solver import RiverSolver
    cases = [S.small_channel(), S.stage_discharge_channel(), S.rating_channel(), S.critical_channel(),
             S.small_rotor_channel(), S.lake_at_rest()]
    s = RiverSolver(cases, precision=precision)
    for _ in range(3):
        out = s.step(1.0)
        for d in out["diagnostics"]:
            assert abs(d["water_residual_m3"]) <= d["water_increment_roundoff_limit_m3"]
    assert s.steps == 3
    assert np.all(s.water_ledger[:5] != 0.0) and s.water_ledger[5] == 0.0


def test_hllc_step_passes_the_water_budget():
    from braids_hkt_gb300.solver import RiverSolver
    s = RiverSolver([S.small_channel(), S.stage_discharge_channel()], precision="fp64", method="hllc")
    for _ in range(2):
        out = s.step(1.0)
        for d in out["diagnostics"]:
            assert abs(d["water_residual_m3"]) <= d["water_increment_roundoff_limit_m3"]
