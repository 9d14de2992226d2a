"""Serving loop on the GPU: requests admitted over time into overlapping
cohorts give bitwise the results of the same scenarios run alone over the
same interval sequence, and admission stays within the memory budget."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from braids_hkt_gb300 import serving

pytestmark = pytest.mark.gpu


def alone(case, duration, interval, precision):
    from braids_hkt_gb300.solver import RiverSolver
    s = RiverSolver(case, precision=precision)
    t = 0.0
    while t < duration - 1e-9:
        dt = min(interval, duration - t)
        s.advance(dt, t)
        t += dt
    return s.state().copy(), (s.turbine_record() if s.rotors is not None else None)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_serving_results_equal_alone(precision):
    bases = [S.small_rotor_channel(seed=22), S.small_channel(seed=31, discharge=12.0),
             S.small_rotor_channel(seed=23, rotors=1, nu=0.002), S.small_channel(seed=32, discharge=20.0)]
    durations = [1.5, 1.0, 2.0, 0.5]
    arrivals = [0.0, 0.0, 0.05, 0.3]
    reqs = [serving.Request(rid=k, case=c, duration=d, arrival=a)
            for k, (c, d, a) in enumerate(zip(bases, durations, arrivals))]
    # budget for about two of these scenarios: the later ones wait for memory
    from braids_hkt_gb300.solver import RiverSolver
    probe = RiverSolver(bases[0], precision=precision)
    per = probe.device_bytes()
    probe.close()
    eng = serving.ServingEngine(budget_bytes=2.5 * per, precision=precision, interval=0.5, max_cohort_cells=10_000)
    done = eng.run(reqs, max_wall=120.0)
    assert len(done) == 4 and all(r.failed == 0 for r in done)
    assert eng.peak_bytes <= eng.budget
    for r in done:
        q, rec = alone(r.case, r.duration, 0.5, precision)
        np.testing.assert_array_equal(r.state, q)
        if rec is not None:
            np.testing.assert_array_equal(r.rotors, rec)
    rep = eng.report()
    assert rep["latency_s"]["p50"] > 0 and rep["throughput_cell_updates_s"] > 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_slot_serving_reuses_slots_and_equals_alone(precision):
    """One resident batch of slots (two copies of each pool mesh): six
    requests on three meshes arrive over time, more than the slots of one
    mesh, so later requests wait for a slot and re-use it after its first
    request finished. Each result equals the same request run alone, bit
    for bit, and nothing is rebuilt."""
    pool = [S.small_rotor_channel(seed=22), S.small_channel(seed=31, discharge=12.0),
            S.small_rotor_channel(seed=23, rotors=1, nu=0.002)]
    picks = [0, 0, 0, 1, 2, 2]
    discharge = [150.0, 120.0, 90.0, 14.0, 130.0, 110.0]
    durations = [1.0, 1.5, 0.5, 1.0, 0.5, 1.5]
    arrivals = [0.0, 0.0, 0.0, 0.02, 0.05, 0.1]
    reqs = [serving.Request(rid=k, case=serving.request_case(pool[b], qd), duration=d, arrival=a, base=b)
            for k, (b, qd, d, a) in enumerate(zip(picks, discharge, durations, arrivals))]
    eng = serving.SlotServingEngine(pool, precision=precision, interval=0.5, copies=2)
    done = eng.run(reqs, max_wall=120.0)
    rep = eng.report()
    eng.close()
    assert len(done) == 6 and all(r.failed == 0 for r in done)
    assert rep["slots"] == 6
    # three requests on mesh 0 with two slots: one waited and re-used a slot
    assert max(r.admitted - r.arrival for r in done if r.base == 0) > 0.0
    for r in done:
        q, rot = alone(r.case, r.duration, 0.5, precision)
        np.testing.assert_array_equal(r.state, q)
        if rot is not None:
            np.testing.assert_array_equal(r.rotors, rot)
