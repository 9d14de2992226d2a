"""Full-size channel configurations on the GPU against the oracle (FP64 form).

config 1: the 2000 m x 200 m channel, 4 m jittered Delaunay (50k triangles),
Q = 400 m3/s by conveyance, stage outlet 3.0 m, Manning 0.03, CFL 0.9. Five
owner steps of 1 s from the lake at rest: after each, the state within 1e-10
of the oracle's (scaled by each row's maximum) with the same substep count,
the owner's water budget passed (volume change = boundary ledger within the
FP64 roundoff allowance), and the volume equal to the oracle's to 1e-12
relative.

config 2: the same channel with three tandem rotors 150 m apart (D 5 m,
Ct 0.8, incident-speed power curve rated 500 kW) and the mesh refined to 1 m
across the channel downstream of each rotor (124k cells, about 370
substeps per simulated second). Three owner steps of 0.5 s with the
per-rotor thrust and power history at each output time (the
reference worker's TURBINE_PERFORMANCE rows) within 1e-8 relative of the
oracle's, and the state within 1e-10. It starts in uniform unit discharge
Q / W so that the rotors see flow from the first output on.
"""
import os

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
import braids_hkt_gb300.turbines as TB

pytestmark = pytest.mark.gpu

FORCE = TB.DIAG_FIELDS.index("force_per_density_m4_s2")
POWER = TB.DIAG_FIELDS.index("useful_power_per_density_m5_s3")
WORK = TB.DIAG_FIELDS.index("hydraulic_power_removed_per_density_m5_s3")


def _oracle(case):
    from oracle import Oracle
    return Oracle(case, threads=os.cpu_count() or 4)


def _volume(q, area):
    return float(np.sum(q[0] * area))


def test_config1_trajectory_matches_oracle():
    from braids_hkt_gb300.solver import RiverSolver
    case = S.config1()
    area = case["mesh"].area
    s = RiverSolver(case, precision="fp64")
    o = _oracle(case)
    q = case["q"].copy()
    for k in range(5):
        d = s.step(1.0)["diagnostics"]
        st, _, stats = o.advance(q, 1.0, float(k))
        assert st == 0 and d["failed"] == 0
        assert d["hydraulic_substeps"] == stats["substeps"], (k, d["hydraulic_substeps"], stats["substeps"])
        assert abs(d["water_residual_m3"]) <= d["water_increment_roundoff_limit_m3"]
        qs = s.state()
        scale = np.abs(q).max(axis=1, keepdims=True)
        err = float((np.abs(qs - q) / scale).max())
        assert err <= 1e-10, (k, err)
        v, vo = _volume(qs, area), _volume(q, area)
        assert abs(v - vo) <= 1e-12 * vo, (k, v, vo)
    assert d["hydraulic_substeps"] > 10


def test_config2_rotor_history_matches_oracle():
    from braids_hkt_gb300.solver import RiverSolver
    case = S.config2()
    assert 110_000 < case["mesh"].nc < 140_000
    # start in uniform unit discharge Q / W: the rotors 700-1000 m downstream
    # would otherwise sit in still water for the first minute
    q0 = case["q"]
    q0[1] = np.where(q0[0] > case["controls"]["dry"], 400.0 / 200.0, 0.0)
    s = RiverSolver(case, precision="fp64")
    history = s.performance_history(1.5, 0.5)
    o = _oracle(case)
    q = case["q"].copy()
    rows_o = []
    for k in range(3):
        st, _, stats = o.advance(q, 0.5, 0.5 * k)
        assert st == 0
        err, rec = o.diagnose(q)
        assert err == 0
        rows_o.append(rec)
    qs = s.state()
    scale = np.abs(q).max(axis=1, keepdims=True)
    assert (np.abs(qs - q) / scale).max() <= 1e-10
    nrot = len(case["turbines"])
    assert len(history) == 3 * nrot
    for k in range(3):
        rows = history[k * nrot:(k + 1) * nrot]
        assert all(r["time_s"] == pytest.approx(0.5 * (k + 1)) for r in rows)
        ref = rows_o[k]
        for j, r in enumerate(rows):
            assert r["turbine_id"] == case["turbines"][j]["name"]
            assert r["active"], r
            assert r["thrust_N"] == pytest.approx(ref[j, FORCE] * TB.WATER_DENSITY, rel=1e-8, abs=0)
            assert r["useful_power_W"] == pytest.approx(ref[j, POWER] * TB.WATER_DENSITY, rel=1e-8, abs=0)
            assert r["hydraulic_work_W"] == pytest.approx(ref[j, WORK] * TB.WATER_DENSITY, rel=1e-8, abs=0)
    # the rotors extract power from the flow at every output time
    assert all(r["useful_power_W"] > 0 for r in history)
