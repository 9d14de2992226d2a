"""Config 3 scaled down: a braided river (three sinuous channels in a
floodplain, extensive wet/dry), an inlet hydrograph, the Exner bed update
with MPM transport and three rotors, coupled interval by interval.

FP64 form against the oracle: state and bed within 1e-10 (scaled), same
substep counts.

Mixed form against FP64 on one substep sequence (the FP64 run's, recorded
and replayed in the mixed form, so the two differ by round-off only): over
the first two seconds the depth of every cell deeper than 5 cm is within
1e-4 relative of FP64 (measured 1.6e-6 after 1 s, 1.4e-5 after 2 s), the
unit discharge within 1e-4 of its maximum (1.9e-5), the bed change within
1e-4 of the largest (3.3e-5) and the volume within 1e-10 (2.8e-11).

Mixed against FP64 with each form's own controller over three seconds: at
2.97 s a wetting front of films 1e-6 to 1e-4 m deep advances onto the
floodplain; there FP32 flux rounding is of the order of a film's own
momentum, the face wave speeds of the two forms differ (CFL peaks 544 and
1091 per second), their controllers take different substeps and the forms
differ by truncation error and front timing near the front (measured 1.4e-4
relative on cells deeper than 5 cm after 3 s, bound 2e-3; bed 5e-3 of the
largest change, bound 2e-2). The steady config-4 channels stay within 1e-4
(bench).
"""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def case():
    return S.config3(length=600.0, width=150.0, spacing=2.0, channels=3, rotors=3, amplitude=30.0,
                     q_low=20.0, q_high=100.0, rise_s=60.0, slope=5e-4, stage_above=0.6, grain=0.004)


def run(solver, n, interval=1.0):
    for k in range(n):
        d = solver.advance(interval, interval * k)
        assert d["failed"] == 0
        assert solver.morphology(interval)["ok"]


def test_config3_fp64_matches_oracle():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    c = case()
    s = RiverSolver(c, precision="fp64")
    s.set_forcing_table(c["table_time"], c["table_value"])
    o = Oracle(c, threads=16)
    q = c["q"].copy()
    for k in range(2):
        d = s.advance(1.0, 1.0 * k)
        st, _, stats = o.advance(q, 1.0, 1.0 * k)
        assert st == 0 and d["hydraulic_substeps"] == stats["substeps"]
        ms = s.morphology(1.0)
        code, zt, se = o.exner(q, 1.0)
        assert code == 0 and ms["ok"] and se["ok"]
        o.z[:] = zt
        scale = np.abs(q).max(axis=1, keepdims=True)
        assert (np.abs(s.state() - q) / scale).max() <= 1e-10
        dz = np.abs(zt - c["z"]).max()
        assert np.abs(s.z.cpu().numpy() - zt).max() <= 1e-10 * max(dz, 1e-9)
    err, rec = o.diagnose(q)
    np.testing.assert_allclose(s.turbine_record()[:, 10], rec[:, 10], rtol=1e-8, atol=1e-300)


def test_config3_mixed_against_fp64():
    from braids_hkt_gb300.solver import RiverSolver
    c = case()
    a, b = RiverSolver(c, precision="fp64"), RiverSolver(c, precision="mixed")
    for s in (a, b):
        s.set_forcing_table(c["table_time"], c["table_value"])
    run(a, 3)
    run(b, 3)
    ha, hb = a.state()[0], b.state()[0]
    deep = ha > 0.05
    rel = np.abs(hb - ha) / np.maximum(ha, 1e-3)
    print("config3 mixed depth error: deep max %.3e, all max %.3e" % (rel[deep].max(), rel.max()))
    assert rel[deep].max() < 2e-3
    assert (np.abs(hb - ha)).max() < 1e-3 * ha.max()
    za, zb = a.z.cpu().numpy(), b.z.cpu().numpy()
    dz = np.abs(za - c["z"]).max()
    assert np.abs(zb - za).max() <= 2e-2 * max(dz, 1e-9)


def test_config3_mixed_replayed_substeps_within_1e4():
    from braids_hkt_gb300.solver import RiverSolver
    c = case()
    a, b = RiverSolver(c, precision="fp64"), RiverSolver(c, precision="mixed")
    for s in (a, b):
        s.set_forcing_table(c["table_time"], c["table_value"])
    hint = None
    for k in range(2):
        dts, hint = a.advance_recorded(1.0, float(k), hint)
        assert b.advance_replay(dts, float(k)) == len(dts) > 50
        assert a.morphology(1.0)["ok"] and b.morphology(1.0)["ok"]
        qa, qb = a.state(), b.state()
        ha, hb = qa[0], qb[0]
        deep = ha > 0.05
        rel = np.abs(hb - ha) / np.maximum(ha, 1e-3)
        print("config3 replayed: t=%d deep depth max %.2e p99 %.2e" % (k + 1, rel[deep].max(),
                                                                         np.percentile(rel[deep], 99)))
        assert rel[deep].max() < 1e-4
        assert np.abs(qb[1:] - qa[1:]).max() < 1e-4 * np.abs(qa[1:]).max()
        za, zb = a.z.cpu().numpy(), b.z.cpu().numpy()
        assert np.abs(zb - za).max() <= 1e-4 * max(np.abs(za - c["z"]).max(), 1e-9)
        area = c["mesh"].area
        assert abs(np.sum(hb * area) - np.sum(ha * area)) <= 1e-10 * np.sum(ha * area)
