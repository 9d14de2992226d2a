"""Rotor arrays on the GPU against the oracle and the reference fixtures.

FP64 form: the residual matches the oracle to 1e-12 relative of each row's
scale (bitwise in practice), an adaptive advance to 1e-10 with the same
substep count, per-rotor power and thrust to 1e-8 relative (the stated
tolerance; the per-rotor sums differ from the oracle only in order).
Mixed form: depth within 1e-4 relative of the FP64 form, per-rotor power
within 1e-3 relative (power goes with the cube of the FP32-carried speed).
"""
import json
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
import braids_hkt_gb300.turbines as TB

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden" / "turbines"
POWER = TB.DIAG_FIELDS.index("useful_power_per_density_m5_s3")
FORCE = TB.DIAG_FIELDS.index("force_per_density_m4_s2")
REASON = TB.DIAG_FIELDS.index("reason")
COLUMNS = [TB.DIAG_FIELDS.index(f) for f in (
    "active", "minimum_coverage_margin_m", "minimum_bed_clearance_m", "local_velocity_m_s",
    "upstream_velocity_m_s", "mean_depth_m", "thrust_coefficient", "power_coefficient",
    "force_per_density_m4_s2", "useful_power_per_density_m5_s3", "hydraulic_power_removed_per_density_m5_s3")]


def solver(case, precision="fp64"):
    from braids_hkt_gb300.solver import RiverSolver
    return RiverSolver(case, precision=precision)


def oracle(case):
    from oracle import Oracle
    return Oracle(case, threads=4)


def curves():
    return TB.rated_power_curve(5.0, 0.8, 0.4, 500e3)


@pytest.mark.parametrize("control,nu", [(None, 0.0), ("curves", 0.005)])
def test_rotor_rate_matches_oracle(control, nu):
    case = S.small_rotor_channel(control=curves() if control else None, nu=nu)
    q = S.perturbed_state(case, 5, 0.05, 0.2, 0.0)
    s = solver(case)
    s.set_state(q)
    rate, water, status, freq = s.rate(0.005)
    st, rate_o, water_o, freq_o = oracle(case).rate(q, 0.005)
    assert status == 0 and st == 0
    rate = rate.cpu().numpy()
    scale = np.abs(rate_o).max(axis=1, keepdims=True)
    assert (np.abs(rate - rate_o) / scale).max() <= 1e-12


def overlapping_rotors():
    """Two rotors side by side, 3 m apart across the flow with D = 5 m: their
    footprints share cells, whose actuator sink sums both rotors' terms (the
    sink-sum kernel; every other support cell gets its sink from its
    rotor's sample CTA)."""
    case = S.small_rotor_channel(rotors=1)
    x, y = case["turbines"][0]["X"], case["turbines"][0]["Y"]
    case["turbines"] = S.rotor_rows(case, [(x, y - 1.5), (x, y + 1.5)])
    a, _ = TB.bump_integrals(case["mesh"], x, y - 1.5, 5.0)
    b, _ = TB.bump_integrals(case["mesh"], x, y + 1.5, 5.0)
    assert len(set(np.asarray(a).tolist()) & set(np.asarray(b).tolist())) > 0
    return case


def test_overlapping_rotors_match_oracle():
    case = overlapping_rotors()
    q = S.perturbed_state(case, 7, 0.05, 0.2, 0.0)
    s = solver(case)
    s.set_state(q)
    rate, water, status, freq = s.rate(0.005)
    o = oracle(case)
    st, rate_o, water_o, freq_o = o.rate(q, 0.005)
    assert status == 0 and st == 0
    rate = rate.cpu().numpy()
    scale = np.abs(rate_o).max(axis=1, keepdims=True)
    assert (np.abs(rate - rate_o) / scale).max() <= 1e-12
    s2 = solver(case)
    d = s2.advance(1.0, 0.0)
    q2 = case["q"].copy()
    st, _, stats = o.advance(q2, 1.0)
    assert st == 0 and d["failed"] == 0 and d["hydraulic_substeps"] == stats["substeps"]
    scale = np.abs(q2).max(axis=1, keepdims=True)
    assert (np.abs(s2.state() - q2) / scale).max() <= 1e-10


@pytest.mark.parametrize("control,nu", [(None, 0.0), ("curves", 0.005)])
def test_rotor_advance_matches_oracle(control, nu):
    case = S.small_rotor_channel(control=curves() if control else None, nu=nu)
    s = solver(case)
    d = s.advance(2.0, 0.0)
    o = oracle(case)
    q = case["q"].copy()
    st, _, stats = o.advance(q, 2.0)
    assert st == 0 and d["failed"] == 0
    assert d["hydraulic_substeps"] == stats["substeps"]
    qs = s.state()
    scale = np.abs(q).max(axis=1, keepdims=True)
    assert (np.abs(qs - q) / scale).max() <= 1e-10
    rec = s.turbine_record()
    err, rec_o = o.diagnose(q)
    assert err == 0
    np.testing.assert_array_equal(rec[:, REASON], rec_o[:, REASON])
    for col in (POWER, FORCE):
        np.testing.assert_allclose(rec[:, col], rec_o[:, col], rtol=1e-8, atol=0)
    rows = s.turbines()
    assert all(r["active"] for r in rows) and all(r["power_W"] > 0 for r in rows)


def test_rotor_gate_outcomes_match_reference():
    z = np.load(GOLD / "rotor_gate.npz")
    g = {k: z[k] for k in z.files}
    case = S.case_from_arrays(g)
    for name in [k[:-5] for k in g if k.endswith("_diag")]:
        c = dict(case, turbines=json.loads(str(g[f"{name}_rows"])))
        s = solver(c)
        state = str(g[f"{name}_state"])
        if state != "initial":
            s.set_state(g[f"{state}_q"])
        rec = s.turbine_record()
        assert TB.REASONS[int(rec[0, REASON])] == name
        np.testing.assert_allclose(rec[:, COLUMNS], g[f"{name}_diag"], rtol=1e-12, atol=1e-15, err_msg=name)


def test_rotor_steps_match_reference_fixture():
    z = np.load(GOLD / "rotor_steps.npz")
    g = {k: z[k] for k in z.files}
    case = S.case_from_arrays(g)
    for mode in ("constant", "curves", "table", "incident_table"):
        c = dict(case, turbines=json.loads(str(g[f"{mode}_rows"])))
        s = solver(c)
        d = s.advance(1.0, 0.0)
        assert d["hydraulic_substeps"] == int(g[f"{mode}_substeps"])
        ref = g[f"{mode}_advance"]
        scale = np.abs(ref).max(axis=1, keepdims=True)
        assert (np.abs(s.state() - ref) / scale).max() <= 1e-10, mode
        rec = s.turbine_record()
        np.testing.assert_allclose(rec[:, COLUMNS][:, 9], g[f"{mode}_diag"][:, 9], rtol=1e-8, err_msg=mode)


def test_rotor_mixed_against_fp64():
    case = S.small_rotor_channel(control=curves(), nu=0.005)
    a, b = solver(case, "fp64"), solver(case, "mixed")
    for _ in range(3):
        a.step(1.0)
        b.step(1.0)
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() < 1e-4
    pa, pb = a.turbine_record()[:, POWER], b.turbine_record()[:, POWER]
    np.testing.assert_allclose(pb, pa, rtol=1e-3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rotor_batch_equals_alone(precision):
    from braids_hkt_gb300.solver import RiverSolver
    cases = [S.small_rotor_channel(seed=22), S.small_channel(seed=31, discharge=12.0),
             S.small_rotor_channel(seed=23, rotors=1, nu=0.002)]
    batch = RiverSolver(cases, precision=precision)
    batch.advance(1.0, 0.0)
    rec = batch.turbine_record()
    k = 0
    for i, case in enumerate(cases):
        alone = RiverSolver(case, precision=precision)
        alone.advance(1.0, 0.0)
        np.testing.assert_array_equal(batch.state(i), alone.state())
        if case.get("turbines"):
            r = alone.turbine_record()
            np.testing.assert_array_equal(rec[k:k + len(r)], r)
            k += len(r)
