"""The C oracle's rotor array against the reference's own turbine code.

Fixtures (tests/golden/turbines, made by tests/golden/make_turbine_golden.py)
hold the reference's residual, substep and adaptive advance with two rotors in
four control modes, and its rotor diagnostics for every gate outcome. States
are bitwise; per-rotor sums within 1e-12 relative (numpy's pairwise sums
against sequential ones).
"""
import json
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
import braids_hkt_gb300.turbines as TB
from oracle import Oracle

GOLD = Path(__file__).parent / "golden" / "turbines"
MODES = ("constant", "curves", "table", "incident_table")
# oracle record columns of the reference diagnostic fields, in fixture order
COLUMNS = [TB.DIAG_FIELDS.index(f) for f in (
    "active", "minimum_coverage_margin_m", "minimum_bed_clearance_m", "local_velocity_m_s",
    "upstream_velocity_m_s", "mean_depth_m", "thrust_coefficient", "power_coefficient",
    "force_per_density_m4_s2", "useful_power_per_density_m5_s3", "hydraulic_power_removed_per_density_m5_s3")]


def load(name):
    z = np.load(GOLD / name)
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def steps():
    return load("rotor_steps.npz")


@pytest.mark.parametrize("mode", MODES)
def test_rotor_steps_bitwise(steps, mode):
    case = S.case_from_arrays(steps)
    case["turbines"] = json.loads(str(steps[f"{mode}_rows"]))
    o = Oracle(case, threads=2)
    q = case["q"]
    st, rate, _, _ = o.rate(q, 0.005)
    assert st == 0
    np.testing.assert_array_equal(rate, steps[f"{mode}_rate"])
    st, q2, _, _ = o.single(q, 0.01)
    assert st == 0
    np.testing.assert_array_equal(q2, steps[f"{mode}_single"])
    qa = q.copy()
    st, _, stats = o.advance(qa, 1.0)
    assert st == 0 and stats["substeps"] == int(steps[f"{mode}_substeps"])
    np.testing.assert_array_equal(qa, steps[f"{mode}_advance"])
    err, diag = o.diagnose(qa)
    assert err == 0
    np.testing.assert_allclose(diag[:, COLUMNS], steps[f"{mode}_diag"], rtol=1e-12, atol=0)


def test_rotor_gate_outcomes():
    g = load("rotor_gate.npz")
    case = S.case_from_arrays(g)
    names = [k[:-5] for k in g if k.endswith("_diag")]
    assert len(names) == 8
    for name in names:
        c = dict(case, turbines=json.loads(str(g[f"{name}_rows"])))
        o = Oracle(c, threads=2)
        state = str(g[f"{name}_state"])
        q = case["q"] if state == "initial" else g[f"{state}_q"]
        err, diag = o.diagnose(q)
        assert err == 0
        assert TB.REASONS[int(diag[0, TB.DIAG_FIELDS.index("reason")])] == name
        np.testing.assert_allclose(diag[:, COLUMNS], g[f"{name}_diag"], rtol=1e-12, atol=1e-15, err_msg=name)


def test_bump_integrals_partition():
    """Footprint integrals: every cell's part against a brute-force tensor
    Gauss rule on the clipped cell, and the sum against the 1-D integral."""
    case = S.small_rotor_channel(rotors=1)
    r = case["turbines"][0]
    cells, values = TB.bump_integrals(case["mesh"], r["X"], r["Y"], r["D"])
    expected = TB.bump_integral_1d() ** 2 * (r["D"] / 2) ** 2
    assert abs(values.sum() / expected - 1) < 1e-12
    # brute force: 400x400 midpoint samples of the square, binned by containing cell
    m = case["mesh"]
    n = 400
    s = (np.arange(n) + 0.5) / n * r["D"] - r["D"] / 2
    X, Y = np.meshgrid(s + r["X"], s + r["Y"], indexing="ij")
    from scipy.spatial import Delaunay
    owner = Delaunay(m.points).find_simplex(np.c_[X.ravel(), Y.ravel()])
    zx, zy = 2 * (X.ravel() - r["X"]) / r["D"], 2 * (Y.ravel() - r["Y"]) / r["D"]
    bump = np.exp(2 - 1 / (1 - zx ** 2) - 1 / (1 - zy ** 2)) * (r["D"] / n) ** 2
    # map Delaunay simplices of the points to mesh cells by vertex sets
    key = {tuple(sorted(t)): i for i, t in enumerate(m.tri)}
    simp = Delaunay(m.points).simplices
    cell_of = np.array([key.get(tuple(sorted(t)), -1) for t in simp])
    brute = np.bincount(cell_of[owner], weights=bump, minlength=m.nc)
    assert np.all(brute[cells] > 0)
    np.testing.assert_allclose(values, brute[cells], rtol=3e-2, atol=1e-5 * expected)   # pixelated cell edges


def test_rotor_plane_rows():
    case = S.small_rotor_channel(rotors=1)
    r = case["turbines"][0]
    rows, disp = TB.rotor_plane(case["mesh"], r["X"], r["Y"], r["D"])
    ends = case["mesh"].xy[:, rows] + disp
    assert np.allclose(ends[0], r["X"])
    assert ends[1].min() == pytest.approx(r["Y"] - r["D"] / 2) and ends[1].max() == pytest.approx(r["Y"] + r["D"] / 2)
    assert len(rows) % 2 == 0


def test_control_validation():
    with pytest.raises(ValueError):
        TB.validate_control({"mode": "constant_ct", "thrust_coefficient": 1.2, "power_coefficient": None})
    with pytest.raises(ValueError):
        TB.validate_control({"mode": "thetis_speed_table", "model_name": "x", "performance": [
            {"speed_m_s": 1.0, "thrust_coefficient": 0.8, "power_coefficient": 0.4},
            {"speed_m_s": 0.5, "thrust_coefficient": 0.8, "power_coefficient": 0.4}]})
    c = TB.rated_power_curve(5.0, 0.8, 0.4, 500e3)
    assert TB.validate_control(c)["mode"] == "incident_speed_curves"
