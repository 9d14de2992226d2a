"""The C oracle's HLLC / MUSCL-Hancock option against the reference's own operator.

Golden vectors: tests/golden/hllc/*.npz, made by tests/golden/make_hllc_golden.py
from the reference's HLLCHydraulics (src/braids_core/hydraulics/hllc.py) and
its host-compiled kernels. The oracle restatement must reproduce them bit for
bit: one Hancock step's internals, and three adaptive 1 s intervals (states,
substep and retry counts, interval-mean water flux, the step hint).
"""
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from oracle import Oracle

GOLD = Path(__file__).resolve().parent / "golden" / "hllc"
BUILDERS = {"channel": S.small_channel, "lake": S.lake_at_rest, "dam_break": S.dam_break,
            "stage_discharge": S.stage_discharge_channel,
            "rotors": S.small_rotor_channel}


def _case(name):
    g = np.load(GOLD / f"{name}.npz")
    case = BUILDERS[name]()
    np.testing.assert_array_equal(np.asarray(case["q"], dtype=np.float64), g["q0"])
    np.testing.assert_array_equal(np.asarray(case["z"], dtype=np.float64), g["z"])
    return case, g


@pytest.mark.parametrize("name", sorted(BUILDERS))
def test_hllc_step_internals_bitwise(name):
    case, g = _case(name)
    o = Oracle(case)
    st, out, water, peak, k = o.hllc_step(g["q0"], float(g["step_dt"]), 0.0)
    assert st == 0
    assert peak == float(g["step_frequency"])
    for key in ("grad", "half", "qhalf", "fl", "fr", "speed", "theta", "freq", "next"):
        np.testing.assert_array_equal(k[key], g[f"step_{key}"], err_msg=key)
    np.testing.assert_array_equal(out, g["step_q"])
    np.testing.assert_array_equal(water, g["step_water"])


@pytest.mark.parametrize("name", sorted(BUILDERS))
def test_hllc_advance_bitwise(name):
    case, g = _case(name)
    o = Oracle(case)
    q = np.ascontiguousarray(g["q0"]).copy()
    dt = float(g["dt"])
    for k in range(len(g["q"])):
        st, water, stats = o.hllc_advance(q, dt, k * dt)
        assert st == 0
        assert stats["substeps"] == g["substeps"][k] and stats["rejections"] == g["retries"][k]
        assert stats["hint"] == g["hint"][k]
        np.testing.assert_array_equal(q, g["q"][k])
        np.testing.assert_array_equal(water, g["water"][k])


def test_hllc_lake_at_rest_holds():
    """The still lake with emerged islands stays still under HLLC (hydrostatic reconstruction)."""
    case, g = _case("lake")
    q = g["q"][-1]
    eta = (q[0] + g["z"])[q[0] > 1e-6]
    assert np.ptp(eta) < 1e-12
    assert np.abs(q[1:]).max() < 1e-12
