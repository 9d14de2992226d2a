"""HLLC / MUSCL-Hancock option on the GPU against the oracle and the reference fixtures.

The CUDA path runs the FP64 form with the reference's operation order
(no contraction, IEEE divide and square root). Bounds: states within 1e-12
of each row's scale (at least 1e-3) after one Hancock step and 1e-10 after three adaptive
1 s intervals, with the same accepted and rejected substep counts as the
reference's own operator (tests/golden/hllc, made by
tests/golden/make_hllc_golden.py) and as the oracle run on this machine.
The golden state and bed are loaded into the case so that both sides start
from the same bits on any host.
"""
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden" / "hllc"
BUILDERS = {"channel": S.small_channel, "lake": S.lake_at_rest, "dam_break": S.dam_break,
            "stage_discharge": S.stage_discharge_channel,
            "rotors": S.small_rotor_channel}


def case_of(name):
    g = np.load(GOLD / f"{name}.npz")
    case = BUILDERS[name]()
    case["q"] = np.ascontiguousarray(g["q0"]).copy()
    case["z"] = np.ascontiguousarray(g["z"]).copy()
    return case, g


def solver(cases, **kw):
    from braids_hkt_gb300.solver import RiverSolver
    return RiverSolver(cases, precision="fp64", method="hllc", **kw)


def rel(a, b):
    """Largest difference over each row's scale; a row at round-off level
    (the still lake's momentum, ~1e-17) is scaled by at least 1e-3."""
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-3)
    return float((np.abs(np.asarray(a) - b) / scale).max())


@pytest.mark.parametrize("name", sorted(BUILDERS))
def test_hllc_step_matches_reference(name):
    case, g = case_of(name)
    s = solver(case)
    status, peak = s.substep(float(g["step_dt"]))
    assert int(status) == 0
    assert abs(float(peak) - float(g["step_frequency"])) <= 1e-12 * float(g["step_frequency"])
    assert rel(s.state(), g["step_q"]) <= 1e-12


@pytest.mark.parametrize("name", sorted(BUILDERS))
def test_hllc_advance_matches_reference_and_oracle(name):
    from oracle import Oracle
    case, g = case_of(name)
    s = solver(case)
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    dt = float(g["dt"])
    for k in range(len(g["q"])):
        d = s.advance(dt, k * dt)
        st, _, stats = o.hllc_advance(q, dt, k * dt)
        assert st == 0 and d["failed"] == 0
        assert d["hydraulic_substeps"] == g["substeps"][k] == stats["substeps"]
        assert d["hydraulic_rejections"] == g["retries"][k] == stats["rejections"]
        qs = s.state()
        assert rel(qs, g["q"][k]) <= 1e-10
        assert rel(qs, q) <= 1e-10


def test_hllc_batch_matches_single_scenarios():
    """All four cases packed in one solver: each scenario on its own clock, as if alone."""
    names = sorted(BUILDERS)
    pairs = [case_of(n) for n in names]
    s = solver([c for c, _ in pairs])
    for k in range(3):
        diags = s.advance(1.0, float(k))
        for i, (n, (_, g)) in enumerate(zip(names, pairs)):
            assert diags[i]["hydraulic_substeps"] == g["substeps"][k], n
            assert rel(s.state(i), g["q"][k]) <= 1e-10, n


def test_hllc_lake_at_rest_and_mass():
    case, g = case_of("lake")
    s = solver(case)
    area = case["mesh"].area
    v0 = float(np.sum(case["q"][0] * area))
    for k in range(3):
        s.advance(1.0, float(k))
    q = s.state()
    wet = q[0] > 1e-6
    eta = (q[0] + case["z"])[wet]
    assert np.ptp(eta) <= 1e-12
    assert np.abs(q[1:]).max() <= 1e-12
    assert abs(float(np.sum(q[0] * area)) - v0) <= 1e-12 * v0


def test_hllc_closed_dam_break_conserves_mass():
    case, g = case_of("dam_break")
    s = solver(case)
    area = case["mesh"].area
    v0 = float(np.sum(case["q"][0] * area))
    for k in range(3):
        s.advance(1.0, float(k))
    assert abs(float(np.sum(s.state()[0] * area)) - v0) <= 1e-12 * v0


def test_hllc_asynchronous_interval_matches_advance():
    case, g = case_of("channel")
    a, b = solver(case), solver(case)
    a.advance(1.0, 0.0)
    b.advance_start(np.array([1.0]), np.array([0.0]))
    diags = None
    while diags is None:
        diags = b.advance_poll()
    assert diags[0]["hydraulic_substeps"] == g["substeps"][0]
    np.testing.assert_array_equal(a.state(), b.state())


def test_hllc_rotor_record_after_advance():
    """Rotor diagnostics of the HLLC-advanced state match the oracle's on the same state."""
    from oracle import Oracle
    case, g = case_of("rotors")
    s = solver(case)
    s.advance(1.0, 0.0)
    rec = s.turbine_record()
    err, rec_o = Oracle(case, threads=4).diagnose(s.state())
    assert err == 0
    np.testing.assert_allclose(rec[:, :15], rec_o[:, :15], rtol=1e-8, atol=1e-12)


def test_hllc_scope_errors():
    """The mixed HLLC form has no rotor ambient stress: a rotor array with a
    positive ambient viscosity is refused there."""
    from braids_hkt_gb300.solver import RiverSolver
    case = S.small_rotor_channel(nu=0.005)
    with pytest.raises(Exception):
        RiverSolver(case, precision="mixed", method="hllc")
