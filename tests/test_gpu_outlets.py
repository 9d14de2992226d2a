"""Section owners on the GPU: the Q-H rating (mode 11), normal-depth
(mode 10), free-weir (mode 5) and critical (mode 4) outlets and the
exact-discharge inlet (mode 9, with the forcing, critical-depth and
normal-depth reference lines) against
the oracle (FP64 to 1e-10 with identical substep counts; mixed against FP64
to 1e-4 in depth) and its failure without a bracket (the scenario fails,
failed = 5). The reference fixture is checked in test_gpu_parity."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def test_rating_outlet_fp64_oracle_and_mixed():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = S.rating_channel()
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(case, precision="mixed")
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(4):
        da, db = a.advance(2.0, 2.0 * k), b.advance(2.0, 2.0 * k)
        st, _, stats = o.advance(q, 2.0, 2.0 * k)
        assert st == 0 and da["failed"] == 0 and db["failed"] == 0
        assert da["hydraulic_substeps"] == stats["substeps"]
    scale = np.abs(q).max(axis=1, keepdims=True)
    assert (np.abs(a.state() - q) / scale).max() <= 1e-10
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() <= 1e-4


def test_rating_outlet_without_a_bracket_fails_the_scenario():
    from braids_hkt_gb300.solver import RiverSolver
    bad = S.rating_channel(knots=((0.0, -5.0), (1.0, -4.0)))
    good = S.rating_channel()
    s = RiverSolver([good, bad], precision="fp64")
    d = s.advance(1.0, 0.0, raise_on_failure=False)
    assert d[0]["failed"] == 0 and d[1]["failed"] == 5


@pytest.mark.parametrize("make", [S.normal_channel, S.weir_channel, S.critical_channel, S.stage_discharge_channel,
                                  S.critical_inlet_channel, S.normal_inlet_channel],
                         ids=["normal", "weir", "critical", "stage_discharge_inlet", "critical_inlet", "normal_inlet"])
def test_section_outlet_fp64_oracle_and_mixed(make):
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = make()
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(case, precision="mixed")
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(4):
        da, db = a.advance(2.0, 2.0 * k), b.advance(2.0, 2.0 * k)
        st, _, stats = o.advance(q, 2.0, 2.0 * k)
        assert st == 0 and da["failed"] == 0 and db["failed"] == 0
        assert da["hydraulic_substeps"] == stats["substeps"]
    scale = np.abs(q).max(axis=1, keepdims=True)
    assert (np.abs(a.state() - q) / scale).max() <= 1e-10
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() <= 1e-4


def test_outlet_modes_batched_equal_alone():
    """Rating and normal-depth outlets in one batch with the stage-outlet channel: bitwise as alone."""
    from braids_hkt_gb300.solver import RiverSolver
    cases = [S.small_channel(), S.rating_channel(), S.normal_channel(), S.weir_channel(), S.critical_channel(),
             S.stage_discharge_channel(), S.critical_inlet_channel(), S.normal_inlet_channel()]
    batch = RiverSolver(cases, precision="mixed")
    batch.advance(2.0, 0.0)
    for i, c in enumerate(cases):
        one = RiverSolver(c, precision="mixed")
        one.advance(2.0, 0.0)
        np.testing.assert_array_equal(batch.state(i), one.state())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("discharge", [5.0, 35.0])
def test_inlet_net_discharge_exact_on_gpu(precision, discharge):
    """The exact-discharge inlet's boundary water flux of one residual: the
    net section discharge equals the request within the reference's bound
    (1e-10 Q + 1024 eps x gross throughflow). The mixed form solves the
    section in FP64 and carries each open face's water flux in FP32, so its
    bound adds one FP32 rounding of the gross throughflow (2^-23 x gross)."""
    from braids_hkt_gb300.solver import RiverSolver
    case = S.stage_discharge_channel(discharge=discharge)
    case["q"] = S.perturbed_state(case, 12, 0.2, 0.4, 0.0)
    s = RiverSolver(case, precision=precision)
    _, water, status, _ = s.rate(0.01)
    assert int(status) == 0
    m = case["mesh"]
    faces = np.asarray(m.boundary_faces)[m.boundary_offset[0]:m.boundary_offset[1]]
    flow = -water.cpu().numpy()[faces] * m.length[faces]
    gross = np.abs(flow).sum()
    bound = 1e-10 * discharge + 1024 * np.finfo(float).eps * gross
    if precision == "mixed":
        bound += 2.0 ** -23 * gross
    assert abs(flow.sum() - discharge) <= bound


@pytest.mark.parametrize("make", [S.critical_inlet_channel, S.normal_inlet_channel], ids=["critical", "normal"])
def test_inlet_line_matches_oracle(make):
    """The reference line the GPU solved (the forcing stage row after one
    residual) equals the oracle's line within 1e-12 (cube root, pow and log
    of the CUDA library against the host's)."""
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = make()
    s = RiverSolver(case, precision="fp64")
    s.rate(0.01)
    o = Oracle(case, threads=1)
    st, _, _, _ = o.rate(case["q"], 0.01)
    assert st == 0
    line = s.forcing()[1, 0]
    assert abs(line - o.forcing[1, 0]) <= 1e-12 * max(1.0, abs(o.forcing[1, 0]))
