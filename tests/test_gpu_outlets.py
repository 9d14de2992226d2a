"""Outlet section owners on the GPU: the Q-H rating (mode 11), normal-depth
(mode 10), free-weir (mode 5) and critical (mode 4) outlets against
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


@pytest.mark.parametrize("make", [S.normal_channel, S.weir_channel, S.critical_channel],
                         ids=["normal", "weir", "critical"])
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
    cases = [S.small_channel(), S.rating_channel(), S.normal_channel(), S.weir_channel(), S.critical_channel()]
    batch = RiverSolver(cases, precision="mixed")
    batch.advance(2.0, 0.0)
    for i, c in enumerate(cases):
        one = RiverSolver(c, precision="mixed")
        one.advance(2.0, 0.0)
        np.testing.assert_array_equal(batch.state(i), one.state())
