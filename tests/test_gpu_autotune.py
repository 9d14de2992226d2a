"""The launch-schedule autotuner on the GPU: it changes speed only.

After tuning, the state and step hints are those before it, every chosen
shape is within its kernel's limit, and an interval advanced with the tuned
schedule equals the same interval with the default schedule bit for bit
(grid-stride sweeps, order-free reductions).
"""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def batch():
    return [S.small_channel(), S.lake_at_rest(), S.dam_break(), S.small_rotor_channel()]


@pytest.mark.parametrize("precision,method", [("mixed", "fwave"), ("fp64", "fwave"), ("fp64", "hllc")])
def test_tuned_schedule_changes_nothing_but_speed(precision, method):
    from braids_hkt_gb300 import autotune
    from braids_hkt_gb300.solver import RiverSolver
    a = RiverSolver(batch(), precision=precision, method=method)
    b = RiverSolver(batch(), precision=precision, method=method)
    a.advance(0.5, 0.0)
    b.advance(0.5, 0.0)
    q0, h0 = a.state().copy(), a.hints().copy()
    rep = autotune.tune(a, reps=1, cache=False)
    np.testing.assert_array_equal(a.state(), q0)
    np.testing.assert_array_equal(a.hints(), h0)
    assert rep["chunk"] in autotune.CHUNKS and not rep["cached"]
    for k, (blk, per_sm) in rep["shapes"].items():
        assert (blk, per_sm) == a.launch_shape(int(k))[:2]
        assert blk % 32 == 0 and blk <= a.launch_shape(int(k))[2] and 1 <= per_sm <= 64
    da = a.advance(1.0, 0.5)
    db = b.advance(1.0, 0.5)
    assert [d["hydraulic_substeps"] for d in da] == [d["hydraulic_substeps"] for d in db]
    np.testing.assert_array_equal(a.state(), b.state())
