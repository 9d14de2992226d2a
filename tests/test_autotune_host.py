"""Host logic of the launch-schedule autotuner (no GPU): the per-kind choice."""
import math

from braids_hkt_gb300.autotune import KINDS, choose


def test_choose_takes_the_fastest_shape_per_kind():
    timings = {3: {(128, 32): 0.61, (64, 16): 0.58, (128, 8): 0.60},
               6: {(256, 32): 0.51, (128, 32): 0.53}}
    defaults = {3: (128, 32), 6: (256, 32)}
    out = choose(timings, defaults)
    assert out[3][:2] == (64, 16) and math.isclose(out[3][2], 0.58) and math.isclose(out[3][3], 0.61)
    assert out[6][:2] == (256, 32)


def test_choose_keeps_the_default_on_ties_and_skips_empty_kinds():
    timings = {2: {(64, 8): 0.7, (128, 32): 0.7}, 4: {}}
    out = choose(timings, {2: (128, 32), 4: (256, 32)})
    assert out[2][:2] == (128, 32)
    assert 4 not in out


def test_tunable_kinds_are_profile_kinds():
    # the donor limiter runs inside the update: no limit kind (5) in a substep
    assert set(KINDS["fwave"]) == {0, 2, 3, 4, 6, 11}
    assert set(KINDS["hllc"]) == {0, 20, 21, 23, 24, 26}
