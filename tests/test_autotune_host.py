"""Host logic of the launch-schedule autotuner (no GPU): the per-kind choice and
the tile-sweep choice (a stand-in solver whose interval time depends on the tile)."""
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


class FakeTileSolver:
    """Stands in for a solver: interval 'time' depends on the tile set-up."""

    def __init__(self, precision="mixed", method="fwave", costs=None, refuse=()):
        self.precision, self.method = precision, method
        self.costs = costs or {}
        self.refuse = set(refuse)
        self.tile_cells, self.per_sm = 0, 4
        self.now = 0.0
        self.q = _Buffer()
        self.hints_set = None

    def set_tile(self, cells):
        if cells in self.refuse:
            raise RuntimeError("tile refused")
        self.tile_cells = cells

    def set_launch_shape(self, kind, block, per_sm):
        assert kind == 15 and block == 256
        self.per_sm = per_sm

    def set_hints(self, hints):
        self.hints_set = hints

    def advance(self, dt, time, raise_on_failure=True):
        key = "0" if not self.tile_cells else f"{self.tile_cells}x{self.per_sm}"
        self.now += self.costs.get(key, 10.0)

    def clock(self):
        return self.now


class _Buffer:
    def copy_(self, other):
        return self


def test_tile_tuner_picks_the_fastest_and_keeps_it():
    from braids_hkt_gb300.autotune import _tune_tile
    s = FakeTileSolver(costs={"0": 5.0, "128x2": 7.0, "128x4": 4.0, "256x2": 6.0, "256x4": 4.5, "512x2": 9.0,
                              "512x4": 8.0})
    out = _tune_tile(s, s.q, [0.01], 1e-3, 0.0, 0.1, (128, 256, 512), sync=lambda: None, clock=s.clock)
    assert out["cells"] == 128 and out["per_sm"] == 4
    assert s.tile_cells == 128 and s.per_sm == 4
    assert set(out["interval_ms"]) == {"0", "128x2", "128x4", "256x2", "256x4", "512x2", "512x4"}


def test_tile_tuner_keeps_the_separate_sweeps_when_they_win_and_skips_refused_sizes():
    from braids_hkt_gb300.autotune import _tune_tile
    s = FakeTileSolver(costs={"0": 3.0}, refuse={512})
    out = _tune_tile(s, s.q, [0.01], 1e-3, 0.0, 0.1, (128, 256, 512), sync=lambda: None, clock=s.clock)
    assert out["cells"] == 0 and s.tile_cells == 0
    assert not any(k.startswith("512") for k in out["interval_ms"])


def test_tile_tuner_has_nothing_to_tune_outside_the_mixed_fwave_form():
    from braids_hkt_gb300.autotune import _tune_tile
    for precision, method in (("fp64", "fwave"), ("mixed", "hllc")):
        s = FakeTileSolver(precision, method)
        assert _tune_tile(s, s.q, [0.01], 1e-3, 0.0, 0.1, (128,), sync=lambda: None, clock=s.clock) is None
