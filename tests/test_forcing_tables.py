"""Forcing tables: the oracle's sampling against a restatement of the
reference's RiverHydraulicSchedule.sample (river_hydraulic_schedule.py:57-65):
knot = last time at or before t (capped at len - 2), value (1-w) y_i + w y_i+1,
bitwise, including the knots themselves."""
import numpy as np

import braids_hkt_gb300.scenarios as S
from oracle import Oracle


def reference_sample(times, series, t):
    i = min(int(np.searchsorted(times, t, side="right")) - 1, len(times) - 2)
    w = (t - times[i]) / (times[i + 1] - times[i])
    return (1. - w) * series[i] + w * series[i + 1]


def test_table_sampling_bitwise():
    case = S.small_channel()
    times = np.array([0.0, 7.3, 60.0, 61.5, 300.0])
    q = np.array([10.0, 13.7, 40.1, 40.0, 25.3])
    stage = np.array([2.0, 2.1, 2.7, 2.69, 2.4])
    nb = case["mesh"].nb
    value = np.zeros((2, nb, len(times)))
    value[0, 0] = q
    value[1, 1] = stage
    case["table_time"], case["table_value"] = times, value
    o = Oracle(case, threads=1)
    rng = np.random.default_rng(3)
    for t in list(times) + list(rng.uniform(0.0, 300.0, 200)):
        f = o.sample_forcing(t)
        assert f[0, 0] == reference_sample(times, q, t)
        assert f[1, 1] == reference_sample(times, stage, t)
