"""A hydrograph on the GPU: the inlet discharge follows a piecewise-linear
table while the channel advances; FP64 state within 1e-10 of the oracle with
the same substep counts, and the imposed discharge reaches the channel."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def hydrograph_case():
    case = S.small_channel(length=120.0, width=24.0, spacing=4.0, discharge=10.0)
    times = np.array([0.0, 5.0, 20.0, 60.0])
    value = np.zeros((2, case["mesh"].nb, len(times)))
    value[0, 0] = [10.0, 10.0, 40.0, 25.0]           # inlet discharge [m3/s]
    value[1, 1] = case["forcing"][1, 1]                # outlet stage held
    case["table_time"], case["table_value"] = times, value
    return case


def test_hydrograph_matches_oracle():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = hydrograph_case()
    s = RiverSolver(case, precision="fp64")
    s.set_forcing_table(case["table_time"], case["table_value"])
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(6):
        d = s.advance(4.0, 4.0 * k)
        st, _, stats = o.advance(q, 4.0, 4.0 * k)
        assert st == 0 and d["failed"] == 0 and d["hydraulic_substeps"] == stats["substeps"]
        scale = np.abs(q).max(axis=1, keepdims=True)
        assert (np.abs(s.state() - q) / scale).max() <= 1e-10


def test_hydrograph_mixed_follows_fp64():
    from braids_hkt_gb300.solver import RiverSolver
    case = hydrograph_case()
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(case, precision="mixed")
    for s in (a, b):
        s.set_forcing_table(case["table_time"], case["table_value"])
    for k in range(6):
        a.advance(4.0, 4.0 * k)
        b.advance(4.0, 4.0 * k)
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() < 1e-4
