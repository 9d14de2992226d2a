"""Conservative wet-bank viscosity on the GPU against the oracle.

The oracle's term equals the reference's own kernels bit for bit
(tests/test_oracle_viscosity.py). FP64 form: one residual within 1e-12 of
each row's scale, a 2 s adaptive advance within 1e-10 with the same substep
count; mixed form: depth within 1e-4 relative of the FP64 form; scenarios
with and without the term batched in one solver equal each alone; the HLLC
method refuses it.
"""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def banks(nu=0.05):
    case = S.small_channel(length=200.0, width=30.0, spacing=3.0, discharge=150.0)
    case["viscosity"] = nu
    return case


def scaled(a, b):
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-3)
    return float((np.abs(np.asarray(a) - b) / scale).max())


def test_viscosity_rate_matches_oracle():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = banks()
    q = S.perturbed_state(case, 31, 0.3, 0.8, 0.12)
    s = RiverSolver(case, precision="fp64")
    s.set_state(q)
    rate, water, status, freq = s.rate(0.005)
    st, rate_o, water_o, freq_o = Oracle(case, threads=4).rate(q, 0.005)
    assert status == 0 and st == 0
    assert scaled(rate.cpu().numpy(), rate_o) <= 1e-12
    # the term is there: the same residual without it differs
    plain = RiverSolver(banks(0.0), precision="fp64")
    plain.set_state(q)
    r0 = plain.rate(0.005)[0].cpu().numpy()
    assert np.abs(r0 - rate_o)[1:].max() > 1e-6


def test_viscosity_advance_matches_oracle():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = banks()
    s = RiverSolver(case, precision="fp64")
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(2):
        d = s.advance(1.0, float(k))
        st, _, stats = o.advance(q, 1.0, float(k))
        assert st == 0 and d["failed"] == 0
        assert d["hydraulic_substeps"] == stats["substeps"]
    assert scaled(s.state(), q) <= 1e-10


def test_viscosity_mixed_against_fp64():
    from braids_hkt_gb300.solver import RiverSolver
    case = banks(0.5)
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(case, precision="mixed")
    for k in range(3):
        a.step(1.0)
        b.step(1.0)
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_viscosity_batch_equals_alone(precision):
    from braids_hkt_gb300.solver import RiverSolver
    cases = [banks(0.05), S.small_channel(seed=31, discharge=12.0), dict(S.lake_at_rest(), viscosity=0.2)]
    cases[2]["q"] = S.perturbed_state(cases[2], 5, 0.3, 0.5, 0.1)
    batch = RiverSolver(cases, precision=precision)
    batch.advance(1.0, 0.0)
    for i, case in enumerate(cases):
        alone = RiverSolver(case, precision=precision)
        alone.advance(1.0, 0.0)
        np.testing.assert_array_equal(batch.state(i), alone.state())


def test_viscosity_refused_with_hllc():
    from braids_hkt_gb300.solver import RiverSolver
    with pytest.raises(Exception):
        RiverSolver(banks(), precision="fp64", method="hllc")
