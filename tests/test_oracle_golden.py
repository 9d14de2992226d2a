"""The C oracle against golden vectors produced by the reference's own kernels.

The fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py) hold the
outputs of the reference's host-compiled hot-path kernels and its stock-budget
classes on five small cases. Parity is bitwise: the oracle restates the FP64
arithmetic operation for operation with FMA contraction disabled.
"""
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from oracle import Oracle

GOLDEN = sorted((Path(__file__).parent / "golden").glob("*.npz"))


def load(path):
    z = np.load(path)
    arrs = {k: z[k] for k in z.files}
    return S.case_from_arrays(arrs), arrs


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_kernels_bitwise(path):
    case, g = load(path)
    o = Oracle(case, threads=2)
    out = o.kernels(g["input_q"])
    for key in ("v", "active", "grad", "constant", "trace", "kind", "local", "closed", "riemann", "astatus"):
        np.testing.assert_array_equal(out[key], g[f"k_{key}"], err_msg=key)
    inner = ~((case["mesh"].neighbour < 0) & (case["mesh"].bid >= 0))   # open faces belong to the exterior owner
    for key in ("fl", "fr", "speed", "fstatus"):
        np.testing.assert_array_equal(out[key][..., inner], g[f"k_{key}"][..., inner], err_msg=key)


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_rate_and_substep_bitwise(path):
    case, g = load(path)
    o = Oracle(case, threads=2)
    q = g["input_q"]
    dt = float(g["dt"])
    st, rate, water, freq = o.rate(q, dt, 0.0)
    assert st == 0
    np.testing.assert_array_equal(rate, g["rate"])
    np.testing.assert_array_equal(water, g["water"])
    assert freq == float(g["freq"])
    st, q2, w2, peak = o.single(q, dt, 0.0)
    assert st == 0
    np.testing.assert_array_equal(q2, g["single_q"])
    np.testing.assert_array_equal(w2, g["single_water"])
    assert peak == float(g["single_peak"])


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_advance_bitwise(path):
    case, g = load(path)
    o = Oracle(case, threads=2)
    q = np.ascontiguousarray(g["input_q"].copy())
    st, water, stats = o.advance(q, float(g["interval"]), 0.0)
    assert st == 0
    np.testing.assert_array_equal(q, g["advance_q"])
    np.testing.assert_array_equal(water, g["advance_water"])
    for key in ("substeps", "rejections", "min_dt", "max_dt", "accepted_cfl_max", "hint"):
        assert stats[key] == g[f"advance_{key}"].item(), key


def test_fixture_coverage():
    """The fixtures exercise wet/dry fronts, closed faces, walls, open boundaries and rejections."""
    kinds, closed, rejections, dry = set(), 0, 0, 0
    for path in GOLDEN:
        case, g = load(path)
        kinds |= set(np.unique(g["k_kind"]).tolist())
        closed += int(g["k_closed"].sum())
        rejections += int(g["advance_rejections"])
        dry += int((g["input_q"][0] <= 1e-6).sum())
    assert {0, 1, 2, 3} <= kinds
    assert closed > 0 and rejections > 0 and dry > 0
