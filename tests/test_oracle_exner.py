"""The C oracle's Exner bed update against the reference's own kernels.

Fixtures (tests/golden/exner, made by tests/golden/make_exner_golden.py):
an open channel, the same with a thin erodible layer (donor limiter active)
and a prescribed feed, and a perturbed lake with dry cells (wet gating).
The trial bed is bitwise; the budget residual within 1e-15 absolute (numpy's
pairwise sum against a sequential one).
"""
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from oracle import Oracle

GOLD = sorted((Path(__file__).parent / "golden" / "exner").glob("*.npz"))


def load(path):
    z = np.load(path)
    g = {k: z[k] for k in z.files}
    case = S.case_from_arrays(g)
    case["exner"] = {k[3:]: (g[k].item() if g[k].ndim == 0 else g[k]) for k in g if k.startswith("ex_")}
    return case, g


@pytest.mark.parametrize("path", GOLD, ids=[p.stem for p in GOLD])
def test_exner_bitwise(path):
    case, g = load(path)
    o = Oracle(case, threads=2)
    code, zt, st = o.exner(g["input_q"], float(g["interval"]))
    assert code == 0 and st["ok"] == int(g["ok"])
    np.testing.assert_array_equal(zt, g["z_trial"])
    assert abs(st["residual"] - float(g["residual"])) <= 1e-15
    assert st["donor"] == float(g["donor"]) and st["change"] == float(g["change"])
    assert abs(st["boundary"] - float(g["boundary"])) <= 1e-15 * max(1.0, abs(float(g["boundary"])))


def test_exner_conserves_solid_volume():
    """Closed basin: the bed change integrates to zero (budget residual only)."""
    case = S.lake_at_rest(islands=False)
    case["exner"] = S.exner_params(case, diameter=0.002, chezy=30.0)
    q = S.perturbed_state(case, 3, 0.2, 0.6, 0.0)
    o = Oracle(case, threads=2)
    code, zt, st = o.exner(q, 1.0)
    assert code == 0 and st["ok"]
    phi = 1 - case["exner"]["porosity"]
    assert abs(np.sum(phi * (zt - case["z"]) * case["mesh"].area)) < 1e-12
    assert np.abs(zt - case["z"]).max() > 0
