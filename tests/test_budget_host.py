"""The owner's water-budget test on the host (shoreline_solver.py:29-39,
353-360): a volume change equal to the boundary ledger passes, one that
differs by more than the FP64 roundoff allowance fails, a nonfinite one fails.
The planted mistakes are host numbers, not GPU state."""
import numpy as np

from braids_hkt_gb300.solver import water_budget


def test_balanced_step_passes():
    v0 = np.array([1.0e6, 5.0e3])
    ledger = np.array([12.5, -0.75])
    v1 = v0 + ledger
    residual, allowance, ok = water_budget(v0, v1, ledger)
    assert ok.all()
    assert np.all(np.abs(residual) <= allowance)


def test_allowance_is_the_reference_formula():
    _, allowance, _ = water_budget([0.5, 2.0e7], [0.5, 2.0e7], [0.0, 3.0])
    eps = np.finfo(float).eps
    assert allowance[0] == 1e-10                       # the small-domain floor
    assert allowance[1] == 64 * eps * 2.0e7            # 64 eps x the inventory


def test_planted_residual_fails():
    v0 = np.array([2.0e7, 2.0e7])
    ledger = np.array([100.0, 100.0])
    v1 = v0 + ledger
    v1[1] += 1e-6                                       # 1 cm3 appears from nowhere
    _, _, ok = water_budget(v0, v1, ledger)
    assert ok.tolist() == [True, False]


def test_nonfinite_fails():
    _, _, ok = water_budget([1.0], [np.nan], [0.0])
    assert not ok.any()
