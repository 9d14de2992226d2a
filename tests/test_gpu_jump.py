"""Stationary hydraulic jump through the CUDA path: FP64 against the oracle,
mixed against FP64, both holding Belanger's conjugate depths.

Mixed against FP64: depth within 1e-4 relative away from the jump (more
than 3 m from it); across the bore itself a sub-cell difference in the
front position is an O(1) difference in a few cells (measured 1.1%), so
there the jump positions are compared instead (within one cell spacing)."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def test_hydraulic_jump_fp64_oracle_and_mixed():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = S.hydraulic_jump()
    j = case["jump"]
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(case, precision="mixed")
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(4):
        da, db = a.advance(5.0, 5.0 * k), b.advance(5.0, 5.0 * k)
        st, _, stats = o.advance(q, 5.0, 5.0 * k)
        assert st == 0 and da["failed"] == 0 and db["failed"] == 0
        assert da["hydraulic_substeps"] == stats["substeps"]
    qa, qb = a.state(), b.state()
    scale = np.abs(q).max(axis=1, keepdims=True)
    assert (np.abs(qa - q) / scale).max() <= 1e-10
    x, y = case["mesh"].xy
    band = np.abs(y - 1.5) < 1.0
    mid = 0.5 * (j["h1"] + j["h2"])
    xa, xb = x[band & (qa[0] > mid)].min(), x[band & (qb[0] > mid)].min()
    assert abs(xa - xb) <= 0.5
    smooth = np.abs(x - xa) > 3.0
    assert (np.abs(qb[0] - qa[0]) / qa[0])[smooth].max() <= 1e-4
    dn = (x > 40) & (x < 55)
    for s in (qa, qb):
        assert abs(s[0][dn].mean() - j["h2"]) <= 0.02 * j["h2"]
