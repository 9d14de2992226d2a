"""Four-face cells on the GPU: the Cartesian channel in the FP64 form
against the oracle (1e-10 with identical substep counts), the mixed form
against the FP64 form (1e-4 in depth), a lake at rest in both forms, and a
case built from geometry records (mesh_from_records) equal to the original."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def test_cartesian_fp64_oracle_and_mixed():
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = S.cartesian_channel()
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(case, precision="mixed")
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(3):
        da, db = a.advance(1.0, float(k)), b.advance(1.0, float(k))
        st, _, stats = o.advance(q, 1.0, float(k))
        assert st == 0 and da["failed"] == 0 and db["failed"] == 0
        assert da["hydraulic_substeps"] == stats["substeps"]
    scale = np.maximum(np.abs(q).max(axis=1, keepdims=True), 1e-3)
    assert (np.abs(a.state() - q) / scale).max() <= 1e-10
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() <= 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cartesian_lake_at_rest(precision):
    from braids_hkt_gb300.solver import RiverSolver
    case = S.cartesian_channel()
    case["forcing"] = np.array([[0.0, 0.0], [0.0, 3.0]])
    s = RiverSolver(case, precision=precision)
    s.advance(5.0, 0.0)
    q = s.state()
    wet = q[0] > 1e-6
    assert np.ptp((q[0] + case["z"])[wet]) <= 1e-12
    assert np.abs(q[1:]).max() <= 1e-10


def test_records_case_equals_original():
    from braids_hkt_gb300.mesh import mesh_from_records, records_of
    from braids_hkt_gb300.solver import RiverSolver
    case = S.cartesian_channel()
    adapted = dict(case, mesh=mesh_from_records(records_of(case["mesh"])))
    a, b = RiverSolver(case, precision="fp64"), RiverSolver(adapted, precision="fp64")
    a.advance(1.0, 0.0)
    b.advance(1.0, 0.0)
    np.testing.assert_array_equal(a.state(), b.state())


def test_cartesian_hllc_matches_oracle():
    """The HLLC method on four-face cells: GPU (FP64) against the oracle over
    three 1 s intervals, 1e-10 with identical substep counts."""
    from braids_hkt_gb300.solver import RiverSolver
    from oracle import Oracle
    case = S.cartesian_channel()
    s = RiverSolver(case, precision="fp64", method="hllc")
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    for k in range(3):
        d = s.advance(1.0, float(k))
        st, _, stats = o.hllc_advance(q, 1.0, float(k))
        assert st == 0 and d["failed"] == 0
        assert d["hydraulic_substeps"] == stats["substeps"]
    scale = np.maximum(np.abs(q).max(axis=1, keepdims=True), 1e-3)
    assert (np.abs(s.state() - q) / scale).max() <= 1e-10
