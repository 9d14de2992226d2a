"""A case built from a reference owner's geometry records (mesh_from_records):
the records round-trip, the oracle advances the adapted case bit for bit as
the original, and incomplete records are refused."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from braids_hkt_gb300.mesh import mesh_from_records, records_of
from oracle import Oracle


def test_records_round_trip():
    case = S.small_channel()
    m = case["mesh"]
    m2 = mesh_from_records(records_of(m))
    for k in ("owner", "neighbour", "bid", "normal", "length", "mid", "area", "xy", "offset", "faces", "signs",
              "boundary_offset", "boundary_faces"):
        np.testing.assert_array_equal(getattr(m2, k), getattr(m, k), err_msg=k)
    for k in ("ls_matrix", "ls_weight", "ls_delta", "disp", "disp_len", "distance"):
        np.testing.assert_array_equal(m2.records[k], m.records[k], err_msg=k)


def test_adapted_case_advances_bitwise():
    case = S.stage_discharge_channel()
    adapted = dict(case, mesh=mesh_from_records(records_of(case["mesh"])))
    q1, q2 = case["q"].copy(), case["q"].copy()
    st1, w1, s1 = Oracle(case, threads=2).advance(q1, 1.0, 0.0)
    st2, w2, s2 = Oracle(adapted, threads=2).advance(q2, 1.0, 0.0)
    assert st1 == st2 == 0 and s1["substeps"] == s2["substeps"]
    np.testing.assert_array_equal(q1, q2)
    np.testing.assert_array_equal(w1, w2)


def test_incomplete_records_refused():
    d = records_of(S.small_channel()["mesh"])
    del d["distance"]
    with pytest.raises(ValueError):
        mesh_from_records(d)
