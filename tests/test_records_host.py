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


def test_side_major_displacement_converted():
    """The geometry cache's (4, nf) displacement (owner x, y, neighbour x, y)
    gives the same mesh as the exporter's (2, 2, nf) layout."""
    m = S.small_channel()["mesh"]
    d = records_of(m)
    disp = d["displacement"]
    d["displacement"] = np.stack((disp[0, 0], disp[1, 0], disp[0, 1], disp[1, 1]))
    m2 = mesh_from_records(d)
    for k in ("disp", "disp_len"):
        np.testing.assert_array_equal(m2.records[k], m.records[k], err_msg=k)


@pytest.mark.parametrize("key,shape", [("displacement", (3, 7)), ("ls_matrix", (3, 5)), ("ls_delta", (4, 2)),
                                       ("ls_weight", (9,)), ("distance", (1, 4))])
def test_misshapen_records_refused(key, shape):
    d = records_of(S.small_channel()["mesh"])
    d[key] = np.zeros(shape)
    with pytest.raises(ValueError):
        mesh_from_records(d)
