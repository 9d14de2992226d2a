"""The checkpoint format on the host: round trip, and every way a restart
must refuse (identity, inventory, shape, dtype, hash), before anything is
changed; the atomic write leaves no temporary and replaces the target."""
import io
import json

import numpy as np
import pytest

from braids_hkt_gb300 import checkpoint as CK

ID = dict(precision="mixed", method="fwave", scenarios=2, cells=10, faces=20, geometry_sha256="g", boundary_sha256="b")


def arrays(seed=0):
    rng = np.random.default_rng(seed)
    return dict(q=rng.normal(size=(3, 10)), z=rng.normal(size=10), hints=np.array([0.1, 0.2]))


def expected():
    return dict(q=((3, 10), np.float64), z=((10,), np.float64), hints=((2,), np.float64))


def test_round_trip_is_bitwise():
    a = arrays()
    out, header = CK.decode(CK.encode(ID, a, time=12.5, steps=7), ID, expected())
    for k in a:
        np.testing.assert_array_equal(out[k], a[k])
    assert header["time"] == 12.5 and header["steps"] == 7 and header["identity"] == ID


def test_identity_mismatch_refuses():
    other = dict(ID, geometry_sha256="h")
    with pytest.raises(ValueError, match="identity"):
        CK.decode(CK.encode(ID, arrays()), other, expected())


def test_inventory_shape_dtype_refuse():
    a = arrays()
    with pytest.raises(ValueError, match="inventory"):
        CK.decode(CK.encode(ID, dict(a, extra=np.zeros(1))), ID, expected())
    with pytest.raises(ValueError, match="shape or dtype"):
        CK.decode(CK.encode(ID, dict(a, z=np.zeros(11))), ID, expected())
    with pytest.raises(ValueError, match="shape or dtype"):
        CK.decode(CK.encode(ID, dict(a, z=np.zeros(10, np.float32))), ID, expected())


def test_tampered_array_fails_its_hash():
    a = arrays()
    payload = CK.encode(ID, a)
    with np.load(io.BytesIO(payload)) as saved:
        header = str(saved["metadata"])
        items = {k: np.array(saved[k]) for k in saved.files if k != "metadata"}
    items["q"][1, 3] += 1e-12
    stream = io.BytesIO()
    np.savez(stream, metadata=np.array(header), **items)
    with pytest.raises(ValueError, match="hash"):
        CK.decode(stream.getvalue(), ID, expected())


def test_header_is_json_with_format_and_hashes():
    with np.load(io.BytesIO(CK.encode(ID, arrays()))) as saved:
        header = json.loads(str(saved["metadata"]))
    assert header["format"] == CK.FORMAT and set(header["hashes"]) == {"q", "z", "hints"}


def test_atomic_write_replaces_and_leaves_no_temporary(tmp_path):
    path = tmp_path / "state.npz"
    CK.write_atomic(path, CK.encode(ID, arrays(1)))
    CK.write_atomic(path, CK.encode(ID, arrays(2)))
    out, _ = CK.decode(path.read_bytes(), ID, expected())
    np.testing.assert_array_equal(out["q"], arrays(2)["q"])
    assert [p.name for p in tmp_path.iterdir()] == ["state.npz"]
