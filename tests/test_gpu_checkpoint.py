"""Checkpoint and restart of a resident batch on the GPU: a restarted solver
continues bit for bit as the one that wrote the checkpoint; a checkpoint of
another set-up is refused and changes nothing."""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def cases():
    return [S.small_channel(), S.rating_channel(), S.small_rotor_channel()]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_restart_continues_bitwise(tmp_path, precision):
    from braids_hkt_gb300.solver import RiverSolver
    a = RiverSolver(cases(), precision=precision)
    a.advance(1.0, 0.0)
    path = tmp_path / "river.npz"
    a.checkpoint(path, time=1.0, steps=1)
    a.advance(1.0, 1.0)
    b = RiverSolver(cases(), precision=precision)
    header = b.restart(path)
    assert header["time"] == 1.0 and header["steps"] == 1
    b.advance(1.0, header["time"])
    np.testing.assert_array_equal(a.state(0), b.state(0))
    np.testing.assert_array_equal(a.q.cpu().numpy(), b.q.cpu().numpy())
    np.testing.assert_array_equal(a.hints(), b.hints())


def test_restart_refuses_another_setup(tmp_path):
    from braids_hkt_gb300.solver import RiverSolver
    a = RiverSolver(cases(), precision="mixed")
    a.advance(0.5, 0.0)
    path = tmp_path / "river.npz"
    a.checkpoint(path)
    other = RiverSolver(cases()[:2], precision="mixed")
    before = other.q.cpu().numpy().copy()
    with pytest.raises(ValueError, match="identity"):
        other.restart(path)
    np.testing.assert_array_equal(other.q.cpu().numpy(), before)
    fp64 = RiverSolver(cases(), precision="fp64")
    with pytest.raises(ValueError, match="identity"):
        fp64.restart(path)
