"""Mixed FP32/FP64 form of the HLLC / MUSCL-Hancock method against its FP64 form.

Bounds (the mixed form's stated tolerances): depth within 1e-4 relative of
the FP64 form (cells deeper than 1 mm: at least 1e-3 in the denominator),
unit discharge within 1e-3 of its largest value, rotor power within 1e-3
relative; a lake at rest stays at rest to FP64 round-off (the FP32 flux of a
surface at rest is exactly zero), closed-basin mass to 1e-12 relative (FP64
depth with FP64 weights), the owner's water budget passes on an open
channel, and scenarios batched in one solver equal each run alone, bit for
bit.
"""
import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
import braids_hkt_gb300.turbines as TB

pytestmark = pytest.mark.gpu

POWER = TB.DIAG_FIELDS.index("useful_power_per_density_m5_s3")


def solver(cases, precision="mixed"):
    from braids_hkt_gb300.solver import RiverSolver
    return RiverSolver(cases, precision=precision, method="hllc")


def test_hllc_mixed_lake_at_rest():
    case = S.lake_at_rest()
    s = solver(case)
    d = s.advance(5.0, 0.0)
    assert d["failed"] == 0 and d["hydraulic_substeps"] > 10
    q = s.state()
    assert np.abs(q[0] - case["q"][0]).max() < 1e-12
    assert np.abs(q[1:]).max() < 1e-11


def test_hllc_mixed_closed_basin_mass():
    case = S.lake_at_rest()
    s = solver(case)
    s.set_state(S.perturbed_state(case, 9, 0.4, 0.6, 0.05))
    v0 = s.mass()
    s.advance(3.0, 0.0)
    assert abs(s.mass() - v0) <= 1e-12 * v0
    dam = S.dam_break()
    t = solver(dam)
    v0 = t.mass()
    t.advance(3.0, 0.0)
    assert abs(t.mass() - v0) <= 1e-12 * v0


@pytest.mark.parametrize("build", [lambda: S.small_channel(length=400.0, width=60.0, spacing=3.0, discharge=60.0),
                                   S.stage_discharge_channel, S.dam_break])
def test_hllc_mixed_against_fp64(build):
    case = build()
    a, b = solver(case, "fp64"), solver(case, "mixed")
    for k in range(3):
        a.step(1.0)
        b.step(1.0)
    qa, qb = a.state(), b.state()
    rel = np.abs(qb[0] - qa[0]) / np.maximum(qa[0], 1e-3)
    print("hllc mixed depth error %.2e" % rel.max())
    assert rel.max() < 1e-4
    assert np.abs(qb[1:] - qa[1:]).max() <= 1e-3 * max(np.abs(qa[1:]).max(), 1e-12)


def test_hllc_mixed_rotors_against_fp64():
    case = S.small_rotor_channel(control=TB.rated_power_curve(5.0, 0.8, 0.4, 500e3))
    a, b = solver(case, "fp64"), solver(case, "mixed")
    for k in range(3):
        a.step(1.0)
        b.step(1.0)
    ha, hb = a.state()[0], b.state()[0]
    assert (np.abs(hb - ha) / np.maximum(ha, 1e-3)).max() < 1e-4
    pa, pb = a.turbine_record()[:, POWER], b.turbine_record()[:, POWER]
    assert (pa > 0).all()
    np.testing.assert_allclose(pb, pa, rtol=1e-3)


def test_hllc_mixed_batch_equals_alone():
    cases = [S.small_channel(seed=21, discharge=15.0), S.lake_at_rest(seed=5),
             S.small_rotor_channel(seed=23, rotors=1), S.dam_break(length=60.0)]
    batch = solver(cases)
    diags = batch.advance(1.5, 0.0)
    for i, case in enumerate(cases):
        alone = solver(case)
        d = alone.advance(1.5, 0.0)
        assert d["hydraulic_substeps"] == diags[i]["hydraulic_substeps"]
        np.testing.assert_array_equal(batch.state(i), alone.state())
