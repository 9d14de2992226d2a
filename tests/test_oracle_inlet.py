"""The exact-discharge inlet (mode 9) in the C oracle.

Parity: the inlet section solve is pinned through the reference's own
CompatibleInlet owner and host-built kernel (tests/golden/
stage_discharge_inlet.npz, checked bit for bit by test_oracle_golden.py); the
stock-aware allocation is pinned here against the reference's
OutletFeasibility + InletFeasibility classes (tests/golden/feasibility, made
by tests/golden/make_feasibility_golden.py). Known answers: the net section
discharge of the boundary Riemann fluxes equals the requested Q within the
reference's acceptance bound (1e-10 Q + 1024 eps x gross throughflow), and a
zero request closes every inlet face.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S
from oracle import Oracle

FEAS = sorted((Path(__file__).parent / "golden" / "feasibility").glob("*.npz"))
EPS = np.finfo(float).eps


@pytest.mark.parametrize("path", FEAS, ids=[p.stem for p in FEAS])
def test_allocation_matches_reference(path):
    z = np.load(path)
    arrs = {k: z[k] for k in z.files}
    case = S.case_from_arrays(arrs)
    o = Oracle(case, threads=1)
    flux, trace = arrs["flux"].copy(), arrs["trace"].copy()
    o.boundary_allocation(arrs["base"], float(arrs["dt"]), flux, trace)
    np.testing.assert_array_equal(flux, arrs["flux_out"])
    np.testing.assert_array_equal(trace, arrs["trace_out"])


def test_allocation_fixture_coverage():
    changed = {p.stem: int(np.sum(np.load(p)["flux_out"] != np.load(p)["flux"])) for p in FEAS}
    assert changed["cap"] > 0 and changed["infeasible"] == 0 and changed["pass"] == 0


def exterior(o, q, time=0.0):
    m = o.m
    nf, nb = m.nf, len(o.seg_mode)
    trace, flux = np.zeros((3, nf)), np.zeros((3, nf))
    status = np.zeros(nf, np.int32)
    work = np.zeros(3 * nf + 3 * m.nc)
    stage, total = np.zeros(2 * nb), np.zeros(nb)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    st = o.L.om_exterior(o.cp, p(np.ascontiguousarray(q)), p(o.z), float(time), p(trace), p(flux), p(status),
                         p(work), p(stage), p(total))
    return st, trace, flux, status


@pytest.mark.parametrize("discharge", [5.0, 20.0, 60.0])
def test_net_section_discharge_is_exact(discharge):
    case = S.stage_discharge_channel(discharge=discharge)
    o = Oracle(case, threads=1)
    q = S.perturbed_state(case, 12, 0.2, 0.4, 0.0)
    st, trace, flux, status = exterior(o, q)
    assert st == 0 and not status.any()
    m = case["mesh"]
    faces = np.asarray(m.boundary_faces)[m.boundary_offset[0]:m.boundary_offset[1]]
    rate = -flux[0, faces] * m.length[faces]
    gross = np.abs(rate).sum()
    assert abs(rate.sum() - discharge) <= 1e-10 * discharge + 1024 * EPS * gross
    np.testing.assert_array_equal(trace[0, faces] > 0, True)


def test_zero_discharge_closes_the_inlet():
    case = S.stage_discharge_channel(discharge=0.0)
    o = Oracle(case, threads=1)
    q = S.perturbed_state(case, 13, 0.2, 0.4, 0.0)
    st, trace, flux, status = exterior(o, q)
    assert st == 0
    m = case["mesh"]
    faces = np.asarray(m.boundary_faces)[m.boundary_offset[0]:m.boundary_offset[1]]
    assert np.all(flux[0, faces] == 0.0)
    # reflected-owner pressure only: the normal momentum flux is 0.5 g h*^2 along the normal
    assert np.all(np.abs(flux[1:, faces]).sum(axis=0) > 0)


def test_dry_reference_line_with_discharge_rejects():
    """A requested line below every inlet face's bed has no wet reference area:
    the section has no root and the trial is rejected (nonzero status)."""
    case = S.stage_discharge_channel(reference_stage=-50.0)
    o = Oracle(case, threads=1)
    st, *_ = exterior(o, case["q"])
    assert st != 0


def section(case):
    m = case["mesh"]
    faces = np.asarray(m.boundary_faces)[m.boundary_offset[0]:m.boundary_offset[1]]
    return faces, case["exterior_bed"][faces], m.length[faces]


@pytest.mark.parametrize("discharge", [8.0, 20.0, 60.0])
def test_critical_line_is_critical(discharge):
    """inlet.critical_discharge: the reference line has Froude one for the
    section (Q^2 W / (g A^3) = 1 over the wet faces of the exterior beds)."""
    case = S.critical_inlet_channel(discharge=discharge)
    o = Oracle(case, threads=1)
    st, *_ = exterior(o, S.perturbed_state(case, 12, 0.2, 0.4, 0.0))
    assert st == 0
    eta = o.forcing[1, 0]
    _, bed, length = section(case)
    h = eta - bed
    wet = h > case["controls"]["dry"]
    area, width = (h[wet] * length[wet]).sum(), length[wet].sum()
    g = case["controls"]["grav"]
    assert abs(discharge ** 2 * width / (g * area ** 3) - 1.0) <= 1e-9


@pytest.mark.parametrize("discharge", [8.0, 20.0, 60.0])
def test_normal_line_carries_the_discharge(discharge):
    """inlet.normal_discharge: uniform flow at the reference line,
    A sqrt(A S / sum(P_i / C^2)) with Manning C = R^(1/6) / n at the section
    radius R = A / P and wetted steps to the neighbouring faces, equals Q."""
    slope = 2e-3
    case = S.normal_inlet_channel(discharge=discharge, energy_slope=slope)
    o = Oracle(case, threads=1)
    st, *_ = exterior(o, S.perturbed_state(case, 12, 0.2, 0.4, 0.0))
    assert st == 0
    eta = o.forcing[1, 0]
    from braids_hkt_gb300.mesh import section_neighbours
    faces, bed, length = section(case)
    left, right = section_neighbours(case["mesh"], 0)
    ext = case["exterior_bed"]
    dry = case["controls"]["dry"]
    depth = lambda f: 0.0 if f < 0 or eta - ext[f] <= dry else max(eta - ext[f], 0.0)
    area = perimeter = 0.0
    per = []
    for f, z, ln in zip(faces, bed, length):
        h = eta - z
        p = ln + max(h - depth(left[f]), 0.0) + max(h - depth(right[f]), 0.0) if h > dry else 0.0
        per.append(p)
        if h > dry:
            area += h * ln
            perimeter += p
    n = case["controls"]["roughness_value"]
    chezy = (area / perimeter) ** (1.0 / 6.0) / n
    rate = area * np.sqrt(area * slope / (sum(per) / chezy ** 2))
    assert abs(rate / discharge - 1.0) <= 1e-9


def test_section_neighbours_follow_the_reference_rules():
    """NormalSection's adjacency (river_exterior_normal.py:11-27): faces of a
    straight section sorted by station, neighbours where the facing ends
    meet; a section that is not one straight, consistently oriented line is
    refused."""
    from braids_hkt_gb300.mesh import section_neighbours
    case = S.normal_inlet_channel()
    m = case["mesh"]
    left, right = section_neighbours(m, 0)
    ids = np.flatnonzero((m.neighbour < 0) & (m.bid == 0))
    assert np.sum(left[ids] < 0) == 1 and np.sum(right[ids] < 0) == 1      # one bank at each end
    for f in ids:
        if right[f] >= 0:
            assert left[right[f]] == f
    bent = S.normal_inlet_channel()
    mb = bent["mesh"]
    g = np.flatnonzero((mb.neighbour < 0) & (mb.bid == 0))[0]
    mb.normal = mb.normal.copy()
    mb.normal[:, g] = [np.sqrt(0.5), np.sqrt(0.5)]
    with pytest.raises(ValueError):
        section_neighbours(mb, 0)


def test_inlet_line_host_validation():
    from braids_hkt_gb300.solver import inlet_lines
    case = S.normal_inlet_channel()
    case["inlet"] = {0: {"line": "normal", "energy_slope": 0.0}}
    with pytest.raises(ValueError):
        inlet_lines([case])
    case = S.small_channel()
    case["inlet"] = {1: {"line": "critical"}}                  # segment 1 is a stage outlet
    with pytest.raises(ValueError):
        inlet_lines([case])
