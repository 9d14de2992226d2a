"""brx_rate_noalloc: the allocation-free residual against brx_rate.

The entry point exists for callers that may not allocate device memory once
running (fixed device-memory budgets handed out at start-up, real-time loops
where an allocation would synchronise the device). This test allocates the
caller-side buffers with torch, as such a caller would have done at start-up,
then calls the entry point through the C ABI twice in a row: both calls must
reproduce brx_rate bit for bit (the tolerance the closed-domain residual
tests use), which also shows that the shared static scratch carries nothing
from one call into the next. This file is named so that pytest collects it
last.
"""
import ctypes as C

import numpy as np
import pytest

import braids_hkt_gb300.scenarios as S

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _setup(torch):
    import braids_hkt_gb300._lib as L
    lib = L.load()
    case = S.lake_at_rest(seed=17)
    q = S.perturbed_state(case, 23, 0.5, 0.6, 0.1)
    m = case["mesh"]
    r = m.records
    i32, f64 = np.int32, np.float64
    bufs = {k: _dev(torch, v, i32) for k, v in
            dict(owner=m.owner, neighbour=m.neighbour, offset=m.offset, faces=m.faces, signs=m.signs).items()}
    bufs.update({k: _dev(torch, v, f64) for k, v in
                 dict(normal=m.normal, length=m.length, area=m.area, ls_matrix=r["ls_matrix"],
                      ls_weight=r["ls_weight"], ls_delta=r["ls_delta"], disp=r["disp"], disp_len=r["disp_len"],
                      distance=r["distance"], q=q, z=case["z"]).items()})
    return lib, case, q, bufs


def _call(lib, case, bufs, dt, rate, water):
    m = case["mesh"]
    ctl = case["controls"]
    p = lambda t: C.c_void_p(t.data_ptr())
    status = C.c_uint(99)
    freq = C.c_double(-1.0)
    rc = lib.brx_rate_noalloc(m.nc, m.nf, m.nadj, p(bufs["owner"]), p(bufs["neighbour"]), p(bufs["offset"]),
                              p(bufs["faces"]), p(bufs["signs"]), p(bufs["normal"]), p(bufs["length"]),
                              p(bufs["area"]), p(bufs["ls_matrix"]), p(bufs["ls_weight"]), p(bufs["ls_delta"]),
                              p(bufs["disp"]), p(bufs["disp_len"]), p(bufs["distance"]), p(bufs["q"]),
                              p(bufs["z"]), ctl["grav"], ctl["dry"], ctl["cfl"], dt, p(rate), p(water),
                              C.byref(status), C.byref(freq), None)
    return rc, status.value, freq.value


def test_noalloc_rate_matches_rate_twice():
    import torch
    from braids_hkt_gb300.solver import RiverSolver
    lib, case, q, bufs = _setup(torch)
    m = case["mesh"]
    dt = 0.01
    ref = RiverSolver(case)
    ref.set_state(q)
    rate_ref, water_ref, status_ref, freq_ref = ref.rate(dt, 0.0)
    torch.cuda.synchronize()
    for call in range(2):
        rate = torch.full((3, m.nc), np.nan, dtype=torch.float64, device="cuda")
        water = torch.full((m.nf,), np.nan, dtype=torch.float64, device="cuda")
        rc, status, freq = _call(lib, case, bufs, dt, rate, water)
        assert rc == 0, lib.brx_last_error()
        assert status == status_ref
        assert freq == freq_ref
        np.testing.assert_array_equal(rate.cpu().numpy(), rate_ref.cpu().numpy())
        np.testing.assert_array_equal(water.cpu().numpy(), water_ref.cpu().numpy())


def test_noalloc_rejected_topology_writes_nothing():
    """A face index out of range in the caller's incidence is caught by the
    entry point's device-side topology check before any kernel indexes with
    it: the call returns BRX_ERR_ARGUMENT with the spatial status bit and
    leaves rate and water as they were, although the shared scratch still
    holds the previous call's fluxes. A valid call afterwards is exact again."""
    import torch
    lib, case, q, bufs = _setup(torch)
    m = case["mesh"]
    dt = 0.01
    rate = torch.full((3, m.nc), np.nan, dtype=torch.float64, device="cuda")
    water = torch.full((m.nf,), np.nan, dtype=torch.float64, device="cuda")
    rc, _, _ = _call(lib, case, bufs, dt, rate, water)          # fills the scratch with valid fluxes
    assert rc == 0, lib.brx_last_error()
    good_rate, good_water = rate.clone(), water.clone()
    faces = bufs["faces"].clone()
    bufs["faces"][m.nadj // 2] = m.nf + 5                       # out of range: checked on the device
    rate.fill_(7.0)
    water.fill_(7.0)
    rc, status, _ = _call(lib, case, bufs, dt, rate, water)
    assert rc == 1 and b"topology" in lib.brx_last_error()
    assert status & 1
    assert bool((rate == 7.0).all()) and bool((water == 7.0).all())
    bufs["faces"] = faces
    rc, _, _ = _call(lib, case, bufs, dt, rate, water)
    assert rc == 0, lib.brx_last_error()
    assert torch.equal(rate, good_rate) and torch.equal(water, good_water)


def test_noalloc_rejects_oversize_mesh():
    import braids_hkt_gb300._lib as L
    lib = L.load()
    rc = lib.brx_rate_noalloc(20000, 40000, 60000, *([None] * 16), 9.81, 1e-6, 0.9, 0.01, None, None, None,
                              None, None)
    assert rc == 5 and b"at most 16384 cells" in lib.brx_last_error()
