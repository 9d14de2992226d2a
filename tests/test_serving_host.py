"""Serving engine host logic on the CPU with a stand-in solver: admission
against the memory budget, cohort formation, interval splitting, completion
order and accounting."""
import numpy as np

import braids_hkt_gb300.solver as solver_mod
from braids_hkt_gb300 import serving


class FakeMesh:
    def __init__(self, nc):
        self.nc = nc


class FakeSolver:
    """Each interval finishes on the second poll; dt seconds cost 10 substeps per second."""
    live = 0
    peak = 0
    BYTES_PER_CELL = 1000

    def __init__(self, cases, precision="mixed"):
        self.cases = cases
        self.packed = {"cell_offset": np.cumsum([0] + [c["mesh"].nc for c in cases])}
        self.rotors = None
        self.state_ = [np.full((3, c["mesh"].nc), float(c["tag"])) for c in cases]
        self.polls = 0
        FakeSolver.live += 1
        FakeSolver.peak = max(FakeSolver.peak, FakeSolver.live)

    def device_bytes(self):
        return self.BYTES_PER_CELL * int(self.packed["cell_offset"][-1])

    def advance_start(self, dt, time):
        self.dt = np.asarray(dt, dtype=float)
        self.polls = 0

    def advance_poll(self):
        self.polls += 1
        if self.polls < 2:
            return None
        return [dict(hydraulic_substeps=int(round(10 * d)), failed=0) for d in self.dt]

    def state(self, i):
        return self.state_[i]

    def close(self):
        FakeSolver.live -= 1


def make_requests(sizes, durations, arrivals):
    return [serving.Request(rid=k, case={"mesh": FakeMesh(n), "tag": k}, duration=d, arrival=a)
            for k, (n, d, a) in enumerate(zip(sizes, durations, arrivals))]


def test_admission_respects_budget(monkeypatch):
    monkeypatch.setattr(solver_mod, "RiverSolver", FakeSolver)
    FakeSolver.live = FakeSolver.peak = 0
    # budget for 25k cells at 1000 B/cell; requests of 10k cells: at most two in flight at once
    eng = serving.ServingEngine(budget_bytes=25_000 * 1000, interval=1.0, max_cohort_cells=10_000)
    eng.bytes_per_cell = 1000.0
    reqs = make_requests([10_000] * 5, [2.0, 1.0, 3.0, 1.0, 2.0], [0.0] * 5)
    done = eng.run(reqs, idle_sleep=0.0)
    assert sorted(r.rid for r in done) == [0, 1, 2, 3, 4]
    assert FakeSolver.peak <= 2
    assert eng.peak_bytes <= eng.budget
    for r in done:
        assert r.substeps == int(10 * r.duration)            # intervals split exactly to the duration
        assert np.all(r.state == r.rid)                      # each request gets its own scenario's state
        assert r.latency is not None and r.latency >= 0
    assert eng.cell_updates == sum(10 * r.duration * 10_000 for r in done)


def test_cohorts_batch_queued_requests(monkeypatch):
    monkeypatch.setattr(solver_mod, "RiverSolver", FakeSolver)
    FakeSolver.live = FakeSolver.peak = 0
    eng = serving.ServingEngine(budget_bytes=1e12, interval=0.5, max_cohort_cells=25_000, max_cohort=64)
    eng.bytes_per_cell = 1000.0
    reqs = make_requests([10_000, 10_000, 10_000, 4_000], [1.0, 0.5, 1.5, 0.5], [0.0, 0.0, 0.0, 0.0])
    done = eng.run(reqs, idle_sleep=0.0)
    assert len(done) == 4
    # 25k-cell cap: the first cohort takes two 10k requests, the next the remaining two
    assert FakeSolver.peak == 2
    rep = eng.report()
    assert rep["requests"] == 4 and rep["failed"] == 0 and rep["latency_s"]["p99"] >= rep["latency_s"]["p50"]


def test_poisson_arrivals():
    t = serving.poisson_arrivals(20.0, 50.0, seed=1)
    assert np.all(np.diff(t) > 0) and t[-1] < 50.0
    assert abs(len(t) / 50.0 - 20.0) < 3.0


def test_head_request_starts_when_idle(monkeypatch):
    """An estimate above the whole budget (an over-calibrated bytes-per-cell)
    must not stall the queue: with nothing in flight the head request starts."""
    monkeypatch.setattr(solver_mod, "RiverSolver", FakeSolver)
    FakeSolver.live = FakeSolver.peak = 0
    eng = serving.ServingEngine(budget_bytes=15_000 * 1000, interval=1.0)
    eng.bytes_per_cell = 5000.0            # 10k cells -> 50 MB estimate against a 15 MB budget
    reqs = make_requests([10_000, 10_000], [1.0, 1.0], [0.0, 0.0])
    done = eng.run(reqs, idle_sleep=0.0, max_wall=30.0)
    assert len(done) == 2 and FakeSolver.peak == 1


def test_wall_guard(monkeypatch):
    monkeypatch.setattr(solver_mod, "RiverSolver", FakeSolver)

    class Never(FakeSolver):
        def advance_poll(self):
            return None
    monkeypatch.setattr(solver_mod, "RiverSolver", Never)
    eng = serving.ServingEngine(budget_bytes=1e12, interval=1.0)
    import pytest
    with pytest.raises(TimeoutError):
        eng.run(make_requests([100], [1.0], [0.0]), idle_sleep=1e-3, max_wall=0.2)
