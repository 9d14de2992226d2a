"""Serving loop: continuous batching of river scenario solves on one GPU.

Requests (a scenario case, a simulated duration) arrive over time. The engine
keeps a FIFO queue and a set of in-flight cohorts:

  * Admission. As long as the head of the queue fits the free part of the HBM
    budget, the engine takes as many queued requests as fit (and at most a
    cohort cap of cells / requests) and builds one batched RiverSolver for
    them - the cohort - in a builder thread, on its own CUDA stream. Device
    bytes are estimated per cell before the build (calibrated on the exact
    footprint of every solver built so far) and charged exactly after it.
  * Overlap. Every cohort advances interval by interval through the
    asynchronous brx_advance_start / brx_advance_poll pair, so cohorts
    admitted at different times run concurrently on the device, and requests
    that arrive while others are running start as soon as memory frees up.
  * Completion. A request leaves its cohort when its simulated time is
    reached: its scenario goes idle, its final state and rotor record are
    copied out and its latency (arrival to result) recorded. A cohort whose
    requests are all done frees its memory, which admits the next cohort.

State stays device-resident between intervals; only a finished request's
state crosses to the host. A request's result is bitwise the same whether it
ran alone or in any cohort (scenarios in a batch share no arithmetic), which
tests/test_serving.py checks.
"""
from __future__ import annotations

import queue as _queue
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

DEFAULT_BYTES_PER_CELL = 2048.0     # before the first solver calibrates it


@dataclass
class Request:
    rid: int
    case: dict
    duration: float                  # simulated seconds
    arrival: float = 0.0             # engine clock [s]
    admitted: float | None = None
    finished: float | None = None
    state: np.ndarray | None = None  # (3, nc) at the end
    rotors: np.ndarray | None = None
    failed: int = 0
    substeps: int = 0
    base: int = 0                    # pool mesh of a slot-serving request

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


@dataclass
class _Cohort:
    solver: object
    requests: list
    bytes: int
    t: np.ndarray = field(default=None)
    running: bool = False


class ServingEngine:
    def __init__(self, budget_bytes=150e9, precision="mixed", interval=5.0, max_cohort_cells=4_000_000,
                 max_cohort=64, clock=time.perf_counter):
        self.budget = float(budget_bytes)
        self.precision = precision
        self.interval = float(interval)
        self.max_cells = int(max_cohort_cells)
        self.max_requests = int(max_cohort)
        self.clock = clock
        self.t0 = None
        self.queue = deque()
        self.cohorts = []
        self.done = []
        self.in_use = 0.0            # charged bytes (estimates while building, exact after)
        self.live_bytes = 0          # exact device bytes of the running cohorts
        self.peak_bytes = 0
        self.bytes_per_cell = None
        self.cell_updates = 0
        self._built = _queue.Queue()
        self._building = 0

    # ------------------------------------------------------------------
    def now(self):
        return self.clock() - self.t0

    def submit(self, req):
        if self.t0 is None:
            self.t0 = self.clock()
        self.queue.append(req)

    def estimate(self, req):
        return req.case["mesh"].nc * (self.bytes_per_cell or DEFAULT_BYTES_PER_CELL)

    def _admit(self):
        while self.queue:
            pick, est, cells = [], 0.0, 0
            idle = not self.cohorts and not self._building
            for req in self.queue:
                e, n = self.estimate(req), req.case["mesh"].nc
                if pick and (cells + n > self.max_cells or len(pick) >= self.max_requests):
                    break
                # with nothing in flight the head request always starts (an
                # estimate above the free budget could otherwise wait forever)
                if self.in_use + est + e > self.budget and not (idle and not pick):
                    break
                pick.append(req)
                est += e
                cells += n
            if not pick:
                return
            for _ in pick:
                self.queue.popleft()
            self.in_use += est
            now = self.now()
            for r in pick:
                r.admitted = now
            self._building += 1
            threading.Thread(target=self._build, args=(pick, est), daemon=True).start()

    def _build(self, pick, est):
        from .solver import RiverSolver
        try:
            solver = RiverSolver([r.case for r in pick], precision=self.precision)
            self._built.put((pick, est, solver, None))
        except Exception as exc:                     # reported on the engine thread
            self._built.put((pick, est, None, exc))

    def _collect_built(self):
        while True:
            try:
                pick, est, solver, exc = self._built.get_nowait()
            except _queue.Empty:
                return
            self._building -= 1
            if exc is not None:
                raise exc
            exact = solver.device_bytes()
            cells = sum(r.case["mesh"].nc for r in pick)
            self.bytes_per_cell = max(self.bytes_per_cell or 0.0, exact / cells)
            self.in_use += exact - est
            self.live_bytes += exact
            self.peak_bytes = max(self.peak_bytes, self.live_bytes)
            c = _Cohort(solver, pick, exact, np.zeros(len(pick)))
            self.cohorts.append(c)
            self._start(c)

    def _start(self, c):
        left = np.array([r.duration for r in c.requests]) - c.t
        dt = np.where(left > 1e-12, np.minimum(self.interval, left), 0.0)
        c.solver.advance_start(dt, c.t)
        c._dt = dt
        c.running = True

    def _poll(self):
        still = []
        for c in self.cohorts:
            diags = c.solver.advance_poll()
            if diags is None:
                still.append(c)
                continue
            off = c.solver.packed["cell_offset"]
            finished = []
            for i, (r, d) in enumerate(zip(c.requests, diags)):
                if c._dt[i] <= 0:
                    continue
                r.substeps += d["hydraulic_substeps"]
                self.cell_updates += d["hydraulic_substeps"] * int(off[i + 1] - off[i])
                if d["failed"]:
                    r.failed = d["failed"]
                    c.t[i] = r.duration
                else:
                    c.t[i] += c._dt[i]
                if c.t[i] >= r.duration - 1e-9 * max(1.0, r.duration):
                    finished.append(i)
            if finished:
                rec = c.solver.turbine_record() if c.solver.rotors is not None else None
                now = self.now()
                for i in finished:
                    r = c.requests[i]
                    r.state = c.solver.state(i).copy()
                    if rec is not None:
                        rows = np.flatnonzero(c.solver.rotors["scenario"] == i)
                        r.rotors = rec[rows].copy()
                    r.finished = now
                    self.done.append(r)
            if all(c.t[i] >= r.duration - 1e-9 * max(1.0, r.duration) for i, r in enumerate(c.requests)):
                self.in_use -= c.bytes
                self.live_bytes -= c.bytes
                c.solver.close()
                continue
            self._start(c)
            still.append(c)
        self.cohorts = still

    def busy(self):
        return bool(self.queue or self.cohorts or self._building)

    def pump(self):
        """One pass: collect built cohorts, poll the running ones, admit from the queue."""
        self._collect_built()
        self._poll()
        self._admit()

    def run(self, arrivals, idle_sleep=2e-4, max_wall=None):
        """Serve a list of requests whose ``arrival`` is an engine-clock time;
        returns the finished requests. ``max_wall`` bounds the loop in wall
        seconds (TimeoutError), for callers that must not wait unboundedly."""
        pending = sorted(arrivals, key=lambda r: r.arrival)
        self.t0 = self.clock()
        k = 0
        while k < len(pending) or self.busy():
            now = self.now()
            if max_wall is not None and now > max_wall:
                raise TimeoutError(f"serving loop exceeded {max_wall} s with {len(self.queue)} queued, "
                                   f"{len(self.cohorts)} running, {self._building} building")
            while k < len(pending) and pending[k].arrival <= now:
                self.queue.append(pending[k])
                k += 1
            before = (len(self.done), len(self.cohorts), self._building)
            self.pump()
            if (len(self.done), len(self.cohorts), self._building) == before:
                time.sleep(idle_sleep)
        return self.done

    def report(self):
        lat = np.array([r.latency for r in self.done if r.latency is not None])
        wall = max((r.finished for r in self.done), default=0.0)
        return {"requests": len(self.done), "failed": sum(1 for r in self.done if r.failed),
                "latency_s": {"p50": float(np.percentile(lat, 50)) if len(lat) else None,
                              "p99": float(np.percentile(lat, 99)) if len(lat) else None,
                              "max": float(lat.max()) if len(lat) else None},
                "throughput_cell_updates_s": self.cell_updates / wall if wall > 0 else None,
                "wall_s": wall, "peak_bytes": self.peak_bytes, "budget_bytes": self.budget,
                "bytes_per_cell": self.bytes_per_cell}


class SlotServingEngine:
    """Continuous batching over one resident batch of scenario slots.

    The engine builds one RiverSolver once: ``copies`` slots of every mesh in
    the pool (a prepared scenario mesh with its rotor layout), as many copies
    as the HBM budget holds. A request names a pool mesh, its own discharge
    (in its case's forcing) and a simulated duration. Between two intervals
    of the batch, queued requests take free slots of their mesh (first fit,
    any queue position): the slot's state, forcing and step hint are loaded
    (RiverSolver.load_scenario) and the slot joins the next interval; a slot
    whose request is done goes idle (dt 0: the device active set skips it at
    no cost) and is free for the next request. So requests that arrive while
    others run join the resident batch within one interval, nothing is
    rebuilt, and state stays on the device until a request finishes.
    """

    def __init__(self, pool, precision="mixed", interval=0.5, budget_bytes=150e9, copies=None, max_copies=4,
                 clock=time.perf_counter):
        from .solver import RiverSolver
        self.pool = list(pool)
        self.precision = precision
        self.interval = float(interval)
        self.budget = float(budget_bytes)
        self.clock = clock
        if copies is None:
            # device bytes per cell from the smallest pool mesh, 10% margin
            small = min(self.pool, key=lambda c: c["mesh"].nc)
            probe = RiverSolver(small, precision=precision)
            per_cell = 1.1 * probe.device_bytes() / small["mesh"].nc
            probe.close()
            per_copy = per_cell * sum(c["mesh"].nc for c in self.pool)
            copies = int(max(1, min(max_copies, self.budget // max(per_copy, 1.0))))
        self.copies = int(copies)
        self.slot_mesh = [i for i in range(len(self.pool)) for _ in range(self.copies)]
        self.solver = RiverSolver([self.pool[i] for i in self.slot_mesh], precision=precision)
        self.bytes = self.solver.device_bytes()
        if self.bytes > self.budget:
            self.solver.close()
            raise MemoryError(f"{self.copies} copies of the pool take {self.bytes} B, above the budget")
        n = len(self.slot_mesh)
        self.free = {i: deque(k for k in range(n) if self.slot_mesh[k] == i) for i in range(len(self.pool))}
        self.req = [None] * n
        self.t = np.zeros(n)
        self.queue = deque()
        self.done = []
        self.cell_updates = 0
        self.running = False
        self.t0 = None
        self.trace = []                  # (engine time, queued, running requests) per interval
        off = self.solver.packed["cell_offset"]
        self.cells = np.diff(off).astype(np.int64)

    def now(self):
        return self.clock() - self.t0

    def _admit(self):
        left = deque()
        now = self.now()
        while self.queue:
            r = self.queue.popleft()
            slots = self.free[r.base]
            if not slots:
                left.append(r)
                continue
            k = slots.popleft()
            self.solver.load_scenario(k, r.case["q"], r.case.get("forcing"))
            self.req[k] = r
            self.t[k] = 0.0
            r.admitted = now
        self.queue = left

    def _start(self):
        dt = np.zeros(len(self.req))
        for k, r in enumerate(self.req):
            if r is not None:
                dt[k] = min(self.interval, r.duration - self.t[k])
        if not (dt > 0).any():
            return False
        self._dt = dt
        self.solver.advance_start(dt, self.t)
        self.running = True
        self.trace.append((self.now(), len(self.queue), int((dt > 0).sum())))
        return True

    def _finish(self, diags):
        self.running = False
        finished = []
        for k, (r, d) in enumerate(zip(self.req, diags)):
            if r is None or self._dt[k] <= 0:
                continue
            r.substeps += d["hydraulic_substeps"]
            self.cell_updates += d["hydraulic_substeps"] * int(self.cells[k])
            if d["failed"]:
                r.failed = d["failed"]
                self.t[k] = r.duration
            else:
                self.t[k] += self._dt[k]
            if self.t[k] >= r.duration - 1e-9 * max(1.0, r.duration):
                finished.append(k)
        if finished:
            rec = self.solver.turbine_record() if self.solver.rotors is not None else None
            now = self.now()
            for k in finished:
                r = self.req[k]
                r.state = self.solver.state(k).copy()
                if rec is not None:
                    r.rotors = rec[np.flatnonzero(self.solver.rotors["scenario"] == k)].copy()
                r.finished = now
                self.done.append(r)
                self.req[k] = None
                self.free[self.slot_mesh[k]].append(k)

    def run(self, arrivals, idle_sleep=2e-4, max_wall=None):
        """Serve requests (each with ``base``, the pool index of its mesh) whose
        ``arrival`` is an engine-clock time; returns the finished requests."""
        pending = sorted(arrivals, key=lambda r: r.arrival)
        self.t0 = self.clock()
        k = 0
        while k < len(pending) or self.queue or self.running or any(r is not None for r in self.req):
            now = self.now()
            if max_wall is not None and now > max_wall:
                raise TimeoutError(f"serving loop exceeded {max_wall} s with {len(self.queue)} queued")
            while k < len(pending) and pending[k].arrival <= now:
                self.queue.append(pending[k])
                k += 1
            if self.running:
                diags = self.solver.advance_poll()
                if diags is None:
                    time.sleep(idle_sleep)
                    continue
                self._finish(diags if isinstance(diags, list) else [diags])
            self._admit()
            if not self._start():
                time.sleep(idle_sleep)
        return self.done

    def report(self):
        lat = np.array([r.latency for r in self.done if r.latency is not None])
        wait = np.array([r.admitted - r.arrival for r in self.done if r.admitted is not None])
        wall = max((r.finished for r in self.done), default=0.0)
        q = np.array([x[1] for x in self.trace]) if self.trace else np.zeros(1)
        act = np.array([x[2] for x in self.trace]) if self.trace else np.zeros(1)
        return {"requests": len(self.done), "failed": sum(1 for r in self.done if r.failed),
                "latency_s": {"p50": float(np.percentile(lat, 50)) if len(lat) else None,
                              "p99": float(np.percentile(lat, 99)) if len(lat) else None,
                              "max": float(lat.max()) if len(lat) else None},
                "admission_wait_s": {"p50": float(np.percentile(wait, 50)) if len(wait) else None,
                                     "p99": float(np.percentile(wait, 99)) if len(wait) else None},
                "queue_length": {"mean": float(q.mean()), "max": int(q.max()),
                                 "by_decile": [int(x) for x in q[np.linspace(0, len(q) - 1, 10).astype(int)]]},
                "running_requests": {"mean": float(act.mean()), "max": int(act.max())},
                "throughput_cell_updates_s": self.cell_updates / wall if wall > 0 else None,
                "wall_s": wall, "intervals": len(self.trace), "slots": len(self.req), "copies": self.copies,
                "resident_bytes": self.bytes, "budget_bytes": self.budget}

    def close(self):
        self.solver.close()


def poisson_arrivals(rate, window, seed):
    """Arrival times of a Poisson process of the given rate over [0, window)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= window:
            return out
        out.append(t)


def request_case(base, discharge):
    """A request on a prepared scenario mesh with its own discharge (uniform-flow start)."""
    case = dict(base)
    case["forcing"] = np.array(base["forcing"], dtype=float).copy()
    case["forcing"][0, 0] = discharge
    q = np.array(base["q"], dtype=float).copy()
    width = float(np.ptp(base["mesh"].points[:, 1]))
    q[1] = np.where(q[0] > 0.0, discharge / width, 0.0)
    q[2] = 0.0
    case["q"] = q
    return case
