"""Benchmark of the GB300 river solver step (one JSON line on rank 0).

Metric: cell-updates/s, one cell-update = one cell advanced by one accepted
SSPRK(2,2) substep (two spatial evaluations). A bench "step" is one outer
interval ``brx_advance(dt_outer)`` of the whole workload: the adaptive
substep loop over every scenario, resident in HBM.

  python bench.py [--gpus N --steps K --warmup W] [--workload config1|config4] [--impl ours|reference]

--impl reference times the reference's own CPU arithmetic of the path (the
oracle port of its kernels, OpenMP on every host core; the reference's
compiled kernels cannot be rebuilt where the reference checkout is absent)
on the same workload and metric. For N > 1, scenarios are independent and
shard across ranks with no collective on the data path ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "cell-updates/s"
BYTES_PER_CELL_UPDATE = {"fp64": 680.0, "mixed": 384.0}   # algorithmic bytes, two-sweep design
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per cell of one
# launch of each mixed-form sweep, each kernel captured alone (ncu --set full,
# one launch) on the 24-scenario subset with rotors (scenarios 20..43 sorted
# by size, 1,967,962 cells, inputs larger than L2): a launch of the full batch
# is scaled by its cells
TRAFFIC_BYTES_PER_CELL = {"mixed": {"cells": 244.21, "faces": 213.25, "gather": 145.97, "update": 190.15,
                                    "drag": 63.07}}
KERNEL_NAMES = ["drag", "boundary", "cells", "faces", "gather", "update", "control"]
# FP64 flops (2 DFMA + DMUL + DADD thread instructions) per cell (per face for
# the face sweep) of one launch of each FP64-form sweep, each kernel captured
# alone on config 1 (ncu, one launch from the initial state), and their sum
# over one substep per cell-update
FP64_FLOPS = {"cells": ("cell", 995.0), "faces": ("face", 1190.0), "gather": ("cell", 97.0),
              "update": ("cell", 89.0), "drag": ("cell", 259.0)}
FP64_FLOPS_PER_CELL_UPDATE = 6220.0


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def aggregate(seconds, updates, dist=None, device="cpu"):
    """Whole-job figures over ranks: the slowest rank's timed seconds and the
    sum of every rank's cell-updates (each rank advances its own scenarios,
    no exchange on the data path)."""
    if dist is None:
        return seconds, updates
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(updates)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), int(u.item())


def build_workload(name, rank=0, world=1, subset=None):
    """(cases, precision, outer dt [s], config dict). Built before CUDA starts (spawn pool)."""
    import braids_hkt_gb300.scenarios as S
    if name == "config1":
        return [S.config1()], "fp64", 1.0, dict(workload="config1: straight channel 2000x200 m, 4 m jittered "
                                               "Delaunay, 50k triangles, Q=400 m3/s, stage 3.0 m, Manning 0.03, "
                                               "CFL 0.9, FP64 plain form")
    if name == "config2":
        return [S.config2()], "fp64", 0.5, dict(workload="config2: the config-1 channel with 3 tandem rotors 150 m "
                                               "apart (D 5 m, Ct 0.8, incident-speed power curve rated 500 kW), "
                                               "refined to 1 m across the channel downstream of each rotor "
                                               "(124k triangles), FP64 plain form")
    if name == "config3":
        return [S.config3()], "mixed", 1.0, dict(workload="config3: braided river 10 km x 1.5 km, 5 seeded sinuous "
                                                "channels, 3.87 m jittered Delaunay (about 2M triangles), "
                                                "hydrograph 200 -> 2000 m3/s over 3600 s, stage outlet, MPM bed "
                                                "update (d50 20 mm, porosity 0.4) after every interval, 12 "
                                                "rotors, mixed FP32/FP64 form; the FP64 form over the same "
                                                "intervals for the error")
    if name == "config4":
        params = S.config4_params(64, seed=4 + rank)
        if subset:
            a, b = (int(v) for v in subset.split(":"))
            params = sorted(params, key=lambda p: p["cells"])[a:b]
        workers = max(1, (os.cpu_count() or 1) // max(world, 1))
        cases = S.build_cases(params, workers)
        rotors = sum(len(c.get("turbines", [])) for c in cases)
        return cases, "mixed", 0.5, dict(
            workload="config4: 64 channel scenarios in one batch, cells logU(1e4,5e5), width U(100,400) m, "
                     "Q U(100,1500) m3/s, length 10 widths, jittered Delaunay, Manning 0.03, CFL 0.9, "
                     "0-8 rotors each (D 5 m, Ct 0.8, rated 500 kW incident-speed curves, >= 5 D apart, "
                     "1.5 m refined footprints), mixed FP32/FP64 form",
            scenarios=len(cases), rotors=rotors)
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(torch, buf):
    buf.fill_(1.0)            # 256 MiB write evicts the 129 MB L2


def algorithmic_bytes(kernel, nc, nf, nadj, nslot, precision="fp64", rotor_cells=0, rotor_faces=0):
    """Compulsory unique bytes one launch of each kernel reads and writes.

    Every array a kernel touches counts once per element (neighbour gathers
    that re-read a cell already counted are free), for the layout of the given
    arithmetic form. rotor_cells / rotor_faces: cells and faces of scenarios
    with rotor arrays, whose face terms the mixed face sweep forms in its tail.
    """
    i4, d8 = 4, 8
    if precision == "mixed":
        if kernel == "cells":    # state, bed, id, CSR, LS inverse, record out; per entry: index, geometry, weight;
            # rotor tail: wet gradients out (6 floats) per cell, flow-metric offsets per entry
            return (nc * (3 * d8 + d8 + i4 + i4 + 16 + 64) + nadj * (8 + 16 + 4) +
                    rotor_cells * (6 * 4 + 3 * 8))
        if kernel == "faces":    # two records (each cell once), face ids/geometry, water/speed + 4 momentum out;
            # rotor tail: two wet-gradient components and the support mask per cell, midpoint
            # displacements in and the pressure correction out per face (rotor_cells x 3 CSR entries
            # in the cell sweep above: triangles)
            return (nc * 64 + nf * (2 * i4 + i4 + i4 + 8 + 16 + 8) + nf * (8 + 16) +
                    rotor_cells * (2 * 4 + 1) + rotor_faces * (16 + 8))
        if kernel == "gather":   # id, CSR, record flags, stock, rate/theta out; per entry weight; face fluxes
            return nc * (i4 + i4 + 4 + d8 + 3 * d8 + d8 + i4) + nadj * (i4 + d8) + nf * (8 + 16)
        if kernel == "update":    # id, CSR, rate, stage states in/out, primitives out, donor factors; per
            # entry face id, FP64 and FP32 weights, other cell + flags; per face the FP32 water
            return nc * (i4 + i4 + 2 * 4 + 3 * d8 + 3 * d8 + d8 + 32 + 4) + nadj * (i4 + d8 + 4 + 8) + nf * 8
        if kernel == "drag":
            return nc * (i4 + 6 * d8)
        return 0
    if kernel == "faces":
        return nf * (2 * i4 + 2 * d8 + 4 * d8 + 2 * d8 + i4 + i4) + nc * 128 + nf * (16 + 32)
    if kernel == "cells":
        return (nc * (3 * d8 + d8 + i4 + i4 + 4 * d8 + 128) + nadj * (2 * i4 + 3 * d8) +
                nf * (3 * i4 + 2 * d8 + 2 * 2 * d8 + 2 * 2 * d8 + 2 * d8) + 3 * nc * d8)
    if kernel == "gather":
        return nc * (i4 + d8 + 128 // 8 + 3 * d8 + d8 + i4 + i4) + nadj * 2 * i4 + nf * (d8 + 16 + 32) + nc * 3 * d8
    if kernel == "limit":
        return nf * (16 + 2 * i4 + i4 + i4 + 32) + nc * (d8 + 3 * d8)
    if kernel == "update":
        return nc * (i4 + d8 + 3 * d8 + 3 * d8 + 3 * d8 + 3 * d8 + i4) + nadj * 2 * i4 + nf * (d8 + 32)
    if kernel == "drag":
        return nc * (i4 + 6 * d8)
    return 0


def prepare(solver, cases):
    """Forcing tables of the workload (hydrograph), before any interval."""
    if len(cases) == 1 and cases[0].get("table_time") is not None:
        solver.set_forcing_table(cases[0]["table_time"], cases[0]["table_value"])


def outer_step(solver, dt, t, raise_on_failure=False):
    """One outer interval of the owner: the adaptive hydraulic substeps, then
    the Exner bed update where the workload has a bed model
    (ShorelineSolver.step -> finish, shoreline_solver.py:345-372)."""
    diags = solver.advance(dt, t, raise_on_failure=raise_on_failure)
    if solver.bed_model is not None:
        solver.morphology(dt)
    return diags


def run_step(solver, dt, t, chain, raise_on_failure=False):
    """One bench step: `chain` outer intervals of dt, chained on the device
    when chain > 1 (brx_advance_chain; workloads without a per-interval bed
    update), else one owner interval. Returns the diagnostics of the step's
    last interval per scenario, the step's cell-updates, the failed scenarios
    and the simulated time after the step (advanced interval by interval, as
    the chain forms its start times)."""
    cells = np.diff(solver.packed["cell_offset"]).astype(np.int64)
    if chain > 1:
        rows = solver.advance_chain(dt, t, chain, raise_on_failure=raise_on_failure)
        rows = [rows] if solver.single else rows
        for _ in range(chain):
            t += dt
        updates = sum(int(r["hydraulic_substeps"]) * int(cells[i]) for i, rr in enumerate(rows) for r in rr)
        failed = {i for i, rr in enumerate(rows) if any(r["failed"] for r in rr)}
        return [rr[-1] for rr in rows], updates, failed, t
    diags = outer_step(solver, dt, t, raise_on_failure=raise_on_failure)
    diags = diags if isinstance(diags, list) else [diags]
    updates = sum(int(d["hydraulic_substeps"]) * int(cells[i]) for i, d in enumerate(diags))
    return diags, updates, {i for i, d in enumerate(diags) if d["failed"]}, t + dt


def fp64_comparison(cases, outer, steps, mixed_state, mixed_z, mixed_rotors, torch):
    """The same single-scenario workload in the FP64 form over the same
    intervals from the same initial state: its throughput and the mixed
    form's error against it after the last interval."""
    from braids_hkt_gb300.solver import RiverSolver
    import braids_hkt_gb300.turbines as TB
    case = cases[0]
    one = RiverSolver(case, precision="fp64")
    prepare(one, cases)
    t, ms, ups = 0.0, 0.0, 0
    for _ in range(steps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(one.stream)
        d = outer_step(one, outer, t)
        e1.record(one.stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
        ups += int(d["hydraulic_substeps"]) * one.nc
        t += outer
    q64 = one.q.cpu().numpy()
    h64, hmx = q64[0], mixed_state[0]
    deep = h64 > 0.05
    rel = np.abs(hmx - h64) / np.maximum(h64, 1e-3)
    area = case["mesh"].area
    out = {"fp64_value": ups / (ms / 1e3), "unit": METRIC, "after_sim_s": steps * outer,
           "depth_rel_max_deep": float(rel[deep].max()), "depth_rel_p99_deep": float(np.percentile(rel[deep], 99)),
           "depth_abs_max_over_depth_max": float(np.abs(hmx - h64).max() / h64.max()),
           "unit_discharge_rel_max": float(np.abs(mixed_state[1:] - q64[1:]).max() / max(np.abs(q64[1:]).max(), 1e-12)),
           "volume_rel": float(abs(np.sum(hmx * area) - np.sum(h64 * area)) / np.sum(h64 * area)),
           "deep": "cells deeper than 5 cm", "stated_tolerance": 1e-4}
    if one.bed_model is not None and mixed_z is not None:
        z64 = one.z.cpu().numpy()
        scale = max(float(np.abs(z64 - case["z"]).max()), 1e-12)
        out["bed_abs_max_over_bed_change_max"] = float(np.abs(mixed_z - z64).max() / scale)
    if one.rotors is not None and mixed_rotors is not None:
        col = TB.DIAG_FIELDS.index("useful_power_per_density_m5_s3")
        p64 = one.turbine_record()[:, col]
        out["rotor_power_abs_max_over_max"] = float(np.abs(mixed_rotors[:, col] - p64).max() /
                                                    max(float(np.abs(p64).max()), 1e-30))
        out["rotor_power_max_W"] = float(np.abs(p64).max() * TB.WATER_DENSITY)
    one.close()
    return out


def fp64_roofline(per_kind, nc, nf, value, peak_tflops):
    """Compute roofline of the FP64 form: the FP64 flops of the slower of the
    two FP64 sweeps over its live duration, and of the whole step at the
    measured throughput, against the measured FP64 FMA rate."""
    dom = max(("cells", "faces"), key=lambda k: sum(per_kind.get(k, [0.0])))
    unit, per = FP64_FLOPS[dom]
    flops = per * (nf if unit == "face" else nc)
    ms = float(np.mean(per_kind[dom]))
    achieved = flops / (ms * 1e-3) / 1e12
    step = value * FP64_FLOPS_PER_CELL_UPDATE / 1e12
    return {"bound": "fp64", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
            "frac": achieved / peak_tflops, "kernel_ms": ms, "flops_per_launch": flops,
            "flops_source": f"ncu FP64 thread-instruction counts per {unit} of a config-1 capture, scaled",
            "peak_source": "brx_fma_rate (measured FP64 FMA rate of this GPU)",
            "step_flops_per_cell_update": FP64_FLOPS_PER_CELL_UPDATE, "step_achieved_tflops": step,
            "step_frac": step / peak_tflops}


def fma_peaks(lib):
    """Measured FMA throughput of this GPU (brx_fma_rate): the compute
    roofline of the FP64 form and of the FP32 sweeps, TFLOP/s."""
    import ctypes as C
    out = {}
    for name, prec in (("fp64_tflops", 0), ("fp32_tflops", 1)):
        t, ms = C.c_double(0.0), C.c_double(0.0)
        if lib.brx_fma_rate(prec, C.byref(t), C.byref(ms)) == 0:
            out[name] = t.value
    return out


def serving_session(cases, precision, rate=20.0, window=60.0, duration=2.5, interval=0.5, budget=150e9, seed=5,
                    copies=2, checks=3):
    """Config 5 on one resident batch: Poisson arrivals of requests drawn from
    the config-4 scenario pool (a pool mesh with its rotor layout, their own
    discharge U(100, 1500) m3/s), each asking for ``duration`` simulated
    seconds, served by continuous batching over ``copies`` resident slots of
    every pool mesh within the HBM budget (serving.SlotServingEngine);
    latency is arrival to result on the host clock. A few finished requests
    are re-run alone in FP64 for the depth error."""
    import braids_hkt_gb300.serving as SV
    from braids_hkt_gb300.solver import RiverSolver
    rng = np.random.default_rng(seed)
    times = SV.poisson_arrivals(rate, window, seed)
    reqs = []
    for k, t in enumerate(times):
        b = int(rng.integers(len(cases)))
        reqs.append(SV.Request(rid=k, case=SV.request_case(cases[b], float(rng.uniform(100.0, 1500.0))),
                               duration=duration, arrival=t, base=b))
    eng = SV.SlotServingEngine(cases, precision=precision, interval=interval, budget_bytes=budget, copies=copies)
    try:
        done = eng.run(reqs, max_wall=window + 240.0)
    finally:
        rep = eng.report()
        eng.close()
    errs = []
    for r in sorted(done, key=lambda r: r.case["mesh"].nc)[::max(1, len(done) // checks)][:checks]:
        one = RiverSolver(r.case, precision="fp64")
        t = 0.0
        while t < r.duration - 1e-9:
            dt = min(interval, r.duration - t)
            one.advance(dt, t)
            t += dt
        h64 = one.state()[0]
        errs.append(float((np.abs(r.state[0] - h64) / np.maximum(h64, 1e-3)).max()))
        one.close()
    offered = len(times) / window * duration * float(np.mean([c["mesh"].nc for c in cases]))
    rep.update(arrival_rate_per_s=rate, arrival_window_s=window, simulated_s_per_request=duration,
               interval_s=interval, depth_rel_vs_fp64_max=max(errs) if errs else None,
               offered_cell_seconds_per_s=offered,
               note=f"config 5 on one resident batch: Poisson {rate:g}/s over {window:g} s, {duration:g} s simulated "
                    "per request (config 5 asks 600 s: that load is about a hundred times this GPU's throughput "
                    "and queues without bound), requests from the config-4 pool with their own discharge")
    return rep


def cpu_baseline(cases, outer, seconds=10.0, threads=None):
    """The oracle port on the host cores over a bounded sample of the workload."""
    from oracle import Oracle
    threads = threads or os.cpu_count() or 1
    o = Oracle(cases[0], threads=threads)
    q = cases[0]["q"].copy()
    nc = cases[0]["mesh"].nc
    updates, t0, sim = 0, time.perf_counter(), 0.0
    # short intervals on large meshes, so the sample stays near its time bound
    interval = min(outer, 0.5, 0.5 * 2.0e5 / nc)
    while time.perf_counter() - t0 < seconds:
        st, _, stats = o.advance(q, interval, sim)
        if st:
            break
        updates += stats["substeps"] * nc
        sim += interval
    el = time.perf_counter() - t0
    return {"value": updates / el, "unit": METRIC, "cores": threads, "kind": "port", "seconds": el,
            "sample": f"{cases[0].get('name', 'case')}: {sim:g} s simulated ({updates} cell-updates) "
                      f"from the initial state, oracle port with OpenMP on {threads} threads"}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cases, precision, outer, cfg = build_workload(args.workload)
    cases = sorted(cases, key=lambda c: c["mesh"].nc)[len(cases) // 2:len(cases) // 2 + 1]   # a median scenario
    cfg = dict(cfg, cpu_sample="one median-size scenario of the workload")
    threads = os.cpu_count() or 1
    per_step = []
    for _ in range(args.warmup):
        cpu_baseline(cases, outer, seconds=2.0, threads=threads)
    for _ in range(args.steps):
        per_step.append(cpu_baseline(cases, outer, seconds=max(5.0, 60.0 / max(args.steps, 1)), threads=threads))
    value = float(np.mean([p["value"] for p in per_step]))
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean([p["seconds"] for p in per_step])) * 1e3,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": per_step[-1]["sample"]},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--workload", default="config4")
    ap.add_argument("--plain", type=int, default=3, help="scenarios re-run one by one in plain FP64")
    ap.add_argument("--chain", type=int, default=1,
                    help="outer intervals per bench step, chained on the device (1: one interval per step; "
                         "the chained form is then timed as a separate leg)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the config-5 serving session")
    ap.add_argument("--serving-rate", type=float, default=20.0, help="Poisson arrivals per second")
    ap.add_argument("--serving-window", type=float, default=60.0, help="arrival window [s]")
    ap.add_argument("--serving-duration", type=float, default=2.5, help="simulated seconds per request")
    ap.add_argument("--subset", default=None,
                    help="START:STOP slice of the config-4 scenarios sorted by size (profiling a smaller case)")
    ap.add_argument("--no-hllc", dest="hllc", action="store_false",
                    help="skip the HLLC MUSCL-Hancock legs (per-scenario and whole batch, FP64 form)")
    ap.add_argument("--profile-only", type=int, default=0,
                    help="only time N substeps kernel by kernel (brx_profile_substep) and exit")
    ap.add_argument("--profile-method", default="fwave", choices=("fwave", "fwave-fp64", "hllc", "hllc-mixed"),
                    help="hydraulic method of --profile-only (fwave runs the workload's form, fwave-fp64 the FP64 "
                         "form, hllc the FP64 form, hllc-mixed the mixed FP32/FP64 form)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cases, precision, outer, cfg = build_workload(args.workload, rank, world, args.subset)   # before any CUDA use
    import torch
    torch.cuda.set_device(local)
    if args.profile_only:
        from braids_hkt_gb300.solver import RiverSolver
        if args.profile_method == "hllc":
            solver = RiverSolver(cases, precision="fp64", method="hllc")
        elif args.profile_method == "hllc-mixed":
            solver = RiverSolver(cases, precision="mixed", method="hllc")
        elif args.profile_method == "fwave-fp64":
            solver = RiverSolver(cases, precision="fp64")
        else:
            solver = RiverSolver(cases, precision=precision)
        dt = 1e-3                   # one trial of every kernel from the initial state, no interval before it
        for _ in range(args.profile_only):
            print(json.dumps({"cells": solver.nc, "substep_kernels_ms": solver.profile_substep(dt, 0.0)}))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from braids_hkt_gb300.solver import RiverSolver

    solver = RiverSolver(cases, precision=precision)
    prepare(solver, cases)
    nc, nf = solver.nc, solver.nf
    nadj = int(solver.packed["nadj"])
    nslot = len(solver.packed["boundary_faces"])
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = solver.stream

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    sim_time = 0.0
    failed = set()
    for _ in range(args.warmup):
        diags = outer_step(solver, outer, sim_time)
        diags = diags if isinstance(diags, list) else [diags]
        failed |= {i for i, d in enumerate(diags) if d["failed"]}
        sim_time += outer
    # launch schedule picked by the autotuner on this batch (outside the timed region)
    from braids_hkt_gb300 import autotune
    tuned = autotune.tune(solver, dt=0.25 * min(d["hydraulic_next_substep_hint_s"] for d in diags), time0=sim_time,
                          cache=False)
    cfg["autotune"] = {k: tuned.get(k) for k in ("kernels", "chunk", "chunk_ms", "tile", "substep_ms_default",
                                                 "substep_ms_tuned", "tuning_s")}
    # timed region: K steps of `chain` outer intervals each, device time by
    # events on the solver stream
    chain = max(1, args.chain) if solver.bed_model is None else 1
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = solver.launches()
    updates = 0
    device_ms = 0.0
    step_ms = []
    barrier()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        diags, n_up, f, sim_time = run_step(solver, outer, sim_time, chain)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        device_ms += step_ms[-1]
        failed |= f
        updates += n_up
    barrier()
    wall = time.perf_counter() - wall0
    gpu_launches = solver.launches() - launches0
    # substeps of the last timed interval per scenario: the batch runs as many
    # graph substeps as its slowest scenario needs
    subs = np.array([int(d["hydraulic_substeps"]) for d in diags])
    cells = np.diff(solver.packed["cell_offset"]).astype(np.int64)
    rej = np.array([int(d["hydraulic_rejections"]) for d in diags])
    cfg["substeps_per_interval"] = {"min": int(subs.min()), "median": float(np.median(subs)), "max": int(subs.max()),
                                    "cell_weighted_mean": float((subs * cells).sum() / cells.sum()),
                                    "rejected_trials_cell_weighted_mean": float((rej * cells).sum() / cells.sum())}
    clock_info = clocks.stop()
    t_max, updates = aggregate(device_ms / 1e3, updates, dist, "cuda")
    value = updates / t_max

    state_after_timed = solver.q.cpu().numpy()       # for the accuracy check against FP64 below
    bed_after_timed = solver.z.cpu().numpy()
    rotors_after_timed = solver.turbine_record() if solver.rotors is not None else None
    sim_after_timed = sim_time
    # end to end through the public API with host buffers: H2D of the step's
    # input state from pinned memory, advance, D2H of the result
    q_host = torch.empty_like(solver.q, device="cpu").pin_memory()
    q_host.copy_(solver.q)
    out_host = torch.empty_like(q_host).pin_memory()
    e2e_updates = 0
    barrier()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        solver.q.copy_(q_host, non_blocking=True)
        diags, n_up, _, sim_time = run_step(solver, outer, sim_time, chain, raise_on_failure=True)
        out_host.copy_(solver.q, non_blocking=True)
        torch.cuda.synchronize()
        e2e_updates += n_up
    e2e_s = time.perf_counter() - t0
    h2d = int(q_host.numel() * 8)
    # the other schedule of the same batch: interval by interval when the
    # steps were chained (each interval waits for the batch's slowest
    # scenario), else the steps' intervals chained on the device in one call
    interval_ms, iv_updates, chained = [], 0, None
    for _ in range(max(1, args.steps) if chain > 1 else 0):
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        diags, n_up, _, sim_time = run_step(solver, outer, sim_time, 1)
        e1.record(stream)
        e1.synchronize()
        interval_ms.append(e0.elapsed_time(e1))
        iv_updates += n_up
    if chain == 1 and solver.bed_model is None and len(cases) > 1:
        k = max(2, args.steps)
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        diags, n_up, _, sim_time = run_step(solver, outer, sim_time, k)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        chained = {"value": n_up / (ms / 1e3), "unit": METRIC, "intervals": k, "ms_per_interval": ms / k,
                   "note": "the same batch over the same number of outer intervals in one brx_advance_chain "
                           "call: each scenario begins its next interval on the device as soon as it has "
                           "finished one"}

    # live per-kernel timing of one substep for the roofline of the dominant kernel
    prof = solver.profile_substep(0.5 * min(d["hydraulic_next_substep_hint_s"] for d in diags), sim_time)
    per_kind = {}
    for name, ms in prof:
        per_kind.setdefault(name, []).append(ms)
    dom = max(per_kind, key=lambda k: sum(per_kind[k]))
    dom_ms = float(np.mean(per_kind[dom]))
    with_rotors = [i for i, c in enumerate(cases) if c.get("turbines")]
    rotor_cells = sum(int(solver.packed["cell_offset"][i + 1] - solver.packed["cell_offset"][i]) for i in with_rotors)
    rotor_faces = sum(int(solver.packed["face_offset"][i + 1] - solver.packed["face_offset"][i]) for i in with_rotors)
    dom_bytes = algorithmic_bytes(dom, nc, nf, nadj, nslot, precision, rotor_cells, rotor_faces)
    peak, peak_kind = peaks()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    per_cell = TRAFFIC_BYTES_PER_CELL.get(precision, {}).get(dom)
    traffic = per_cell * nc if per_cell is not None and args.workload == "config4" else None
    total_ms = sum(sum(v) for v in per_kind.values())
    roofline = {"bound": "hbm", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "traffic_source": ("ncu DRAM bytes per cell of a 24-scenario subset capture, scaled by cells"
                                   if traffic is not None else None),
                "peak_source": peak_kind,
                "kernel_ms": dom_ms, "kernel_share_of_substep": sum(per_kind[dom]) / total_ms,
                "substep_kernels_ms": {k: [round(v, 4) for v in vs] for k, vs in per_kind.items()},
                "algorithmic_bytes_per_launch": dom_bytes,
                "step_bytes_per_cell_update": BYTES_PER_CELL_UPDATE[precision],
                "step_achieved_gbs": value * BYTES_PER_CELL_UPDATE[precision] / 1e9}
    # the same scenarios one by one in the plain FP64 form, from the same initial state over the same
    # intervals: FP64 throughput and the mixed form's depth error against it
    plain = None
    if precision == "mixed" and args.plain > 0 and len(cases) > 1:
        # smallest / median / largest scenario among those with rotors (all, without rotors)
        pool = [i for i, c in enumerate(cases) if c.get("turbines")] or list(range(len(cases)))
        order = sorted(pool, key=lambda i: cases[i]["mesh"].nc)
        pick = [int(order[0]), int(order[len(order) // 2]), int(order[-1])][:args.plain]
        p_updates, p_ms, errs, perr, qerrs, merrs = 0, 0.0, [], [], [], []
        rotor_first = {}
        if solver.rotors is not None:
            for k, sid in enumerate(solver.rotors["scenario"]):
                rotor_first.setdefault(int(sid), []).append(k)
        batch_state = state_after_timed
        off = solver.packed["cell_offset"]
        nsteps = args.warmup + args.steps * chain
        h_updates, h_ms, h_failed = 0, 0.0, False
        for i in pick:
            if args.hllc:
                # the HLLC MUSCL-Hancock method on the same scenario, intervals and CFL (FP64 form)
                hs = RiverSolver(cases[i], precision="fp64", method="hllc")
                t_sim = 0.0
                for k in range(nsteps):
                    torch.cuda.synchronize()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(hs.stream)
                    d = hs.advance(outer, t_sim, raise_on_failure=False)
                    e1.record(hs.stream)
                    e1.synchronize()
                    t_sim += outer
                    h_failed = h_failed or bool(d["failed"])
                    if k >= args.warmup:
                        h_ms += e0.elapsed_time(e1)
                        h_updates += int(d["hydraulic_substeps"]) * int(hs.nc)
                hs.close()
            one = RiverSolver(cases[i], precision="fp64")
            t_sim = 0.0
            for k in range(nsteps):
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(one.stream)
                d = one.advance(outer, t_sim)
                e1.record(one.stream)
                e1.synchronize()
                t_sim += outer
                if k >= args.warmup:
                    p_ms += e0.elapsed_time(e1)
                    p_updates += int(d["hydraulic_substeps"]) * int(one.nc)
            q64 = one.q.cpu().numpy()
            h64 = q64[0]
            qmx = batch_state[:, off[i]:off[i + 1]]
            hmx = qmx[0]
            rel = np.abs(hmx - h64) / np.maximum(h64, 1e-3)
            errs.append((float(rel.max()), float(np.percentile(rel, 99))))
            # unit discharge (hu, hv) against the scenario's largest unit discharge
            qscale = max(float(np.abs(q64[1:]).max()), 1e-12)
            qerrs.append(float(np.abs(qmx[1:] - q64[1:]).max() / qscale))
            m64, mmx = float(np.sum(h64 * cases[i]["mesh"].area)), float(np.sum(hmx * cases[i]["mesh"].area))
            merrs.append(abs(mmx - m64) / m64)
            if one.rotors is not None and i in rotor_first:
                import braids_hkt_gb300.turbines as TB
                col = TB.DIAG_FIELDS.index("useful_power_per_density_m5_s3")
                p64 = one.turbine_record()[:, col]
                pmx = rotors_after_timed[rotor_first[i], col]
                perr += [float(abs(a - b) / max(abs(b), 1e-30)) for a, b in zip(pmx, p64) if b != 0]
            one.close()
        plain = {"value": p_updates / (p_ms / 1e3), "unit": METRIC, "scenarios": pick,
                 "cells": [int(cases[i]["mesh"].nc) for i in pick],
                 "note": "each scenario alone in the FP64 form over the same intervals"}
        if args.hllc:
            plain["hllc"] = {"value": h_updates / (h_ms / 1e3), "unit": METRIC,
                             "speedup_vs_fwave_fp64_same_intervals": p_ms / h_ms, "any_failed": h_failed,
                             "note": "the same scenarios alone with the HLLC MUSCL-Hancock method (FP64 form, one "
                                     "spatial evaluation per substep), the same intervals and CFL; speed-up = "
                                     "f-wave FP64 device time / HLLC device time for the same simulated time"}
        cfg["accuracy_vs_fp64"] = {"depth_rel_max": max(e[0] for e in errs), "depth_rel_p99": max(e[1] for e in errs),
                                   "unit_discharge_rel_max": max(qerrs),
                                   "volume_rel_max": max(merrs),
                                   "scenarios": pick, "after_sim_s": nsteps * outer,
                                   "stated_tolerance": 1e-4,
                                   "rotor_power_rel_max": max(perr) if perr else None,
                                   "rotors_compared": len(perr)}
    if precision == "mixed" and len(cases) == 1:
        # config 3: the FP64 form over the warm-up and timed intervals, from the same initial state
        cfg["accuracy_vs_fp64"] = fp64_comparison(cases, outer, args.warmup + args.steps * chain, state_after_timed,
                                                  bed_after_timed, rotors_after_timed, torch)
        plain = {"value": cfg["accuracy_vs_fp64"]["fp64_value"], "unit": METRIC,
                 "note": "the same scenario in the FP64 form over the same intervals"}
    hllc_batch, hllc_mixed = None, None
    if args.hllc and precision == "mixed" and len(cases) > 1:
        # the whole batch with the HLLC method, FP64 form then mixed form: one warm-up and up to two timed
        # intervals each, from the same initial state, so the mixed form's depth is compared after the same
        # intervals
        from braids_hkt_gb300 import autotune
        legs, finals = {}, {}
        for hprec in ("fp64", "mixed"):
            hs = RiverSolver(cases, precision=hprec, method="hllc")
            htuned = autotune.tune(hs, cache=False)
            t_sim, ms, ups, hfail = 0.0, 0.0, 0, set()
            for k in range(1 + max(1, min(args.steps, 2))):
                flush_l2(torch, flush)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(hs.stream)
                ds = hs.advance(outer, t_sim, raise_on_failure=False)
                e1.record(hs.stream)
                e1.synchronize()
                t_sim += outer
                hfail |= {i for i, d in enumerate(ds) if d["failed"]}
                if k >= 1:
                    ms += e0.elapsed_time(e1)
                    ups += sum(int(d["hydraulic_substeps"]) *
                               int(hs.packed["cell_offset"][i + 1] - hs.packed["cell_offset"][i])
                               for i, d in enumerate(ds))
            finals[hprec] = hs.q.cpu().numpy()
            hprof = hs.profile_substep(0.5 * min(d["hydraulic_next_substep_hint_s"] for d in ds), t_sim)
            legs[hprec] = {"value": ups / (ms / 1e3), "unit": METRIC,
                           "ms_per_interval": ms / max(1, min(args.steps, 2)), "failed_scenarios": sorted(hfail),
                           "substep_kernels_ms": [(n, round(v, 4)) for n, v in hprof],
                           "autotune": {k: htuned[k] for k in ("kernels", "chunk", "substep_ms_default",
                                                              "substep_ms_tuned")},
                           "note": f"the whole batch (rotors included) with the HLLC MUSCL-Hancock method, {hprec} "
                                   "form; one cell-update = one cell advanced by one accepted Hancock substep"}
            hs.close()
        hllc_batch, hllc_mixed = legs["fp64"], legs["mixed"]
        h64, hmx = finals["fp64"][0], finals["mixed"][0]
        rel = np.abs(hmx - h64) / np.maximum(h64, 1e-3)
        deep = h64 > 0.05
        hllc_mixed["accuracy_vs_fp64"] = {"depth_rel_max": float(rel.max()),
                                          "depth_rel_p99_deep": float(np.percentile(rel[deep], 99)),
                                          "unit_discharge_rel_max": float(np.abs(finals["mixed"][1:] - finals["fp64"][1:]).max() /
                                                                          max(np.abs(finals["fp64"][1:]).max(), 1e-12)),
                                          "after_sim_s": (1 + max(1, min(args.steps, 2))) * outer,
                                          "stated_tolerance": 1e-4}
        hllc_mixed["speedup_vs_fp64_hllc"] = hllc_mixed["value"] / hllc_batch["value"]
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": device_ms / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f32/f64 mixed",
            "data": "synthetic", "config": dict(cfg, cells=nc, faces=nf, outer_dt_s=outer, intervals_per_step=chain,
                                                step=(f"{chain} outer intervals per scenario, chained on the device "
                                                      "(brx_advance_chain)" if chain > 1 else "one outer interval"),
                                                failed_scenarios=sorted(failed),
                                                l2="flushed between steps (256 MiB write)",
                                                wall_s=wall),
            "roofline": roofline, "clocks": clock_info, "gpu_launches": int(gpu_launches),
            "latency_ms": ({"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                            "what": "device time of one outer interval of the whole batch"} if chain == 1 else
                           {"p50": float(np.percentile(interval_ms, 50)), "p99": float(np.percentile(interval_ms, 99)),
                            "what": "device time of one outer interval of the whole batch, run interval by interval",
                            "step_p50": float(np.percentile(step_ms, 50))}),
            "e2e": {"value": e2e_updates / e2e_s, "unit": METRIC, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": h2d}}
    line["compute_peaks"] = dict(fma_peaks(solver.lib), source="brx_fma_rate: 8 independent FMA chains per "
                                 "thread at full occupancy, CUDA events, best of 5")
    fp64_peak = line["compute_peaks"]["fp64_tflops"]
    if precision == "fp64":
        line["roofline_fp64"] = fp64_roofline(per_kind, nc, nf, value, fp64_peak)
    if plain is not None:
        plain["roofline_fp64"] = {"achieved": plain["value"] * FP64_FLOPS_PER_CELL_UPDATE / 1e12, "peak": fp64_peak,
                                  "unit": "TFLOP/s",
                                  "frac": plain["value"] * FP64_FLOPS_PER_CELL_UPDATE / 1e12 / fp64_peak,
                                  "step_flops_per_cell_update": FP64_FLOPS_PER_CELL_UPDATE,
                                  "flops_source": "ncu FP64 thread-instruction counts per cell-update of config 1"}
        line["roofline_fp64"] = dict(plain["roofline_fp64"], leg="plain_fp64")
    if chained is not None:
        line["chained"] = chained
    if interval_ms:
        line["interval_by_interval"] = {"value": iv_updates / (sum(interval_ms) / 1e3), "unit": METRIC,
                                        "intervals": len(interval_ms),
                                        "note": "the same batch advanced one outer interval per call: every "
                                                "interval waits for the batch's slowest scenario"}
    if plain is not None:
        line["plain_fp64"] = plain
        line["batched_vs_plain_fp64"] = value / plain["value"]
    if hllc_batch is not None:
        line["hllc_fp64_batch"] = hllc_batch
    if hllc_mixed is not None:
        line["hllc_mixed_batch"] = hllc_mixed
    if precision == "mixed" and not args.no_serving and len(cases) > 1:
        solver.close()
        try:
            line["serving"] = serving_session(cases, precision, rate=args.serving_rate, window=args.serving_window,
                                              duration=args.serving_duration)
            line["latency_ms"]["serving_p50_s"] = line["serving"]["latency_s"]["p50"]
            line["latency_ms"]["serving_p99_s"] = line["serving"]["latency_s"]["p99"]
        except TimeoutError as exc:
            line["serving"] = {"error": str(exc)}
    if not args.no_cpu_baseline:
        median = sorted(cases, key=lambda c: c["mesh"].nc)[len(cases) // 2]
        line["cpu_baseline"] = cpu_baseline([median], outer)
        line["cpu_baseline"].pop("seconds", None)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
