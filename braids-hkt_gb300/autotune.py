"""Autotuner of the launch schedule of a resident batch.

What it picks, per solver (a packed batch of scenarios, one arithmetic form
and hydraulic method):

  * the launch shape of every sweep kernel: the edge / cell tile a CTA takes
    per grid-stride step (threads per block, a multiple of 32 up to the
    kernel's own limit) and the grid cap (resident blocks per SM), through
    brx_launch_shape_set;
  * the CUDA-graph chunk: how many substeps one graph replay carries before
    the host reads the scenario clocks back (brx_graph_chunk_set);
  * mixed f-wave form, cells of at most four faces: the cell tile of the
    tile sweep (brx_tile_set: cells per tile, 0 for the separate cell, face
    and gather sweeps) and its grid cap.

How: every candidate shape is applied to all tunable kinds at once and one
trial substep is timed kernel by kernel with CUDA events
(brx_profile_substep); each kind keeps the shape with its smallest time (the
minimum over repetitions). Kernels are grid-stride sweeps whose results do
not depend on the shape, and the state, the step hints and the clock are
restored after every trial, so tuning changes nothing but speed. The chunk is
then chosen by timing a short fixed interval per candidate, and so is the
cell tile (the tile sweep waits for the boundary and rotor kernels that the
separate cell sweep overlaps, so only whole intervals compare them). Choices are cached
per (device, form, method, cells, faces, scenarios) in a JSON file beside the
built library, so a solver of the same shape is tuned once.

The reference has no counterpart: its kernels launch with fixed 128-thread
blocks (src/braids_support/gpu_fwave/reconstruction.py, resident_update.py).
"""
from __future__ import annotations

import json
import os
import time
from pathlib import Path

import numpy as np

from .build import BUILD

# tunable kernel kinds (brx_profile_substep kinds) per method; the rotor
# gradient / face kernels (12, 13) are timed inside the rotor group (11)
KINDS = {
    "fwave": {0: "drag", 2: "cells", 3: "faces", 4: "gather", 6: "update", 11: "rotors"},
    "hllc": {0: "drag", 20: "hllc_cells", 21: "hllc_predict", 23: "hllc_faces", 24: "hllc_budget",
             26: "hllc_update"},
}
ROTOR_MEMBERS = (12, 13)
BLOCKS = (64, 128, 256, 512)
PER_SM = (4, 8, 16, 32)
CHUNKS = (4, 8, 16, 32)
TILES = (128, 256, 512)            # cells per tile (0, the separate sweeps, is always a candidate)
TILE_PER_SM = (2, 4)
K_TILE = 15
CACHE = BUILD / "autotune.json"


def _key(solver):
    import torch
    dev = torch.cuda.get_device_name(torch.cuda.current_device())
    return f"{dev}|{solver.precision}|{solver.method}|{solver.nc}|{solver.nf}|{solver.nscen}"


def _members(solver, kind):
    """The shape slots a timed kind stands for (the rotor group sets its two sweeps)."""
    if kind == 11:
        return [k for k in ROTOR_MEMBERS if _limit(solver, k)]
    return [kind] if _limit(solver, kind) else []


def _limit(solver, kind):
    try:
        return solver.launch_shape(kind)[2]
    except Exception:
        return 0


def choose(timings, defaults):
    """Per kind, the candidate with the smallest time; ties keep the default.

    timings: {kind: {(block, per_sm): ms}}; defaults: {kind: (block, per_sm)}.
    Returns {kind: (block, per_sm, ms, default_ms)}.
    """
    out = {}
    for kind, table in timings.items():
        if not table:
            continue
        base = defaults[kind]
        best = min(table, key=lambda c: (table[c], c != base))
        out[kind] = (best[0], best[1], table[best], table.get(base, float("nan")))
    return out


def _trial(solver, dt, saved_q, time0):
    solver.q.copy_(saved_q)
    rows = solver.profile_substep(dt, time0, kinds=True)
    solver.q.copy_(saved_q)
    per = {}
    for kind, ms in rows:
        per[kind] = per.get(kind, 0.0) + ms
    return per


def _tune_tile(solver, saved_q, saved_hints, dt, time0, interval, tiles, sync=None, clock=time.perf_counter):
    """Cells per tile and grid cap of the tile sweep, or 0 (separate sweeps):
    the fastest of a short fixed interval, each candidate run twice from the
    same state (the first run builds its graph). None where the solver has
    no tile sweep (FP64 form, HLLC, cells of more than four faces). sync
    waits for the device (torch.cuda.synchronize by default)."""
    if sync is None:
        import torch
        sync = torch.cuda.synchronize
    if solver.precision != "mixed" or solver.method != "fwave":
        return None
    try:
        solver.set_tile(0)
    except Exception:
        return None
    hints = np.where(np.asarray(saved_hints) > 0, saved_hints, dt)
    span = interval if interval is not None else 32 * float(np.median(hints))

    def run():
        solver.q.copy_(saved_q)
        solver.set_hints(hints)
        solver.advance(span, time0, raise_on_failure=False)        # builds the graph
        solver.q.copy_(saved_q)
        solver.set_hints(hints)
        sync()
        w0 = clock()
        solver.advance(span, time0, raise_on_failure=False)
        sync()
        return (clock() - w0) * 1e3

    table = {"0": run()}
    best = (table["0"], 0, 0)
    for cells in tiles:
        try:
            solver.set_tile(cells)
        except Exception:
            continue
        for p in TILE_PER_SM:
            solver.set_launch_shape(K_TILE, 256, p)
            ms = run()
            table[f"{cells}x{p}"] = ms
            if ms < best[0]:
                best = (ms, cells, p)
    _, cells, p = best
    solver.set_tile(cells)
    if cells:
        solver.set_launch_shape(K_TILE, 256, p)
    return {"cells": int(cells), "per_sm": int(p), "interval_ms": {k: round(v, 3) for k, v in table.items()}}


def tune(solver, dt=1e-3, time0=0.0, reps=2, blocks=BLOCKS, per_sm=PER_SM, chunks=CHUNKS, interval=None,
         cache=True, verbose=False, tiles=TILES):
    """Tune the solver's launch shapes and graph chunk in place; returns a summary dict."""
    import torch
    key = _key(solver)
    store = {}
    if cache and CACHE.exists():
        try:
            store = json.loads(CACHE.read_text())
        except ValueError:
            store = {}
    kinds = KINDS[solver.method]
    if key in store:
        entry = store[key]
        for k, (b, p) in entry["shapes"].items():
            solver.set_launch_shape(int(k), b, p)
        solver.set_graph_chunk(entry["chunk"])
        if entry.get("tile"):
            solver.set_tile(entry["tile"]["cells"])
        return dict(entry, cached=True)
    t0 = time.perf_counter()
    torch.cuda.synchronize()
    saved_q = solver.q.clone()
    saved_hints = solver.hints()
    slots = {k: _members(solver, k) for k in kinds}
    slots = {k: v for k, v in slots.items() if v}
    member_default = {m: solver.launch_shape(m)[:2] for v in slots.values() for m in v}
    defaults = {k: member_default[v[0]] for k, v in slots.items()}
    limit = {k: min(_limit(solver, m) for m in v) for k, v in slots.items()}
    timings = {k: {} for k in slots}
    # warm the kernels (first launches load modules)
    _trial(solver, dt, saved_q, time0)
    for b in blocks:
        for p in per_sm:
            applied = []
            for k, members in slots.items():
                if b <= limit[k]:
                    for m in members:
                        solver.set_launch_shape(m, b, p)
                    applied.append(k)
            if not applied:
                continue
            best = {}
            for _ in range(reps):
                per = _trial(solver, dt, saved_q, time0)
                for k in applied:
                    if k in per:
                        best[k] = min(best.get(k, float("inf")), per[k])
            for k in applied:
                if k in best:
                    timings[k][(b, p)] = best[k]
            for members in slots.values():
                for m in members:
                    solver.set_launch_shape(m, *member_default[m])
    picked = choose(timings, defaults)
    for k, (b, p, _, _) in picked.items():
        for m in slots[k]:
            solver.set_launch_shape(m, b, p)
    # graph chunk: a fixed short interval from the same state, per candidate
    chunk_ms = {}
    if chunks:
        # about 32 substeps at the solver's current step hints (dt where it has none)
        hints = np.where(np.asarray(saved_hints) > 0, saved_hints, dt)
        span = interval if interval is not None else 32 * float(np.median(hints))
        for c in chunks:
            solver.set_graph_chunk(c)
            solver.q.copy_(saved_q)
            solver.set_hints(hints)
            solver.advance(span, time0, raise_on_failure=False)        # builds the graph
            solver.q.copy_(saved_q)
            solver.set_hints(hints)
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            solver.advance(span, time0, raise_on_failure=False)
            torch.cuda.synchronize()
            chunk_ms[c] = (time.perf_counter() - w0) * 1e3
        chunk = min(chunk_ms, key=chunk_ms.get)
        solver.set_graph_chunk(chunk)
    else:
        chunk = solver.graph_chunk
    # cell tile of the tile sweep: whole intervals from the same state per candidate
    tile = _tune_tile(solver, saved_q, saved_hints, dt, time0, interval, tiles) if tiles else None
    solver.q.copy_(saved_q)
    solver.set_hints(saved_hints)
    torch.cuda.synchronize()
    shapes = {}
    for k, (b, p, ms, base_ms) in picked.items():
        for m in slots[k]:
            shapes[str(m)] = [b, p]
    if tile is not None and tile["cells"]:
        shapes[str(K_TILE)] = [256, tile["per_sm"]]
    entry = dict(shapes=shapes, chunk=int(chunk), tile=tile,
                 kernels={kinds[k]: dict(block=b, per_sm=p, ms=round(ms, 4), default_ms=round(base_ms, 4))
                          for k, (b, p, ms, base_ms) in picked.items()},
                 substep_ms_default=round(sum(v[3] for v in picked.values()), 4),
                 substep_ms_tuned=round(sum(v[2] for v in picked.values()), 4),
                 chunk_ms={str(c): round(v, 3) for c, v in chunk_ms.items()},
                 tuning_s=round(time.perf_counter() - t0, 2), candidates=len(blocks) * len(per_sm))
    if cache:
        store[key] = entry
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            tmp = CACHE.with_suffix(".tmp")
            tmp.write_text(json.dumps(store, indent=1))
            os.replace(tmp, CACHE)
        except OSError:
            pass
    if verbose:
        print(json.dumps(entry))
    return dict(entry, cached=False)
