"""Host-side owner of resident river scenarios on one GB300.

``RiverSolver`` mirrors the reference's solver owner and explicit controller:

  reference                                               here
  ShorelineSolver(deck, data, backend='gpu', ...)          RiverSolver(case(s), precision=...)
    src/braids_core/sediment/shoreline_solver.py:244
  ShorelineSolver.step(dt) -> dict(q, z, ..., diagnostics) RiverSolver.step(dt)
    shoreline_solver.py:345-372
  RiverExplicit.advance(base, dt, time)                   RiverSolver.advance(dt, time)
    -> (q, water/dt, diagnostics)                           -> diagnostics (state updated in place)
    src/braids_core/sediment/river_explicit.py:121-154
  RiverExplicit._single(base, dt, time)                   RiverSolver.substep(dt, time)
    river_explicit.py:94-119
  RiverExplicit.rate(q, dt, time) -> (rate, water)        RiverSolver.rate(dt, time)
    river_explicit.py:63-92

Device memory for the resident state is owned by PyTorch tensors (``q`` and
``z``); all arithmetic runs in the CUDA library through its C ABI. Several
scenarios passed together are packed into one index space and advanced by the
same launches, each on its own clock.
"""
from __future__ import annotations

import ctypes as C
import numpy as np

from . import _lib
from ._lib import AdvanceStats, check

PRECISIONS = {"fp64": 0, "mixed": 1}
METHODS = {"fwave": 0, "hllc": 1}
METHOD = "explicit_fwave_ssprk22_river_v1"
METHOD_NAMES = {"fwave": METHOD, "hllc": "explicit_hllc_muscl_hancock_river_v1"}


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def rating_tables(cases):
    """Q-H rating curves of the mode-11 outlets of a batch: (offset (nseg+1),
    discharge, elevation) over the packed segments; case["rating"] maps a
    segment to its knots [(Q [m3/s], water elevation [m]), ...], elevation
    increasing (the reference's rating_curve rows, river_rating_outlet.py:12-16)."""
    off, rq, re_ = [0], [], []
    for case in cases:
        nb = case["mesh"].nb
        curves = case.get("rating") or {}
        modes = np.asarray(case.get("seg_mode", np.zeros(0)), dtype=int)
        for b in range(nb):
            knots = curves.get(b)
            if modes[b] == 11:
                if knots is None or len(knots) < 2:
                    raise ValueError(f"rating outlet segment {b} needs a curve of at least two knots")
                eta = np.array([float(e) for _, e in knots])
                if not np.all(np.diff(eta) > 0):
                    raise ValueError("rating curve elevations must increase")
                for qv, e in knots:
                    rq.append(float(qv))
                    re_.append(float(e))
            off.append(len(rq))
    return (np.asarray(off, np.int32), np.asarray(rq if rq else [0.0], np.float64),
            np.asarray(re_ if re_ else [0.0], np.float64))


def normal_chains(cases, face_offset=None):
    """Face chains of the normal-depth outlets (mode 10) of a batch, in
    scenario and segment order: (offset (nchain+1), faces (global ids), bed
    slope per chain). case["outlet"][segment]["bed_slope"] is the slope that
    stands in for the energy slope (river_normal_outlet.py:20-27)."""
    from .mesh import opening_chains
    off, faces, slopes = [0], [], []
    for i, case in enumerate(cases):
        F0 = 0 if face_offset is None else int(face_offset[i])
        modes = np.asarray(case.get("seg_mode", np.zeros(0)), dtype=int)
        for b in range(case["mesh"].nb):
            if modes[b] != 10:
                continue
            slope = float((case.get("outlet") or {}).get(b, {}).get("bed_slope", 0.0))
            if not slope > 0:
                raise ValueError(f"normal-depth outlet segment {b} needs a positive bed_slope")
            for chain in opening_chains(case["mesh"], b):
                faces.extend(int(f) + F0 for f in chain)
                off.append(len(faces))
                slopes.append(slope)
    return (np.asarray(off, np.int32), np.asarray(faces if faces else [0], np.int32),
            np.asarray(slopes, np.float64))


def critical_chains(cases, face_offset=None):
    """Connected face chains of the critical outlets (mode 4) of a batch:
    (chain range per packed segment (nseg+1), chain offsets, faces (global
    ids)) in scenario and segment order (CriticalOutlet's chains,
    river_exterior_outlet.py:20-21)."""
    from .mesh import opening_chains
    segc, off, faces = [0], [0], []
    for i, case in enumerate(cases):
        F0 = 0 if face_offset is None else int(face_offset[i])
        modes = np.asarray(case.get("seg_mode", np.zeros(0)), dtype=int)
        for b in range(case["mesh"].nb):
            if modes[b] == 4:
                for chain in opening_chains(case["mesh"], b):
                    faces.extend(int(f) + F0 for f in chain)
                    off.append(len(faces))
            segc.append(len(off) - 1)
    return (np.asarray(segc, np.int32), np.asarray(off, np.int32), np.asarray(faces if faces else [0], np.int32))


class WaterBudgetError(RuntimeError):
    """A step whose volume change differs from its boundary ledger (the reference's BendTrialRejected)."""


def water_budget(v0, v1, ledger, inventory=None, gross=None):
    """The owner's water-budget test per scenario (shoreline_solver.py:29-39,
    353-360): residual = (V1 - V0) - ledger against the FP64 roundoff
    allowance max(1e-10, 64 eps max(1, inventory, gross)). Without per-cell
    data the inventory is max(V0, V1) and the gross boundary volume |ledger|.
    Returns (residual, allowance, ok)."""
    v0, v1, ledger = (np.asarray(a, dtype=np.float64) for a in (v0, v1, ledger))
    residual = (v1 - v0) - ledger
    inventory = np.maximum(v0, v1) if inventory is None else np.asarray(inventory, dtype=np.float64)
    gross = np.abs(ledger) if gross is None else np.asarray(gross, dtype=np.float64)
    scale = np.maximum(1.0, np.maximum(np.abs(inventory), np.abs(gross)))
    allowance = np.maximum(1e-10, 64 * np.finfo(float).eps * scale)
    ok = np.isfinite(residual) & (np.abs(residual) <= allowance)
    return residual, allowance, ok


LINES = {"stage": 0, "critical": 1, "normal": 2}


def inlet_lines(cases, face_offset=None):
    """Reference water lines of the exact-discharge inlets (mode 9) of a batch:
    (kind (nseg): 0 the forcing stage (inlet.stage_discharge /
    depth_discharge), 1 critical depth (inlet.critical_discharge), 2 normal
    depth (inlet.normal_discharge); energy slope (nseg); left, right (nf
    global face ids, -1 none) the physical neighbours along normal-depth
    sections (river_exterior_section.py, river_exterior_normal.py)).
    case["inlet"][segment] = {"line": "stage" | "critical" | "normal",
    "energy_slope": s (normal only, > 0)}."""
    from .mesh import section_neighbours
    kind, slope, left, right = [], [], [], []
    for i, case in enumerate(cases):
        F0 = 0 if face_offset is None else int(face_offset[i])
        m = case["mesh"]
        modes = np.asarray(case.get("seg_mode", np.zeros(0)), dtype=int)
        lt = np.full(len(m.owner), -1, np.int64)
        rt = lt.copy()
        for b in range(m.nb):
            row = (case.get("inlet") or {}).get(b, {})
            line = row.get("line", "stage")
            if line not in LINES:
                raise ValueError(f"inlet segment {b}: unknown reference line {line!r}")
            if line != "stage" and modes[b] != 9:
                raise ValueError(f"segment {b}: a {line} reference line needs an exact-discharge inlet (mode 9)")
            value = float(row.get("energy_slope", 0.0))
            if line == "normal":
                if not (np.isfinite(value) and value > 0):
                    raise ValueError(f"normal inlet segment {b} needs a positive energy slope")
                l, r = section_neighbours(m, b)
                sel = l >= 0
                lt[sel] = l[sel] + F0
                sel = r >= 0
                rt[sel] = r[sel] + F0
            kind.append(LINES[line])
            slope.append(value)
        left.append(lt)
        right.append(rt)
    cat = lambda a: np.concatenate(a) if a else np.zeros(0)
    return (np.asarray(kind, np.int32), np.asarray(slope, np.float64), cat(left).astype(np.int32),
            cat(right).astype(np.int32))


def weir_parameters(cases):
    """(3, nseg) crest [m], coefficient [m^0.5/s] and effective width [m] of
    the free-weir outlets (mode 5) of a batch (FreeWeir's parameters,
    river_exterior_outlet.py:77-79); zero rows elsewhere.
    case["outlet"][segment] = {"crest_m", "coefficient_m_half_s", "effective_width_m"}."""
    cols = []
    for case in cases:
        modes = np.asarray(case.get("seg_mode", np.zeros(0)), dtype=int)
        for b in range(case["mesh"].nb):
            row = (case.get("outlet") or {}).get(b, {})
            vals = [float(row.get(k, 0.0)) for k in ("crest_m", "coefficient_m_half_s", "effective_width_m")]
            if modes[b] == 5 and not (np.isfinite(vals[0]) and vals[1] > 0 and vals[2] > 0):
                raise ValueError(f"free-weir segment {b} needs a finite crest and positive coefficient and width")
            cols.append(vals)
    return np.ascontiguousarray(np.array(cols, dtype=np.float64).T.reshape(3, -1))


def pack(cases):
    """Concatenate scenario meshes into one global index space."""
    out = {k: [] for k in ("owner", "neighbour", "bid", "offset", "faces", "signs", "normal", "length", "area",
                           "ls_matrix", "ls_weight", "ls_delta", "disp", "disp_len", "distance", "boundary_offset",
                           "boundary_faces", "seg_mode", "stage_policy", "exterior_bed", "forcing", "q", "z")}
    cell_off, face_off, seg_off = [0], [0], [0]
    nadj_total = 0
    nslot_total = 0
    for case in cases:
        m = case["mesh"]
        r = m.records
        C0, F0, S0 = cell_off[-1], face_off[-1], seg_off[-1]
        out["owner"].append(m.owner + C0)
        out["neighbour"].append(np.where(m.neighbour >= 0, m.neighbour + C0, -1))
        out["bid"].append(np.where(m.bid >= 0, m.bid + S0, -1))
        out["offset"].append(m.offset[:-1] + nadj_total)
        out["faces"].append(m.faces + F0)
        out["signs"].append(m.signs)
        out["normal"].append(m.normal)
        out["length"].append(m.length)
        out["area"].append(m.area)
        out["ls_matrix"].append(r["ls_matrix"])
        out["ls_weight"].append(r["ls_weight"])
        out["ls_delta"].append(r["ls_delta"])
        out["disp"].append(r["disp"])
        out["disp_len"].append(r["disp_len"])
        out["distance"].append(r["distance"])
        nb = m.nb
        out["boundary_offset"].append(m.boundary_offset[:-1] + nslot_total)
        out["boundary_faces"].append(m.boundary_faces + F0)
        if nb:
            out["seg_mode"].append(np.asarray(case["seg_mode"], np.int32))
            out["stage_policy"].append(np.asarray(case.get("stage_policy", np.zeros(nb)), np.int32))
            out["forcing"].append(np.asarray(case["forcing"], np.float64)[:, :nb])
        out["exterior_bed"].append(np.asarray(case.get("exterior_bed", np.zeros(m.nf)), np.float64))
        out["q"].append(np.asarray(case["q"], np.float64))
        out["z"].append(np.asarray(case["z"], np.float64))
        nadj_total += m.nadj
        nslot_total += len(m.boundary_faces)
        cell_off.append(C0 + m.nc)
        face_off.append(F0 + m.nf)
        seg_off.append(S0 + nb)
    p = {}
    for k in ("owner", "neighbour", "bid", "faces", "signs", "boundary_faces", "seg_mode", "stage_policy"):
        p[k] = _i32(np.concatenate(out[k]) if out[k] else np.zeros(0))
    p["offset"] = _i32(np.concatenate(out["offset"] + [np.array([nadj_total])]))
    p["boundary_offset"] = _i32(np.concatenate(out["boundary_offset"] + [np.array([nslot_total])]))
    for k in ("length", "area", "ls_weight", "exterior_bed", "z"):
        p[k] = _f64(np.concatenate(out[k]))
    for k in ("normal", "ls_matrix", "ls_delta", "disp_len", "distance", "q"):
        p[k] = _f64(np.concatenate(out[k], axis=-1))
    p["disp"] = _f64(np.concatenate(out["disp"], axis=-1))
    p["forcing"] = _f64(np.concatenate(out["forcing"], axis=1)) if out["forcing"] else np.zeros((2, 0))
    p["cell_offset"] = _i32(cell_off)
    p["face_offset"] = _i32(face_off)
    p["seg_offset"] = _i32(seg_off)
    p["nc"], p["nf"], p["nadj"], p["nseg"] = cell_off[-1], face_off[-1], nadj_total, seg_off[-1]
    return p


class RiverSolver:
    """Resident GB300 river scenarios advanced by the CUDA step (see module docstring)."""

    def __init__(self, cases, precision="fp64", graph_chunk=8, method="fwave"):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("RiverSolver needs a CUDA device; the step has no CPU implementation")
        self.torch = torch
        self.single = isinstance(cases, dict)
        self.cases = [cases] if self.single else list(cases)
        self.precision = precision
        self.lib = _lib.load()
        p = self.packed = pack(self.cases)
        self.nscen = len(self.cases)
        self.nc, self.nf = p["nc"], p["nf"]
        handle = C.c_void_p()
        check(self.lib.brx_solver_create(
            self.nscen, _ptr(p["cell_offset"]), _ptr(p["face_offset"]), p["nc"], p["nf"], p["nadj"],
            _ptr(p["owner"]), _ptr(p["neighbour"]), _ptr(p["bid"]), _ptr(p["offset"]), _ptr(p["faces"]),
            _ptr(p["signs"]), _ptr(p["normal"]), _ptr(p["length"]), _ptr(p["area"]), _ptr(p["ls_matrix"]),
            _ptr(p["ls_weight"]), _ptr(p["ls_delta"]), _ptr(p["disp"]), _ptr(p["disp_len"]), _ptr(p["distance"]),
            p["nseg"],
            _ptr(p["seg_offset"]), _ptr(p["boundary_offset"]), _ptr(p["boundary_faces"]),
            PRECISIONS[precision], C.byref(handle)))
        self.h = handle
        for i, case in enumerate(self.cases):
            c = case["controls"]
            check(self.lib.brx_controls_set(self.h, i, c["grav"], c["dry"], c["cfl"], c["speed_limit"],
                                            int(c["roughness_mode"]), c["roughness_value"]))
        if p["nseg"]:
            if np.any(p["seg_mode"] == 11):
                off, rq, re_ = rating_tables(self.cases)
                check(self.lib.brx_rating_set(self.h, _ptr(off), _ptr(rq), _ptr(re_)))
            if np.any(p["seg_mode"] == 4):
                segc, off, faces = critical_chains(self.cases, p["face_offset"])
                check(self.lib.brx_critical_chains_set(self.h, _ptr(segc), _ptr(off), _ptr(faces)))
            if np.any(p["seg_mode"] == 5):
                check(self.lib.brx_weir_set(self.h, _ptr(weir_parameters(self.cases))))
            if np.any(p["seg_mode"] == 10):
                off, faces, slope = normal_chains(self.cases, p["face_offset"])
                check(self.lib.brx_outlet_chains_set(self.h, len(slope), _ptr(off), _ptr(faces), _ptr(slope)))
            if any(case.get("inlet") for case in self.cases):
                kind, slope, left, right = inlet_lines(self.cases, p["face_offset"])
                check(self.lib.brx_inlet_lines_set(self.h, _ptr(kind), _ptr(slope), _ptr(left), _ptr(right)))
            check(self.lib.brx_boundary_set(self.h, _ptr(p["seg_mode"]), _ptr(p["stage_policy"]),
                                            _ptr(p["exterior_bed"]), _ptr(p["forcing"])))
        else:
            check(self.lib.brx_boundary_set(self.h, None, None, None, None))
        dev = torch.device("cuda", torch.cuda.current_device())
        self.q = torch.from_numpy(p["q"]).to(dev).contiguous()
        self.z = torch.from_numpy(p["z"]).to(dev).contiguous()
        check(self.lib.brx_state_bind(self.h, C.c_void_p(self.q.data_ptr()), C.c_void_p(self.z.data_ptr())))
        check(self.lib.brx_graph_chunk_set(self.h, int(graph_chunk)))
        self.graph_chunk = int(graph_chunk)
        self.rotors = None
        from . import turbines as TB
        tp = TB.pack(self.cases, p["cell_offset"])
        if tp is not None:
            self.rotors = tp
            check(self.lib.brx_turbines_set(
                self.h, tp["nrotor"], _ptr(tp["scenario"]), _ptr(tp["param"]), _ptr(tp["curve"]),
                len(tp["curve_x"]), _ptr(tp["curve_x"]), _ptr(tp["curve_y"]), _ptr(tp["support_offset"]),
                _ptr(tp["support_cell"]), _ptr(tp["support_weight"]), _ptr(tp["support_density"]),
                _ptr(tp["plane_offset"]), _ptr(tp["plane_cell"]), _ptr(tp["plane_delta"]), _ptr(tp["dxdy"]),
                _ptr(tp["inverse"]), _ptr(tp["xy"]), _ptr(tp["mid_disp"]), _ptr(tp["nu"]), _ptr(tp["hkt"])))
        if any(c.get("viscosity", 0.0) > 0.0 for c in self.cases):
            # the wet-bank viscosity (shoreline_viscosity.py:46-72) and its least-squares metric
            from .turbines import flow_geometry
            nu = _f64([float(c.get("viscosity", 0.0)) for c in self.cases])
            geo = [flow_geometry(c["mesh"]) for c in self.cases]
            dxdy = _f64(np.concatenate([g[0] for g in geo], axis=1))
            inverse = _f64(np.concatenate([g[1] for g in geo], axis=1))
            xy = _f64(np.concatenate([c["mesh"].xy for c in self.cases], axis=1))
            check(self.lib.brx_viscosity_set(self.h, _ptr(nu), _ptr(dxdy), _ptr(inverse), _ptr(xy)))
        self.method = method
        if method not in METHODS:
            raise ValueError(f"unknown hydraulic method {method!r}")
        if method == "hllc":
            # the HLLC owner (river_hllc.install, river_hllc.py:95-101): its own stencil, then the switch
            from . import hllc as HL
            hp = HL.pack(self.cases, p["cell_offset"], p["face_offset"])
            check(self.lib.brx_hllc_set(self.h, _ptr(hp["entry_face"]), _ptr(hp["entry_other"]),
                                        _ptr(hp["entry_geo"]), _ptr(hp["inverse"])))
            check(self.lib.brx_method_set(self.h, METHODS[method]))
        self.bed_model = None
        if any(c.get("exner") for c in self.cases):
            self._set_exner()
        self.time = np.zeros(self.nscen)
        self.steps = 0

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.brx_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self.torch.cuda.ExternalStream(self.lib.brx_stream(self.h))

    def launches(self):
        return int(self.lib.brx_launch_count(self.h))

    # --- Exner bed model -------------------------------------------------
    def _set_exner(self):
        from . import turbines as TB
        p = self.packed
        en = np.zeros(self.nscen, np.int32)
        par = np.zeros((self.nscen, 5))
        bedbc = np.zeros(self.nf, np.int32)
        feed = np.zeros(self.nf)
        rock = np.full(self.nc, -1e30)
        dxdy, inv, xy = [], [], []
        for i, case in enumerate(self.cases):
            m = case["mesh"]
            c0, c1 = p["cell_offset"][i], p["cell_offset"][i + 1]
            f0, f1 = p["face_offset"][i], p["face_offset"][i + 1]
            ex = case.get("exner")
            flow = case.get("_flow") or TB.flow_geometry(m)
            case["_flow"] = flow
            dxdy.append(flow[0]); inv.append(flow[1]); xy.append(m.xy)
            if not ex:
                continue
            en[i] = 1
            par[i] = (ex["diameter"], ex["porosity"], ex["chezy"], ex.get("morfac", 1.0), ex["sediment_depth"])
            bedbc[f0:f1] = ex["bedbc"]
            feed[f0:f1] = ex["feed"]
            rock[c0:c1] = ex["rock"]
        self.bed_model = en
        cat = lambda a: np.ascontiguousarray(np.concatenate(a, axis=1))
        self._ex_keep = (cat(dxdy), cat(inv), cat(xy))
        check(self.lib.brx_exner_set(self.h, _ptr(en), _ptr(_f64(par)), _ptr(bedbc), _ptr(feed), _ptr(rock),
                                     _ptr(self._ex_keep[0]), _ptr(self._ex_keep[1]), _ptr(self._ex_keep[2])))

    def morphology(self, dt):
        """One Exner bed update of the current state over dt (scalar or per scenario);
        per-scenario dicts: ok, solid-volume residual and boundary [m3], donor
        minimum, maximum relative change. The bed is replaced where ok."""
        if self.bed_model is None:
            raise ValueError("no bed model")
        self.torch.cuda.current_stream().synchronize()
        d = _f64(np.broadcast_to(dt, (self.nscen,)) * (self.bed_model > 0))
        stats = np.zeros((self.nscen, 8))
        check(self.lib.brx_exner(self.h, _ptr(d), _ptr(stats)))
        out = [dict(ok=bool(r[0]), residual=r[1], boundary=r[2], donor=r[3], change=r[4], slope_failure=bool(r[5]))
               for r in stats]
        return out[0] if self.single else out

    # --- rotor arrays ---------------------------------------------------
    def turbine_record(self, last=False):
        """(nrotor, 16) rotor record of the current state (or of the last evaluated stage)."""
        from . import turbines as TB
        if self.rotors is None:
            raise ValueError("no rotor arrays")
        self.torch.cuda.current_stream().synchronize()
        out = np.zeros((self.rotors["nrotor"], TB.NDIAG))
        fn = self.lib.brx_turbines_last if last else self.lib.brx_turbines_diagnose
        check(fn(self.h, _ptr(out)))
        return out

    def turbines(self, scenario=None):
        """Per-rotor diagnostics of the current state (the reference's hkt_diagnose),
        with thrust [N] and power [W] at water density 1000 kg/m3."""
        from . import turbines as TB
        rec = self.turbine_record()
        rows = TB.diagnostics_rows(rec, self.rotors["names"])
        for row, sid in zip(rows, self.rotors["scenario"]):
            row["scenario"] = int(sid)
            err = int(row["error"])
            if err:
                raise ValueError(f"rotor {row['turbine_id']}: {TB.ERRORS.get(err, 'model error')}")
        if scenario is not None:
            rows = [r for r in rows if r["scenario"] == scenario]
        return rows

    def performance_history(self, duration, interval):
        """Per-rotor thrust and power at fixed output times, as the reference
        worker publishes them (TURBINE_PERFORMANCE rows,
        adaptive_river_worker.py:577-587): owner steps of ``interval`` (each
        with its water-budget check) up to ``duration``; after each step one
        row per rotor with time_s, turbine_id, thrust_N, useful_power_W,
        hydraulic_work_W and the rest of the rotor's diagnostics."""
        rows = []
        for _ in range(int(round(duration / interval))):
            self.step(interval)
            for r in self.turbines():
                rows.append(dict(r, time_s=float(self.time[r["scenario"]])))
        return rows

    def set_forcing_table(self, time, value):
        """value (2, nseg, len): discharge and stage tables for every segment."""
        t = _f64(time)
        v = _f64(value)
        check(self.lib.brx_forcing_table_set(self.h, len(t), _ptr(t), _ptr(v)))

    # ------------------------------------------------------------------
    def identity(self):
        """What a checkpoint must match: format, form, method and digests of
        the packed geometry and boundary set-up."""
        from .checkpoint import digest
        p = self.packed
        geometry = digest(*(p[k] for k in ("cell_offset", "face_offset", "owner", "neighbour", "bid", "offset",
                                            "faces", "signs", "normal", "length", "area")))
        boundary = digest(*(p[k] for k in ("seg_mode", "stage_policy", "exterior_bed", "forcing")))
        return dict(precision=self.precision, method=self.method, scenarios=int(self.nscen), cells=int(self.nc),
                    faces=int(self.nf), geometry_sha256=geometry, boundary_sha256=boundary)

    def checkpoint_bytes(self, time=0.0, steps=0):
        """Accepted state q, bed z and step hints as checkpoint bytes
        (ShorelineSolver.checkpoint_bytes, shoreline_solver.py:374-381)."""
        from .checkpoint import encode
        if getattr(self, "_pending", False):
            raise ValueError("a checkpoint needs the accepted state (an interval is in flight)")
        self.torch.cuda.current_stream().synchronize()
        arrays = dict(q=self.q.cpu().numpy(), z=self.z.cpu().numpy(), hints=self.hints())
        return encode(self.identity(), arrays, time, steps)

    def checkpoint(self, path, time=0.0, steps=0):
        """Write a checkpoint atomically (temporary file, then os.replace)."""
        from .checkpoint import write_atomic
        write_atomic(path, self.checkpoint_bytes(time, steps))

    def restart_bytes(self, payload):
        """Validate, then load a checkpoint; returns its header (time, steps)
        (ShorelineSolver.restart, shoreline_solver.py:386-408): nothing
        changes unless the identity, inventory, shapes, dtypes and hashes all
        match."""
        from .checkpoint import decode
        expected = dict(q=(tuple(self.q.shape), np.float64), z=(tuple(self.z.shape), np.float64),
                        hints=((self.nscen,), np.float64))
        arrays, header = decode(payload, self.identity(), expected)
        self.torch.cuda.current_stream().synchronize()
        self.q.copy_(self.torch.from_numpy(arrays["q"]))
        self.z.copy_(self.torch.from_numpy(arrays["z"]))
        self.set_hints(arrays["hints"])
        self.torch.cuda.current_stream().synchronize()
        return header

    def restart(self, path):
        with open(path, "rb") as f:
            return self.restart_bytes(f.read())

    def activate(self, mask):
        m = _i32(mask)
        check(self.lib.brx_scenarios_activate(self.h, _ptr(m)))

    def forcing(self):
        """(2, nseg) discharge and stage of the last evaluated stage (solved inlet lines included)."""
        nseg = int(self.packed["nseg"])
        out = np.zeros((2, max(nseg, 1)))
        check(self.lib.brx_forcing_get(self.h, _ptr(out)))
        return out[:, :nseg]

    def hints(self):
        out = np.zeros(self.nscen)
        check(self.lib.brx_hint_get(self.h, _ptr(out)))
        return out

    def set_hints(self, hints):
        h = _f64(hints)
        check(self.lib.brx_hint_set(self.h, _ptr(h)))

    # ------------------------------------------------------------------
    def advance(self, dt, time=None, raise_on_failure=True):
        """Advance over [time, time+dt]; per-scenario diagnostics.

        dt and time may be scalars (all active scenarios) or arrays of one
        interval per scenario (dt <= 0 leaves a scenario idle).
        """
        self.torch.cuda.current_stream().synchronize()
        stats = (AdvanceStats * self.nscen)()
        if np.ndim(dt) == 0 and (time is None or np.ndim(time) == 0):
            t = float(self.time[0] if time is None else time)
            code = self.lib.brx_advance(self.h, float(dt), t, stats)
        else:
            d = _f64(np.broadcast_to(dt, (self.nscen,)))
            t = _f64(np.broadcast_to(self.time if time is None else time, (self.nscen,)))
            code = self.lib.brx_advance_batch(self.h, _ptr(d), _ptr(t), stats)
        if code and (raise_on_failure or code != 4):
            check(code)
        out = []
        for s in stats:
            out.append(dict(integrator=METHOD_NAMES[self.method], hydraulic_substeps=s.substeps, hydraulic_rejections=s.rejections,
                            hydraulic_minimum_dt=s.min_dt, hydraulic_maximum_dt=s.max_dt,
                            accepted_cfl_max=s.accepted_cfl_max, hydraulic_next_substep_hint_s=s.hint,
                            failed=s.failed))
        return out[0] if self.single else out

    def advance_chain(self, dt, time, intervals, raise_on_failure=True):
        """`intervals` consecutive intervals of dt per scenario from `time`,
        chained on the device: a scenario that completes an interval begins
        the next at once (interval k starts at time + dt + ... + dt, k terms
        added one by one). Returns per scenario a list of per-interval
        diagnostics (as advance gives them, plus the interval's boundary
        ledger and gross boundary volume); each interval is the one that
        `intervals` consecutive advance calls with those start times give.
        """
        self.torch.cuda.current_stream().synchronize()
        k = int(intervals)
        d = _f64(np.broadcast_to(dt, (self.nscen,)))
        t = _f64(np.broadcast_to(self.time if time is None else time, (self.nscen,)))
        stats = (AdvanceStats * (self.nscen * k))()
        ledger = np.zeros(self.nscen * k)
        gross = np.zeros(self.nscen * k)
        code = self.lib.brx_advance_chain(self.h, _ptr(d), _ptr(t), k, stats, _ptr(ledger), _ptr(gross))
        if code and (raise_on_failure or code != 4):
            check(code)
        out = []
        for i in range(self.nscen):
            rows = []
            for j in range(k):
                s = stats[i * k + j]
                rows.append(dict(integrator=METHOD_NAMES[self.method], hydraulic_substeps=s.substeps,
                                 hydraulic_rejections=s.rejections, hydraulic_minimum_dt=s.min_dt,
                                 hydraulic_maximum_dt=s.max_dt, accepted_cfl_max=s.accepted_cfl_max,
                                 hydraulic_next_substep_hint_s=s.hint, failed=s.failed,
                                 boundary_ledger_m3=float(ledger[i * k + j]),
                                 gross_boundary_volume_m3=float(gross[i * k + j])))
            out.append(rows)
        return out[0] if self.single else out

    # --- asynchronous intervals (serving loops) ---------------------------
    def advance_start(self, dt, time):
        """Launch one interval per scenario (arrays; dt <= 0 idles a scenario) and return at once."""
        self.torch.cuda.current_stream().synchronize()
        d = _f64(np.broadcast_to(dt, (self.nscen,)))
        t = _f64(np.broadcast_to(time, (self.nscen,)))
        check(self.lib.brx_advance_start(self.h, _ptr(d), _ptr(t)))
        self._async_stats = (AdvanceStats * self.nscen)()
        self._pending = True

    def advance_poll(self):
        """None while the interval runs; per-scenario diagnostics once it has finished."""
        done = C.c_int(0)
        code = self.lib.brx_advance_poll(self.h, C.byref(done), self._async_stats)
        if code and code != 4:
            check(code)
        if not done.value:
            return None
        self._pending = False
        return [dict(integrator=METHOD_NAMES[self.method], hydraulic_substeps=s.substeps, hydraulic_rejections=s.rejections,
                     hydraulic_minimum_dt=s.min_dt, hydraulic_maximum_dt=s.max_dt,
                     accepted_cfl_max=s.accepted_cfl_max, hydraulic_next_substep_hint_s=s.hint,
                     failed=s.failed) for s in self._async_stats]

    def device_bytes(self):
        """Device memory the solver holds (its allocations plus the bound state)."""
        return int(self.lib.brx_solver_bytes(self.h)) + self.q.numel() * 8 + self.z.numel() * 8

    def ledger(self):
        """Net inflow volume [m3] through the open faces over the last interval, per scenario."""
        out = np.zeros(self.nscen)
        check(self.lib.brx_ledger_get(self.h, _ptr(out)))
        return out

    def gross_boundary_volume(self):
        """Sum over the last interval's accepted substeps of dt x sum |face water x length| [m3],
        per scenario: an upper bound of the reference's gross boundary volume."""
        out = np.zeros(self.nscen)
        check(self.lib.brx_ledger_gross_get(self.h, _ptr(out)))
        return out

    def _inventory(self, h0, h1):
        """sum(max(h0, h1) area) per scenario (shoreline_solver.py:356): the
        water inventory that scales the roundoff allowance."""
        a = self.packed["area"]
        v = np.maximum(h0, h1) * a
        return np.add.reduceat(v, self.packed["cell_offset"][:-1].astype(np.int64))

    def step(self, dt):
        """Advance by dt from the owner clock with the owner's water-budget
        check (ShorelineSolver.step, shoreline_solver.py:345-372): the volume
        change of every scenario must equal its boundary ledger within the
        FP64 roundoff allowance max(1e-10, 64 eps max(1, inventory, gross))
        with the inventory sum(max(h0, h1) A) as the reference's and the gross
        boundary volume bounded from above; else the state is restored and
        WaterBudgetError raised; on success the ledger is committed."""
        self.torch.cuda.current_stream().synchronize()
        q0, z0, hints0 = self.q.clone(), self.z.clone(), self.hints()
        v0 = np.atleast_2d(self.totals())[:, 0]
        try:
            diag = self.advance(dt, self.time[0])
        except BaseException:
            self.q.copy_(q0); self.z.copy_(z0); self.set_hints(hints0)
            raise
        v1 = np.atleast_2d(self.totals())[:, 0]
        ledger = self.ledger()
        inventory = self._inventory(q0[0].cpu().numpy(), self.q[0].cpu().numpy())
        residual, roundoff, ok = water_budget(v0, v1, ledger, inventory, self.gross_boundary_volume())
        if not ok.all():
            self.q.copy_(q0); self.z.copy_(z0); self.set_hints(hints0)
            i = int(np.flatnonzero(~ok)[0])
            raise WaterBudgetError(f"scenario {i}: water budget failed: residual={residual[i]:.6e} m3, "
                                   f"roundoff={roundoff[i]:.6e} m3")
        self.water_ledger = getattr(self, "water_ledger", np.zeros(self.nscen)) + ledger
        self.time += dt
        self.steps += 1
        rows = diag if isinstance(diag, list) else [diag]
        for r, res, lim in zip(rows, residual, roundoff):
            r["water_residual_m3"] = float(res)
            r["water_increment_roundoff_limit_m3"] = float(lim)
        return dict(q=self.q, z=self.z, diagnostics=diag)

    def substep(self, dt, time=0.0):
        """One SSPRK(2,2) trial of exactly dt: (status bits, stage-peak CFL frequency) per scenario."""
        self.torch.cuda.current_stream().synchronize()
        status = np.zeros(self.nscen, np.uint32)
        peak = np.zeros(self.nscen)
        check(self.lib.brx_substep(self.h, float(dt), float(time), _ptr(status), _ptr(peak)))
        return (status[0], peak[0]) if self.single else (status, peak)

    def advance_recorded(self, dt, time, hint=None):
        """Advance one scenario over [time, time + dt] with the substep
        controller run on the host (RiverExplicit.advance's rules,
        river_explicit.py:121-154: trial = min(hint, remaining); reject on a
        status or dt * peak > CFL and retry at min(dt / 2, 0.98 CFL / peak);
        on acceptance grow the hint to 2 dt, capped by 0.98 CFL / peak).
        Returns (accepted substep lengths, next hint). With advance_replay,
        two arithmetic forms can run one substep sequence, which separates
        round-off from the two controllers choosing different sequences."""
        if not self.single:
            raise ValueError("advance_recorded drives one scenario")
        cfl = self.cases[0]["controls"]["cfl"]
        hint = float(dt if hint is None else hint)
        elapsed, dts, rejections = 0.0, [], 0
        while elapsed < dt - 1e-13 * max(1.0, dt):
            trial = min(hint, dt - elapsed)
            truncated = trial < hint * (1 - 1e-12)
            status, peak = self.substep(trial, time + elapsed)
            if status:
                rejections += 1
                if rejections > 100 or trial < dt * 2.0 ** -20:
                    raise RuntimeError(f"substep controller failed at t={time + elapsed}: status {status}")
                hint = min(0.5 * trial, 0.98 * cfl / peak) if peak > 0 else 0.5 * trial
                continue
            elapsed += trial
            dts.append(trial)
            growth = hint if truncated else 2.0 * trial
            hint = min(growth, 0.98 * cfl / peak) if peak > 0 else growth
        return dts, hint

    def advance_replay(self, dts, time):
        """Advance one scenario by exactly the substep lengths ``dts`` from
        ``time``. The CFL acceptance test is lifted (limit 1) for the replay;
        any other rejection raises. Returns the number of substeps."""
        if not self.single:
            raise ValueError("advance_replay drives one scenario")
        c = self.cases[0]["controls"]
        check(self.lib.brx_controls_set(self.h, 0, c["grav"], c["dry"], 1.0, c["speed_limit"],
                                        int(c["roughness_mode"]), c["roughness_value"]))
        try:
            t = float(time)
            for dt in dts:
                status, _ = self.substep(dt, t)
                if int(status):
                    raise RuntimeError(f"replayed substep rejected at t={t}: status {int(status)}")
                t += dt
        finally:
            check(self.lib.brx_controls_set(self.h, 0, c["grav"], c["dry"], c["cfl"], c["speed_limit"],
                                            int(c["roughness_mode"]), c["roughness_value"]))
        return len(dts)

    def rate(self, dt, time=0.0):
        """One spatial residual of the current state: (rate (3,nc), water (nf), status, frequency)."""
        torch = self.torch
        torch.cuda.current_stream().synchronize()
        rate = torch.zeros((3, self.nc), dtype=torch.float64, device=self.q.device)
        water = torch.zeros(self.nf, dtype=torch.float64, device=self.q.device)
        status = np.zeros(self.nscen, np.uint32)
        freq = np.zeros(self.nscen)
        check(self.lib.brx_rate(self.h, float(dt), float(time), C.c_void_p(rate.data_ptr()),
                                C.c_void_p(water.data_ptr()), _ptr(status), _ptr(freq)))
        if self.single:
            return rate, water, status[0], freq[0]
        return rate, water, status, freq

    # ------------------------------------------------------------------
    def load_scenario(self, i, q, forcing=None):
        """Re-use scenario slot i for a new run: its state (3, nc_i) into the
        resident buffer, its open-boundary forcing (2, nseg_i) when given, and
        its step hint cleared (the next interval starts at its full length, as
        a new solver does). Between intervals only."""
        a, b = int(self.packed["cell_offset"][i]), int(self.packed["cell_offset"][i + 1])
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.shape != (3, b - a):
            raise ValueError(f"scenario {i} takes a (3, {b - a}) state")
        self.torch.cuda.current_stream().synchronize()
        self.q[:, a:b].copy_(self.torch.from_numpy(q))
        if forcing is not None:
            s0, s1 = int(self.packed["seg_offset"][i]), int(self.packed["seg_offset"][i + 1])
            f = self.packed["forcing"]
            f[:, s0:s1] = np.asarray(forcing, dtype=np.float64)[:, :s1 - s0]
            check(self.lib.brx_forcing_set(self.h, _ptr(f)))
        hints = self.hints()
        hints[i] = 0.0
        self.set_hints(hints)
        self.torch.cuda.current_stream().synchronize()

    def set_state(self, q):
        self.q.copy_(self.torch.from_numpy(_f64(q)))

    def state(self, scenario=None):
        q = self.q.cpu().numpy()
        if scenario is None:
            return q
        a, b = self.packed["cell_offset"][scenario], self.packed["cell_offset"][scenario + 1]
        return q[:, a:b]

    def totals(self):
        """(nscen, 2) compensated water volume [m3] and mechanical energy per unit density
        [m5/s2] of the current state, summed on the device in a fixed order."""
        self.torch.cuda.current_stream().synchronize()
        out = np.zeros((self.nscen, 2))
        check(self.lib.brx_totals(self.h, _ptr(out)))
        return out[0] if self.single else out

    def mass(self):
        """Water volume per scenario (Kahan-compensated FP64 sum on the host)."""
        q = self.q[0].cpu().numpy()
        area = self.packed["area"]
        out = []
        for i in range(self.nscen):
            a, b = self.packed["cell_offset"][i], self.packed["cell_offset"][i + 1]
            out.append(kahan_sum(q[a:b] * area[a:b]))
        return out[0] if self.single else np.array(out)


def kahan_sum(values):
    s = 0.0
    c = 0.0
    for v in np.asarray(values, dtype=np.float64).tolist():
        y = v - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


def _profile(self, dt, time=0.0, kinds=False):
    """Per-kernel durations (ms) of one trial launched without a graph: [(kernel name, ms), ...]
    (kernel kind ids instead of names with kinds=True)."""
    names = {0: "drag", 1: "boundary", 2: "cells", 3: "faces", 4: "gather", 5: "limit", 6: "update",
             7: "control", 11: "rotors", 14: "viscosity", 15: "tile",
             20: "hllc_cells", 21: "hllc_predict", 22: "boundary", 23: "hllc_faces", 24: "hllc_budget",
             25: "rotors", 26: "hllc_update", 27: "rotors_start"}
    self.torch.cuda.current_stream().synchronize()
    cap = 64
    ms = np.zeros(cap)
    kind = np.zeros(cap, np.int32)
    count = C.c_int()
    check(self.lib.brx_profile_substep(self.h, float(dt), float(time), cap, _ptr(ms), _ptr(kind), C.byref(count)))
    if kinds:
        return [(int(kind[i]), float(ms[i])) for i in range(count.value)]
    return [(names[kind[i]], float(ms[i])) for i in range(count.value)]


def _shape(self, kind):
    """(block, blocks per SM, the kernel's largest block) of a kernel kind."""
    b, p, m = C.c_int(), C.c_int(), C.c_int()
    check(self.lib.brx_launch_shape_get(self.h, int(kind), C.byref(b), C.byref(p), C.byref(m)))
    return b.value, p.value, m.value


def _set_shape(self, kind, block, per_sm):
    check(self.lib.brx_launch_shape_set(self.h, int(kind), int(block), int(per_sm)))


def _set_tile(self, cells):
    """Cells per tile of the mixed f-wave tile sweep (0: the separate cell, face and gather sweeps)."""
    check(self.lib.brx_tile_set(self.h, int(cells)))


def _tile(self):
    """(cells per tile, shared memory bytes of the tile sweep); (0, 0) for the separate sweeps."""
    cells, smem = C.c_int(), C.c_int()
    check(self.lib.brx_tile_get(self.h, C.byref(cells), C.byref(smem)))
    return cells.value, smem.value


def _set_chunk(self, substeps):
    check(self.lib.brx_graph_chunk_set(self.h, int(substeps)))
    self.graph_chunk = int(substeps)


RiverSolver.profile_substep = _profile
RiverSolver.launch_shape = _shape
RiverSolver.set_launch_shape = _set_shape
RiverSolver.set_graph_chunk = _set_chunk
RiverSolver.set_tile = _set_tile
RiverSolver.tile = _tile
