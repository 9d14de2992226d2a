"""Python driver of the C oracle (``braids_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker. The product never
imports this module.

The library is compiled with FMA contraction disabled, matching the
reference's own CPU build flags (src/braids_support/sediment/
river_morphodynamics/sediment_wave.py:35, ``-ffp-contract=off``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "braids_oracle.c"
LIBRARY = HERE / "_build" / "libbraids_oracle.so"
FLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-std=c11"]


def build(force=False):
    """Compile the oracle (idempotent). Returns the library path."""
    LIBRARY.parent.mkdir(exist_ok=True)
    if force or not LIBRARY.exists() or LIBRARY.stat().st_mtime < SOURCE.stat().st_mtime:
        tmp = LIBRARY.with_suffix(".tmp.so")
        subprocess.run(["gcc", *FLAGS, str(SOURCE), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, LIBRARY)
    return LIBRARY


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _setup(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
D = C.c_double


class Ctx(C.Structure):
    _fields_ = [("nc", I), ("nf", I), ("nadj", I), ("nb", I),
                ("owner", P), ("neighbour", P), ("bid", P), ("bmode", P), ("offset", P), ("faces", P), ("signs", P),
                ("normal", P), ("length", P), ("area", P),
                ("ls_matrix", P), ("ls_weight", P), ("ls_delta", P),
                ("disp", P), ("disp_len", P), ("distance", P),
                ("boundary_offset", P), ("boundary_faces", P),
                ("grav", D), ("dry", D), ("cfl", D), ("speed_limit", D),
                ("roughness_mode", I), ("roughness_value", D),
                ("seg_mode", P), ("stage_policy", P), ("exterior_bed", P), ("forcing", P),
                ("table_len", I), ("table_time", P), ("table_value", P), ("threads", I),
                ("turb", P), ("rating_offset", P), ("rating_q", P), ("rating_eta", P),
                ("nchain", I), ("chain_offset", P), ("chain_face", P), ("chain_slope", P), ("weir", P),
                ("crit_seg_chain", P), ("crit_chain_offset", P), ("crit_chain_face", P),
                ("inlet_line", P), ("inlet_slope", P), ("line_left", P), ("line_right", P),
                ("visc", D), ("vdxdy", P), ("vinv", P), ("xy", P), ("vgrad", P), ("vface", P)]


class Turbines(C.Structure):
    _fields_ = [("nr", I), ("support_offset", P), ("support_cell", P), ("support_weight", P),
                ("support_density", P), ("plane_offset", P), ("plane_cell", P), ("plane_delta", P),
                ("param", P), ("curve", P), ("curve_x", P), ("curve_y", P), ("nu", P), ("pressure", I),
                ("dxdy", P), ("inverse", P), ("xy", P), ("mdisp", P), ("diag", P),
                ("grad", P), ("raw", P), ("face", P), ("work", P), ("trace", P), ("kcell", P), ("fstatus", P)]


class ExnerParams(C.Structure):
    _fields_ = [("diameter", D), ("porosity", D), ("chezy", D), ("morfac", D), ("sediment_depth", D),
                ("bedbc", P), ("feed", P), ("rock", P), ("dxdy", P), ("inverse", P), ("xy", P)]


class ExnerStats(C.Structure):
    _fields_ = [("ok", I), ("residual", D), ("boundary", D), ("donor", D), ("change", D)]


class HllcGeo(C.Structure):
    _fields_ = [("off", P), ("faces", P), ("signs", P), ("xy", P), ("mid", P), ("inverse", P), ("selected", P)]


class Stats(C.Structure):
    _fields_ = [("substeps", I), ("rejections", I), ("status", I),
                ("min_dt", D), ("max_dt", D), ("accepted_cfl_max", D), ("hint", D)]


def _setup(L):
    L.om_ctx_size.restype = C.c_size_t
    assert L.om_ctx_size() == C.sizeof(Ctx), "oracle context layout differs"
    L.om_stats_size.restype = C.c_size_t
    assert L.om_stats_size() == C.sizeof(Stats)
    L.om_scratch_create.restype = P
    L.om_scratch_create.argtypes = [P]
    L.om_scratch_destroy.argtypes = [P]
    L.om_fwave_face.argtypes = [P, D, D, P]
    L.om_fwave_face.restype = I
    for name in ("om_primitive", "om_cells", "om_faces", "om_prepare", "om_fwave", "om_assemble",
                 "om_gather", "om_limit_faces", "om_limit_gather"):
        getattr(L, name).restype = None
    L.om_exterior.restype = I
    L.om_exterior.argtypes = [P, P, P, D, P, P, P, P, P, P]
    L.om_outlet_feasibility.argtypes = [P, P, D, P, P, P]
    L.om_inlet_feasibility.argtypes = [P, P, D, P, P, P]
    L.om_inventory.argtypes = [P, D, P, P, P]
    L.om_reserve.argtypes = [P, D, P, P, P]
    L.om_reserve.restype = I
    L.om_frequency.restype = D
    L.om_drag.argtypes = [P, D, P]
    L.om_rate.argtypes = [P, P, P, P, P, D, D, P, P, P]
    L.om_rate.restype = I
    L.om_single.argtypes = [P, P, P, P, D, D, P, P, P, P]
    L.om_single.restype = I
    L.om_advance.argtypes = [P, P, P, D, D, P, P, P]
    L.om_advance.restype = I
    L.om_set_threads.argtypes = [I]
    L.om_sample_forcing.argtypes = [P, D]
    L.om_sample_forcing.restype = None
    L.om_turbines_size.restype = C.c_size_t
    assert L.om_turbines_size() == C.sizeof(Turbines), "oracle turbine layout differs"
    L.om_exner_size.restype = C.c_size_t
    assert L.om_exner_size() == C.sizeof(ExnerParams), "oracle bed-update layout differs"
    L.om_exner.argtypes = [P, P, P, P, D, P, P]
    L.om_exner.restype = I
    L.om_turbine_diagnose.argtypes = [P, P, P]
    L.om_shoreline_viscosity.argtypes = [P, P, P, P]
    L.om_shoreline_viscosity.restype = None
    L.om_turbine_diagnose.restype = I
    L.om_hkt_gradients.argtypes = [P, P, P, P, P]
    L.om_hkt_gradients.restype = None
    L.om_hllc_geo_size.restype = C.c_size_t
    assert L.om_hllc_geo_size() == C.sizeof(HllcGeo), "oracle HLLC geometry layout differs"
    L.om_hllc_advance.argtypes = [P, P, P, P, D, D, P, P, P]
    L.om_hllc_advance.restype = I
    L.om_hllc_step.argtypes = [P, P, P, P, D, D] + [P] * 12
    L.om_hllc_step.restype = I
    L.om_hllc_reconstruct.argtypes = [P, P, D, P, P, P, P, P, P]
    L.om_hllc_faces.argtypes = [P, P, P, P, P, P, P, P, P]
    L.om_hllc_budget.argtypes = [P, P, D, P, P, P, P, P, P]
    L.om_hllc_limit.argtypes = [P, P, P, P, P, P, P]
    L.om_hllc_update.argtypes = [P, P, D, P, P, P, P, P, P]
    L.om_hllc_turbine_pressure.argtypes = [P, P, P, P, P, P]
    L.om_hllc_predict_source.argtypes = [I, D, D, P, P, P]
    for name in ("om_hllc_reconstruct", "om_hllc_faces", "om_hllc_budget", "om_hllc_limit", "om_hllc_update",
                 "om_hllc_turbine_pressure", "om_hllc_predict_source"):
        getattr(L, name).restype = None


def _p(a):
    return a.ctypes.data_as(P) if a is not None else None


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """CPU oracle bound to one mesh, boundary set-up and control set.

    ``case`` is the dict produced by ``braids_hkt_gb300.scenarios`` (mesh
    arrays, records, boundary modes, forcing, controls).
    """

    def __init__(self, case, threads=None):
        self.L = lib()
        m = case["mesh"]
        r = m.records
        keep = self._keep = {}

        def k(name, arr):
            keep[name] = arr
            return _p(arr)
        nb = m.nb
        seg_mode = _i32(case["seg_mode"]) if nb else np.zeros(1, np.int32)
        bmode = np.zeros(m.nf, np.int32)
        if nb:
            openf = (m.neighbour < 0) & (m.bid >= 0)
            bmode[openf] = seg_mode[m.bid[openf]]
        self.forcing = _f64(case.get("forcing", np.zeros((2, max(nb, 1))))).copy()
        ctx = Ctx()
        ctx.nc, ctx.nf, ctx.nadj, ctx.nb = m.nc, m.nf, m.nadj, nb
        ctx.owner = k("owner", _i32(m.owner))
        ctx.neighbour = k("neighbour", _i32(m.neighbour))
        ctx.bid = k("bid", _i32(m.bid))
        ctx.bmode = k("bmode", bmode)
        ctx.offset = k("offset", _i32(m.offset))
        ctx.faces = k("faces", _i32(m.faces))
        ctx.signs = k("signs", _i32(m.signs))
        ctx.normal = k("normal", _f64(m.normal))
        ctx.length = k("length", _f64(m.length))
        ctx.area = k("area", _f64(m.area))
        ctx.ls_matrix = k("ls_matrix", _f64(r["ls_matrix"]))
        ctx.ls_weight = k("ls_weight", _f64(r["ls_weight"]))
        ctx.ls_delta = k("ls_delta", _f64(r["ls_delta"]))
        ctx.disp = k("disp", _f64(r["disp"]))
        ctx.disp_len = k("disp_len", _f64(r["disp_len"]))
        ctx.distance = k("distance", _f64(r["distance"]))
        ctx.boundary_offset = k("boundary_offset", _i32(m.boundary_offset))
        ctx.boundary_faces = k("boundary_faces", _i32(m.boundary_faces) if len(m.boundary_faces) else np.zeros(1, np.int32))
        c = case["controls"]
        ctx.grav, ctx.dry, ctx.cfl, ctx.speed_limit = c["grav"], c["dry"], c["cfl"], c["speed_limit"]
        ctx.roughness_mode, ctx.roughness_value = c["roughness_mode"], c["roughness_value"]
        ctx.seg_mode = k("seg_mode", seg_mode)
        ctx.stage_policy = k("stage_policy", _i32(case.get("stage_policy", np.zeros(max(nb, 1), np.int32))))
        ctx.exterior_bed = k("exterior_bed", _f64(case.get("exterior_bed", np.zeros(m.nf))))
        ctx.forcing = _p(self.forcing)
        tt = case.get("table_time")
        if tt is not None:
            ctx.table_len = len(tt)
            ctx.table_time = k("table_time", _f64(tt))
            ctx.table_value = k("table_value", _f64(case["table_value"]))
        ctx.threads = threads or 0
        if nb and np.any(seg_mode == 10):
            from braids_hkt_gb300.solver import normal_chains
            off, faces, slope = normal_chains([case])
            ctx.nchain = len(slope)
            ctx.chain_offset = k("chain_offset", _i32(off))
            ctx.chain_face = k("chain_face", _i32(faces))
            ctx.chain_slope = k("chain_slope", _f64(slope))
        if nb and np.any(seg_mode == 4):
            from braids_hkt_gb300.solver import critical_chains
            segc, off, faces = critical_chains([case])
            ctx.crit_seg_chain = k("crit_seg_chain", _i32(segc))
            ctx.crit_chain_offset = k("crit_chain_offset", _i32(off))
            ctx.crit_chain_face = k("crit_chain_face", _i32(faces))
        if nb and np.any(seg_mode == 5):
            from braids_hkt_gb300.solver import weir_parameters
            ctx.weir = k("weir", _f64(weir_parameters([case])))
        if case.get("inlet"):
            from braids_hkt_gb300.solver import inlet_lines
            kind, slope, left, right = inlet_lines([case])
            ctx.inlet_line = k("inlet_line", _i32(kind))
            ctx.inlet_slope = k("inlet_slope", _f64(slope))
            ctx.line_left = k("line_left", _i32(left))
            ctx.line_right = k("line_right", _i32(right))
        if case.get("rating"):
            from braids_hkt_gb300.solver import rating_tables
            off, rq, re_ = rating_tables([case])
            ctx.rating_offset = k("rating_offset", _i32(off))
            ctx.rating_q = k("rating_q", _f64(rq))
            ctx.rating_eta = k("rating_eta", _f64(re_))
        if case.get("viscosity", 0.0) > 0.0:
            # the wet-bank viscosity's least-squares metric (bend_methods_v1.py:100-128)
            from braids_hkt_gb300.turbines import flow_geometry
            delta, inverse, _ = flow_geometry(m)
            ctx.visc = float(case["viscosity"])
            ctx.vdxdy = k("vdxdy", _f64(delta))
            ctx.vinv = k("vinv", _f64(inverse))
            ctx.xy = k("xy", _f64(m.xy))
            ctx.vgrad = k("vgrad", np.zeros((4, m.nc)))
            ctx.vface = k("vface", np.zeros((2, m.nf)))
        self.turbines = None
        self.case_exner = case.get("exner")
        if case.get("turbines"):
            self._bind_turbines(case, k)
            ctx.turb = C.cast(C.pointer(self._turb), P)
        self.ctx = ctx
        self.cp = C.byref(ctx)
        self.m = m
        self.seg_mode = np.asarray(case["seg_mode"])
        self.z = _f64(case["z"]).copy()
        self.L.om_set_threads(threads or os.cpu_count() or 1)
        self._scratch = self.L.om_scratch_create(self.cp)
        self.hint = C.c_double(0.0)

    def _bind_turbines(self, case, k):
        """Rotor array of the case (the product's host-side geometry packing)."""
        from braids_hkt_gb300 import turbines as TB
        pk = TB.pack([case], [0])
        self.turbines = pk
        m = case["mesh"]
        nr, ns = pk["nrotor"], len(pk["support_cell"])
        t = Turbines()
        t.nr = nr
        for name in ("support_offset", "support_cell", "plane_offset", "plane_cell", "curve"):
            setattr(t, name, k("t_" + name, _i32(pk[name])))
        for name in ("support_weight", "support_density", "plane_delta", "param", "curve_x", "curve_y",
                     "dxdy", "inverse", "xy"):
            setattr(t, name, k("t_" + name, _f64(pk[name])))
        t.mdisp = k("t_mdisp", _f64(pk["mid_disp"]))
        t.nu = k("t_nu", _f64(pk["nu"])) if pk["nu"].any() else None
        t.pressure = 1
        self.diag = np.zeros((nr, TB.NDIAG))
        t.diag = k("t_diag", self.diag)
        t.grad = k("t_grad", np.zeros((10, m.nc)))
        t.raw = k("t_raw", np.zeros((3, m.nc)))
        t.face = k("t_face", np.zeros((2, m.nf)))
        t.work = k("t_work", np.zeros((3, m.nc)))
        t.trace = k("t_trace", np.zeros((10, m.nf)))
        t.kcell = k("t_kcell", np.zeros(max(ns, 1)))
        t.fstatus = k("t_fstatus", np.zeros(m.nf, np.int32))
        self._turb = t

    def sample_forcing(self, t):
        """Forcing (2, nb) at time t from the case's tables."""
        self.L.om_sample_forcing(self.cp, float(t))
        return self.forcing.copy()

    def exner(self, q, dt, z0=None):
        """One bed update of the accepted state q over dt: (status, z_trial, stats dict)."""
        from braids_hkt_gb300 import turbines as TB
        ex = self.case_exner
        if not hasattr(self, "_exner"):
            d, inv, _ = TB.flow_geometry(self.m)
            keep = self._keep
            keep.update(ex_bedbc=_i32(ex["bedbc"]), ex_feed=_f64(ex["feed"]), ex_rock=_f64(ex["rock"]),
                        ex_dxdy=_f64(d), ex_inv=_f64(inv), ex_xy=_f64(self.m.xy))
            p = ExnerParams(ex["diameter"], ex["porosity"], ex["chezy"], ex.get("morfac", 1.0), ex["sediment_depth"],
                            _p(keep["ex_bedbc"]), _p(keep["ex_feed"]), _p(keep["ex_rock"]), _p(keep["ex_dxdy"]),
                            _p(keep["ex_inv"]), _p(keep["ex_xy"]))
            self._exner = p
        q = _f64(q)
        z0 = self.z if z0 is None else _f64(z0)
        zt = np.zeros(self.m.nc)
        st = ExnerStats()
        code = self.L.om_exner(self.cp, C.byref(self._exner), _p(q), _p(z0), float(dt), _p(zt), C.byref(st))
        return code, zt, {f: getattr(st, f) for f, _ in ExnerStats._fields_}

    def turbine_pressure(self, on):
        """Switch the balanced-pressure correction (on by default with rotors)."""
        self._turb.pressure = int(bool(on))

    def diagnose(self, q):
        """Rotor diagnostics of state q: (error code, (nrotor, NDIAG) record)."""
        q = _f64(q)
        err = self.L.om_turbine_diagnose(self.cp, _p(q), _p(self.z))
        return err, self.diag.copy()

    def hkt_gradients(self, q):
        q = _f64(q)
        out = np.zeros((10, self.m.nc))
        self.L.om_hkt_gradients(self.cp, C.cast(C.pointer(self._turb), P), _p(q), _p(self.z), _p(out))
        return out

    def __del__(self):
        try:
            self.L.om_scratch_destroy(self._scratch)
        except Exception:
            pass

    # --- full steps ------------------------------------------------------
    def rate(self, q, dt, time=0.0, base=None):
        q = _f64(q)
        base = q if base is None else _f64(base)
        rate = np.zeros_like(q)
        water = np.zeros(self.m.nf)
        freq = C.c_double()
        st = self.L.om_rate(self.cp, self._scratch, _p(q), _p(self.z), _p(base), dt, time,
                            _p(rate), _p(water), C.byref(freq))
        return st, rate, water, freq.value

    def single(self, base, dt, time=0.0):
        base = _f64(base)
        nc, nf = self.m.nc, self.m.nf
        out = np.zeros_like(base)
        water = np.zeros(nf)
        peak = C.c_double()
        tmp = np.zeros(9 * nc + 2 * nf)
        st = self.L.om_single(self.cp, self._scratch, _p(base), _p(self.z), dt, time, _p(out), _p(water),
                              C.byref(peak), _p(tmp))
        return st, out, water, peak.value

    def advance(self, q, dt, time=0.0):
        """Advance q (3,nc) in place over an outer interval; returns (status, water_mean, stats dict)."""
        assert q.dtype == np.float64 and q.flags.c_contiguous
        water = np.zeros(self.m.nf)
        stats = Stats()
        st = self.L.om_advance(self.cp, _p(q), _p(self.z), dt, time, C.byref(self.hint), _p(water), C.byref(stats))
        return st, water, {f: getattr(stats, f) for f, _ in Stats._fields_}

    def viscosity_rate(self, q):
        """The wet-bank viscosity's momentum-rate increment (3, nc) of a state alone."""
        assert self.ctx.visc > 0.0
        q = _f64(q)
        rate = np.zeros_like(q)
        self.L.om_shoreline_viscosity(self.cp, _p(q), _p(self.z), _p(rate))
        return rate

    # --- HLLC / MUSCL-Hancock option ----------------------------------------
    def _hllc(self):
        if not hasattr(self, "_hgeo"):
            from braids_hkt_gb300.hllc import hllc_geometry
            g = hllc_geometry(self.m)
            keep = self._keep
            keep.update(h_off=_i32(g["offset"]), h_faces=_i32(g["faces"]), h_signs=_i32(g["signs"]),
                        h_xy=_f64(self.m.xy), h_mid=_f64(self.m.mid), h_inv=_f64(g["inverse"]),
                        h_sel=_i32(g["selected"]))
            self._hgeo = HllcGeo(*(_p(keep[k]) for k in ("h_off", "h_faces", "h_signs", "h_xy", "h_mid",
                                                           "h_inv", "h_sel")))
            self.hllc_hint = C.c_double(0.0)
        return C.byref(self._hgeo)

    def hllc_advance(self, q, dt, time=0.0):
        """HLLC (MUSCL-Hancock) interval: q (3,nc) advanced in place; (status, water_mean, stats)."""
        assert q.dtype == np.float64 and q.flags.c_contiguous
        G = self._hllc()
        water = np.zeros(self.m.nf)
        stats = Stats()
        st = self.L.om_hllc_advance(self.cp, G, _p(q), _p(self.z), dt, time, C.byref(self.hllc_hint), _p(water),
                                    C.byref(stats))
        return st, water, {f: getattr(stats, f) for f, _ in Stats._fields_}

    def hllc_step(self, q, dt, time=0.0):
        """One Hancock step from q: (status, result, water, frequency peak, internals dict)."""
        G = self._hllc()
        q = _f64(q)
        nc, nf = self.m.nc, self.m.nf
        o = dict(out=np.zeros((3, nc)), water=np.zeros(nf), grad=np.zeros((8, nc)), half=np.zeros((4, nc)),
                 qhalf=np.zeros((3, nc)), fl=np.zeros((3, nf)), fr=np.zeros((3, nf)), speed=np.zeros(nf),
                 theta=np.zeros(nc), freq=np.zeros(nc), next=np.zeros((3, nc)))
        peak = C.c_double()
        st = self.L.om_hllc_step(self.cp, G, _p(q), _p(self.z), dt, time, _p(o["out"]), _p(o["water"]),
                                 C.byref(peak), *(_p(o[k]) for k in ("grad", "half", "qhalf", "fl", "fr", "speed",
                                                                     "theta", "freq", "next")))
        return st, o["out"], o["water"], peak.value, o

    def hllc_kernels(self, q, dt, external=None, ext_trace=None, rotors=False):
        """reconstruct -> faces [-> rotor pressure] -> budget -> limit -> update on q (no exterior call)."""
        G = self._hllc()
        L, cp, m = self.L, self.cp, self.m
        q = _f64(q)
        nc, nf = m.nc, m.nf
        o = dict(grad=np.zeros((8, nc)), half=np.zeros((4, nc)), qhalf=np.zeros((3, nc)),
                 pstatus=np.zeros(nc, np.int32), fl=np.zeros((3, nf)), fr=np.zeros((3, nf)), speed=np.zeros(nf),
                 theta=np.zeros(nc), freq=np.zeros(nc), fstatus=np.zeros(nf, np.int32), next=np.zeros((3, nc)),
                 status=np.zeros(nc, np.int32))
        external = np.zeros((3, nf)) if external is None else _f64(external)
        ext_trace = np.zeros((3, nf)) if ext_trace is None else _f64(ext_trace)
        L.om_hllc_reconstruct(cp, G, dt, _p(q), _p(self.z), _p(o["grad"]), _p(o["half"]), _p(o["qhalf"]),
                              _p(o["pstatus"]))
        L.om_hllc_faces(cp, G, _p(o["half"]), _p(o["grad"]), _p(external), _p(ext_trace), _p(o["fl"]),
                        _p(o["fr"]), _p(o["speed"]))
        if rotors:
            L.om_hllc_turbine_pressure(cp, G, _p(o["half"]), _p(o["grad"]), _p(o["fl"]), _p(o["fr"]))
        o["fl_raw"], o["fr_raw"] = o["fl"].copy(), o["fr"].copy()
        L.om_hllc_budget(cp, G, dt, _p(q), _p(o["fl"]), _p(o["speed"]), _p(o["pstatus"]), _p(o["theta"]),
                         _p(o["freq"]))
        L.om_hllc_limit(cp, G, _p(q), _p(o["theta"]), _p(o["fl"]), _p(o["fr"]), _p(o["fstatus"]))
        L.om_hllc_update(cp, G, dt, _p(q), _p(o["fl"]), _p(o["fr"]), _p(o["fstatus"]), _p(o["next"]),
                         _p(o["status"]))
        return o

    def boundary_allocation(self, base, dt, flux, trace):
        """Stock-aware allocation of the open-boundary fluxes in place: the
        outlet cap, then the exact-discharge inlet allocation when mode-9
        segments exist (river_explicit_boundary_budget.py:37-39)."""
        m = self.m
        work = np.zeros(3 * m.nf + 3 * m.nc)
        base = _f64(base)
        assert flux.flags.c_contiguous and trace.flags.c_contiguous
        self.L.om_outlet_feasibility(self.cp, _p(base), float(dt), _p(flux), _p(trace), _p(work))
        if np.any(self.seg_mode == 9):
            self.L.om_inlet_feasibility(self.cp, _p(base), float(dt), _p(flux), _p(trace), _p(work))

    # --- single kernels (for pinning against the reference kernels) -------
    def kernels(self, q, z=None):
        """Run primitive -> cells -> faces -> prepare -> fwave -> assemble -> gather on q."""
        m, L, cp = self.m, self.L, self.cp
        q = _f64(q)
        z = self.z if z is None else _f64(z)
        nc, nf = m.nc, m.nf
        o = dict(v=np.zeros((4, nc)), active=np.zeros(nc, np.int32), pstatus=np.zeros(nc, np.int32),
                 grad=np.zeros((4, 2, nc)), constant=np.zeros(nc, np.int32),
                 trace=np.zeros((10, nf)), kind=np.zeros(nf, np.int32), rstatus=np.zeros(nf, np.int32),
                 local=np.zeros((8, nf)), closed=np.zeros(nf, np.int32), riemann=np.zeros((18, nf)),
                 astatus=np.zeros(nf, np.int32), fl=np.zeros((3, nf)), fr=np.zeros((3, nf)),
                 speed=np.zeros(nf), fstatus=np.zeros(nf, np.int32), rate=np.zeros((3, nc)))
        L.om_primitive(cp, _p(q), _p(z), _p(o["v"]), _p(o["active"]), _p(o["pstatus"]))
        L.om_cells(cp, _p(q), _p(o["v"]), _p(o["active"]), _p(o["grad"]), _p(o["constant"]))
        L.om_faces(cp, _p(q), _p(o["v"]), _p(o["grad"]), _p(o["constant"]), _p(o["trace"]), _p(o["kind"]), _p(o["rstatus"]))
        L.om_prepare(cp, _p(o["trace"]), _p(q), _p(z), _p(o["kind"]), _p(o["local"]), _p(o["closed"]))
        L.om_fwave(cp, _p(o["local"]), _p(o["riemann"]), _p(o["astatus"]))
        L.om_assemble(cp, _p(o["trace"]), _p(o["local"]), _p(o["riemann"]), _p(q), _p(z), _p(o["kind"]),
                      _p(o["constant"]), _p(o["closed"]), _p(o["fl"]), _p(o["fr"]), _p(o["speed"]), _p(o["fstatus"]))
        L.om_gather(cp, _p(q), _p(o["fl"]), _p(o["fr"]), _p(o["active"]), _p(o["rate"]))
        return o

    def fwave_face(self, states, grav, dry):
        """Augmented f-wave on independent faces: states (8,n) -> (outputs (18,n), status (n))."""
        states = _f64(states)
        n = states.shape[1]
        out = np.zeros((18, n))
        status = np.zeros(n, np.int32)
        col = np.zeros(8)
        res = np.zeros(18)
        for i in range(n):
            col[:] = states[:, i]
            status[i] = self.L.om_fwave_face(_p(col), grav, dry, _p(res))
            out[:, i] = res
        return out, status
