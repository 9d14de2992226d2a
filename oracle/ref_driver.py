"""Drive the reference's own host-compiled kernels (oracle/_ref) through one river step.

TEST INFRASTRUCTURE ONLY, and only where the reference checkout exists (it
generates golden fixtures and pins the C oracle). The kernel arithmetic is
the reference's compiled code; the orchestration between kernels restates
the reference's Python owners line by line:

  RiverMidpoint.rate, GPU branch       src/braids_core/sediment/river_midpoint.py:100-176
  RiverExplicit.rate/_single/advance   src/braids_core/sediment/river_explicit.py:63-154
  ExteriorBed.evaluate/apply_*         src/braids_core/sediment/river_exterior_bed.py:183-233
  Exner bed update (finish + bed_faces) src/braids_core/sediment/shoreline_solver.py:209-240,
                                       flow2dh_mobile_bed.py:101-129, bend_methods_v1.py:415-463,
                                       river_mpm.py:21-33, flow2dh_eh_operator.py:111-120
  turbine momentum (install.add)       src/braids_core/sediment/river_turbine_flow.py:222-239,
                                       with the reference's ThetisRotor.sample / cell_terms
                                       (river_turbine_thetis.py) run on numpy

The HLLC option runs the reference's own ``HLLCHydraulics`` class
(src/braids_core/hydraulics/hllc.py) unchanged; only its kernel engine is
pointed at the host build of the reference's hllc.h in oracle/_ref, and its
exterior, friction, rotor-momentum and rotor-pressure hooks are the ones its
river owner installs (river_hllc.py:14-55, river_turbines.py:27-51) over the
kernels above.

The stock-budget steps run the reference's own Python classes
(``OutletFeasibility`` and ``ExplicitBoundaryBudget``) on a minimal stand-in
owner that carries only the attributes they read.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
# the reference checkout: $BRAIDS_REFERENCE, else a `reference` folder beside this repository
REFERENCE = Path(os.environ.get("BRAIDS_REFERENCE") or HERE.parent.parent / "reference")


class Rejected(Exception):
    pass


class Fatal(Exception):
    """A failure the reference raises as an error, not a trial rejection."""


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def _arg(x):
    if isinstance(x, np.ndarray):
        assert x.flags.c_contiguous
        return _ptr(x)
    if isinstance(x, LL):
        return C.c_longlong(int(x))
    if isinstance(x, (int, np.integer)):
        return C.c_int(int(x))
    return C.c_double(float(x))


class LL(int):
    """Marks a ``long long`` kernel argument."""


class Ref:
    def __init__(self, case, threads=None):
        if not (REF / "libref_update.so").exists():
            raise FileNotFoundError("run oracle/ref_build.py first")
        sys.path.insert(0, str(REFERENCE / "src"))
        self.libs = {n: C.CDLL(str(REF / f"libref_{n}.so")) for n in
                     ("reconstruction", "update", "gather", "midpoint", "explicit", "exterior", "drag")}
        t = threads or os.cpu_count() or 1
        for n in ("midpoint", "explicit", "exterior", "drag"):
            self.libs[n].mobile_threads(C.c_int(t))
        m = case["mesh"]
        r = m.records
        self.case, self.m = case, m
        nc, nf, nadj = m.nc, m.nf, m.nadj
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        nb = m.nb
        self.nb = nb
        seg_mode = i32(case["seg_mode"]) if nb else np.zeros(1, np.int32)
        self.seg_mode = seg_mode
        openf = (m.neighbour < 0) & (m.bid >= 0)
        self.openf = openf
        self.open_idx = np.flatnonzero(openf)
        bmode = np.zeros(nf, np.int32)
        bmode[openf] = seg_mode[m.bid[openf]]
        c = case["controls"]
        self.grav, self.dry, self.cfl = c["grav"], c["dry"], c["cfl"]
        self.speed_limit = c["speed_limit"]
        self.rmode, self.rvalue = c["roughness_mode"], c["roughness_value"]
        self.g = dict(
            owner=i32(m.owner), neighbour=i32(m.neighbour), bid=i32(m.bid), boundary_mode=bmode,
            offset=i32(m.offset), faces=i32(m.faces), signs=i32(m.signs),
            xy=f64(m.xy), mid=f64(m.mid), normal=f64(m.normal), length=f64(m.length), area=f64(m.area),
            ls_matrix=f64(r["ls_matrix"]), ls_weight=f64(r["ls_weight"]), ls_delta=f64(r["ls_delta"]),
            displacement=f64(r["disp"]), distance=f64(r["distance"]),
            rectangle=np.zeros((2, nc)), weno=np.full((5, 2, nf), -1, np.int32),
            triangle=np.zeros(nc, np.int32), wall_ids=np.full((5, 2, nc), -1, np.int32),
            wall_kind=np.zeros((5, 2, nc), np.int32), stencil_normal=np.zeros((2, 5, 2, nc)),
            wall_slot=np.full((2, nf), -1, np.int32), wall_normal=np.zeros((2, nc)),
            wall_mean_distance=np.ones(nc), wall_box_center=np.zeros((2, nc)),
            sampled=np.zeros(nf, np.int32), bedoffset=np.zeros(nf),
            selected=i32(openf), bfaces=i32(m.boundary_faces) if len(m.boundary_faces) else np.zeros(1, np.int32),
            boffset=i32(m.boundary_offset))
        self.z = f64(case["z"]).copy()
        self.exterior_bed = f64(case.get("exterior_bed", np.zeros(nf)))
        self.forcing = f64(case.get("forcing", np.zeros((2, max(nb, 1))))).copy()
        self.stage_policy = i32(case.get("stage_policy", np.zeros(max(nb, 1), np.int32)))
        self.roughness = np.full(nc, self.rvalue)
        self.tiles = max(1, (int(np.max(np.diff(m.boundary_offset))) + 63) // 64) if nb else 1
        self.step_hint = None
        self.frequency_peak = 0.0
        if nb:
            self._budget = self._make_budget()
        self.rotors = None
        if case.get("turbines"):
            self._install_turbines(case)

    # -- rotor array: the reference's Thetis rotors on this mesh ----------------
    @staticmethod
    def _stub_shapely():
        """The turbine modules import shapely at module level for geometry set-up
        that is not exercised here (the footprint integrals come in packed)."""
        import types
        for name in ("shapely", "shapely.geometry", "shapely.strtree", "shapely.ops"):
            sys.modules.setdefault(name, types.ModuleType(name))
        g = sys.modules["shapely.geometry"]
        for attr in ("Polygon", "LineString", "box", "Point"):
            setattr(g, attr, getattr(g, attr, object))
        sys.modules["shapely"].constrained_delaunay_triangles = None
        sys.modules["shapely.strtree"].STRtree = object
        sys.modules["shapely.ops"].unary_union = None

    def _install_turbines(self, case):
        self._stub_shapely()
        from braids_core.sediment import river_turbine_thetis as T
        from braids_core.sediment.bend_methods_v1 import prepared_geometry
        from braids_hkt_gb300 import turbines as TB
        m = self.m
        data = dict(xy=m.xy, area=m.area, owner=m.owner, neighbour=m.neighbour, normal=m.normal,
                    length=m.length, mid=m.mid, offset=m.offset, faces=m.faces, signs=m.signs,
                    distance=m.records["distance"], bid=m.bid)
        self.pg = prepared_geometry(data)
        for n in ("hkt", "stress", "flow"):
            self.libs[n] = C.CDLL(str(REF / f"libref_{n}.so"))
        self.libs["hkt"].hkt_stress_threads(C.c_int(1))
        self.libs["stress"].hkt_stress_threads(C.c_int(1))
        self.libs["flow"].flow_threads(C.c_int(1))
        ra = TB.RotorArray(m, case["turbines"])
        rotors = []
        for k, row in enumerate(case["turbines"]):
            r = object.__new__(T.ThetisRotor)
            D = float(row["D"])
            r.xp, r.dry = np, self.dry
            r.c = dict(row, normal_xy=[1., 0.], ct=0., cp=0., control={"mode": "constant_ct"})
            r.minimum_bed_clearance = row["minimum_bed_clearance_m"]
            r.minimum_surface_clearance = row["minimum_surface_clearance_m"]
            r.top, r.bottom = row["hub_elevation_m"] + D / 2, row["hub_elevation_m"] - D / 2
            cells, weight, density = ra.support[k]
            r.weights = np.zeros(m.nc)
            r.weights[cells] = density * ((D / 2) ** 2 * 1.45661)
            r.normalized = np.zeros(m.nc)
            r.normalized[cells] = weight
            r.area = np.asarray(m.area, dtype=np.float64)
            r.ids = np.asarray(cells)
            r.normal = np.array([1., 0.])
            rows, disp = ra.plane[k]
            r.plane, r.delta = np.asarray(rows, dtype=np.int32), np.ascontiguousarray(disp)
            r.tolerance = max(1e-9, 64 * np.finfo(float).eps * max(1., abs(r.top), abs(r.bottom)))
            r.control = T.validate_control(row["control"])
            r.original = dict(row)
            r.density_integrals = np.zeros(m.nc)
            r.density_integrals[cells] = density
            rotors.append(r)
        self.rotors = rotors
        self.rotor_nu = float(case["turbines"][0].get("nu", 0.0))
        self.last_turbines = None
        self.hkt_pressure = True

    @staticmethod
    def _invoke(fn, *args):
        """Call a host kernel; the argument tuple (and any temporary arrays in
        it) stays referenced until the call returns."""
        fn.restype = None
        fn(*[_arg(a) for a in args])

    # -- conservative wet-bank viscosity, the reference's kernels ---------------
    def viscosity_momentum(self, q, nu, rate):
        """The add_momentum increment of the reference's wet-bank viscosity
        owner (shoreline_viscosity.py:57-72) for a state q: the safe state of
        secondary_vector_ops.safe, the flow engines' gradients
        (bend_methods_v1_kernels.h:23-39) on the reference's own prepared
        geometry (bend_methods_v1.prepared_geometry), shoreline_viscous_faces
        (shoreline_viscosity.h) and flow_momentum_gather with unit weights;
        rate[1:] gets the increment."""
        from braids_core.sediment.bend_methods_v1 import prepared_geometry
        from braids_core.sediment.secondary_vector_ops import safe as ref_safe
        m, g = self.m, self.g
        n, nf = m.nc, m.nf
        for name, fn in (("bend", "bend_threads"), ("visc", "mobile_threads"), ("flow", "flow_threads")):
            if name not in self.libs:
                self.libs[name] = C.CDLL(str(REF / f"libref_{name}.so"))
            getattr(self.libs[name], fn)(C.c_int(1))
        if not hasattr(self, "pg"):
            data = dict(xy=m.xy, area=m.area, owner=m.owner, neighbour=m.neighbour, normal=m.normal,
                        length=m.length, mid=m.mid, offset=m.offset, faces=m.faces, signs=m.signs,
                        distance=m.records["distance"], bid=m.bid)
            self.pg = prepared_geometry(data)
        pg = self.pg
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        q = f64(q)
        safe, _ = ref_safe(np, q, float(self.dry))
        grad = np.zeros((10, n))
        self._invoke(self.libs["bend"].gradients, n, f64(safe), self.z, np.zeros(n), np.zeros(n), pg["offset"],
                     pg["faces"], pg["owner"], pg["neighbour"], f64(pg["dxdy"]), f64(pg["inverse"]), grad)
        face = np.zeros((2, nf))
        self._invoke(self.libs["visc"].shoreline_viscous_faces, nf, n, float(nu), float(self.dry), q, self.z, grad,
                     g["owner"], g["neighbour"], g["normal"], f64(m.records["distance"]), f64(m.xy), face)
        self._momentum_gather(face, rate)
        return grad, face

    # -- Exner bed update with MPM transport, the reference's kernels -----------
    def exner(self, q, z0, dt):
        """One bed update over dt (ShorelinePhysics.finish with morphology):
        (z_trial, stats dict). Parameters come from case["exner"]."""
        from braids_core.sediment.bend_methods_v1 import prepared_geometry
        ex = self.case["exner"]
        m, g = self.m, self.g
        n, nf = m.nc, m.nf
        for name in ("mpm", "mobile", "bend", "slope"):
            if name not in self.libs:
                self.libs[name] = C.CDLL(str(REF / f"libref_{name}.so"))
        for name, fn in (("mpm", "mobile_threads"), ("mobile", "mobile_threads"), ("bend", "bend_threads")):
            getattr(self.libs[name], fn)(C.c_int(1))
        if not hasattr(self, "pg"):
            data = dict(xy=m.xy, area=m.area, owner=m.owner, neighbour=m.neighbour, normal=m.normal,
                        length=m.length, mid=m.mid, offset=m.offset, faces=m.faces, signs=m.signs,
                        distance=m.records["distance"], bid=m.bid)
            self.pg = prepared_geometry(data)
        pg = self.pg
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        d, phi = float(ex["diameter"]), 1.0 - float(ex["porosity"])
        dtm = float(dt) * float(ex.get("morfac", 1.0))
        z0 = f64(z0)
        rock = f64(ex["rock"])
        # division-safe state (secondary_vector_ops.safe) at the sediment depth
        q = f64(q)
        wet = q[0] > ex["sediment_depth"]
        safe = q.copy()
        safe[0] = np.where(wet, q[0], .001001)
        safe[1:] = np.where(wet, q[1:], 0.)
        hi = np.zeros(n)
        # single-grain mixture: D90 and hiding (river_mpm.h mixture)
        hiding, d90, mean = np.zeros(n), np.zeros(n), np.zeros(n)
        self._invoke(self.libs["mpm"].mixture, n, 1, 1, np.ones(n), np.array([d]), hiding, d90, mean)
        grad = np.zeros((10, n))
        self._invoke(self.libs["bend"].gradients, n, safe, z0, hi, np.zeros(n), pg["offset"], pg["faces"],
                     pg["owner"], pg["neighbour"], f64(pg["dxdy"]), f64(pg["inverse"]), grad)
        cell = np.zeros((6, n))
        self._invoke(self.libs["mpm"].mpm, n, d, safe, safe, np.full(n, float(ex["chezy"])), hi, d90, hiding, cell)
        face = np.zeros((10, nf))
        self._invoke(self.libs["mobile"].flow_bed_face_inputs, nf, n, d, safe, z0, cell, grad, g["owner"],
                     g["neighbour"], g["normal"], f64(m.records["distance"]), f64(m.xy), face)
        corrected = np.zeros((2, nf))
        status = np.zeros(nf, np.int32)
        self._invoke(self.libs["slope"].L_flow_bed_slope_direction, LL(nf), LL(nf), 3,
                     *[np.ascontiguousarray(face[k]) for k in range(10)],
                     0., 0., .85, .5, 0., 0., 1., .05, corrected[0], corrected[1], status)
        corrected = np.ascontiguousarray(corrected)
        if np.any(status):
            raise ValueError("Koch--Flokstra rejected face input")
        aux = np.zeros((3, nf))
        self._invoke(self.libs["mobile"].flow_bed_flux, nf, 2650., corrected, g["neighbour"], i32(ex["bedbc"]),
                     g["normal"], f64(ex["feed"]), aux)
        o, j = m.owner, m.neighbour
        active = wet[o] & np.where(j >= 0, wet[np.maximum(j, 0)], True)
        aux[2] *= active
        available = phi * (z0 - rock)
        factors = np.zeros(n)
        self._invoke(self.libs["bend"].donor_factors, n, nf, 2, dtm, available, aux, g["length"], g["area"],
                     g["offset"], g["faces"], g["signs"], factors)
        self._invoke(self.libs["bend"].limit_flux, nf, 2, g["owner"], g["neighbour"], factors, aux)
        donor = float(np.min(factors))
        integral = dtm * aux[2]
        rate = np.zeros(n)
        self._invoke(self.libs["bend"].divergence, n, nf, 2, aux, g["length"], g["area"], g["offset"], g["faces"],
                     g["signs"], rate)
        ztrial = z0 + (dtm / phi) * rate
        outside = (j < 0) & (m.bid >= 0)
        boundary = -np.sum(integral * m.length * outside)
        residual = np.sum(phi * (ztrial - z0) * m.area) - boundary
        change = float(np.max(np.abs(ztrial - z0) / np.maximum(q[0], ex["sediment_depth"])))
        ok = (np.all(np.isfinite(ztrial)) and not np.any(ztrial < rock - 1e-13) and abs(float(residual)) <= 1e-10
              and change <= .05)
        return ztrial, dict(ok=bool(ok), residual=float(residual), boundary=float(boundary), donor=donor,
                            change=change, flux=aux[2].copy(), cell=cell, face=face, corrected=corrected)

    def hkt_gradients(self, q, z=None):
        m = self.m
        z = self.z if z is None else np.ascontiguousarray(z)
        grad = np.zeros((10, m.nc))
        self._invoke(self.libs["hkt"].hkt_wet_gradients, *(m.nc, self.dry, np.ascontiguousarray(q), z, self.pg["offset"], self.pg["faces"],
                       self.pg["owner"], self.pg["neighbour"], np.ascontiguousarray(self.pg["dxdy"]),
                       np.ascontiguousarray(self.pg["inverse"]), grad))
        return grad

    def turbine_sample(self, q, grad=None):
        """Every rotor's reference sample: list of (diagnostic dict, k, u, v)."""
        grad = self.hkt_gradients(q) if grad is None else grad
        return [r.sample(np.ascontiguousarray(q), self.z, grad) for r in self.rotors]

    def _momentum_gather(self, face, rate):
        m, g = self.m, self.g
        work = np.zeros((3, m.nc))
        self._invoke(self.libs["flow"].flow_momentum_gather, *(m.nc, m.nf, np.ones(m.nc), face, g["offset"], g["faces"], g["signs"], g["length"],
                       g["area"], work))
        rate[1:] += work[1:]

    def turbine_momentum(self, q, o, rate):
        """The reference's add_momentum with a rotor array (river_turbine_flow.py:230-239)."""
        m, g = self.m, self.g
        q = np.ascontiguousarray(q)
        grad = self.hkt_gradients(q)
        face = np.zeros((2, m.nf))
        if self.rotor_nu > 0.:
            self._invoke(self.libs["stress"].hkt_full_strain_faces, *(m.nf, m.nc, self.dry, q, self.z, grad, np.full(m.nc, self.rotor_nu), g["owner"],
                           g["neighbour"], g["normal"], np.ascontiguousarray(m.records["distance"]),
                           np.ascontiguousarray(m.xy), face))
            self._momentum_gather(face, rate)
        raw = np.zeros((3, m.nc))
        samples = []
        for r in self.rotors:
            d, k, u, v = r.sample(q, self.z, grad)
            speed = np.hypot(u, v)
            raw[1, r.ids] -= k * speed * u
            raw[2, r.ids] -= k * speed * v
            samples.append((d, k))
        rate[1:] += raw[1:]
        self.last_turbines = dict(samples=samples, grad=grad, raw=raw)
        if self.hkt_pressure:
            trace = np.zeros((10, m.nf))
            self._invoke(self.libs["hkt"].hkt_surface_pack, *(m.nf, m.nc, np.ascontiguousarray(o["local"]), g["owner"], g["neighbour"],
                           np.ascontiguousarray(o["constant"], dtype=np.int32), trace))
            status = np.zeros(m.nf, np.int32)
            self._invoke(self.libs["hkt"].hkt_balanced_pressure, *(m.nf, m.nc, self.grav, self.dry, q, self.z, trace, grad, raw, g["owner"],
                           g["neighbour"], g["normal"], np.ascontiguousarray(m.records["distance"]),
                           np.ascontiguousarray(self.pg["displacement"]), face, status))
            self._momentum_gather(face, rate)
            self.last_turbines.update(trace=trace, pressure=face.copy(), pressure_status=status)

    # -- the reference's own stock-budget classes on a stand-in owner --------
    def _make_budget(self):
        from braids_core.sediment.river_explicit_boundary_budget import ExplicitBoundaryBudget
        m, g = self.m, self.g
        data = dict(boundary_faces=np.asarray(m.boundary_faces, np.int32), owner=g["owner"], bid=g["bid"])
        p = SimpleNamespace(g=dict(offset=g["offset"], faces=g["faces"], signs=g["signs"], length=g["length"],
                                   neighbour=g["neighbour"], bid=g["bid"], area=g["area"]))
        # the exact-discharge inlet owner's control (river_exterior_inlet.py:10-11): mode-9 segments
        inlet = (SimpleNamespace(control=(self.seg_mode[:self.nb] == 9).astype(np.int32))
                 if np.any(self.seg_mode[:self.nb] == 9) else None)
        ext = SimpleNamespace(xp=np, p=p, a=SimpleNamespace(data=data), inlet_compatibility=inlet, nb=self.nb,
                              hydraulic_mode=np.asarray(self.seg_mode[:self.nb], np.int32))
        self._ext_stub = ext
        return ExplicitBoundaryBudget(ext)

    def call(self, lib, name, count, *args, launch=False):
        fn = getattr(self.libs[lib], ("L_" if launch else "") + name)
        fn.restype = None
        pre = (C.c_longlong(int(count)),) if launch else ()
        fn(*pre, *map(_arg, args))

    # -- spatial kernels -----------------------------------------------------
    def kernels(self, q, boundary_trace=None):
        m, g = self.m, self.g
        nc, nf, nadj = m.nc, m.nf, m.nadj
        q = np.ascontiguousarray(q, dtype=np.float64)
        o = dict(v=np.zeros((4, nc)), active=np.zeros(nc, np.int32), pstatus=np.zeros(nc, np.int32),
                 grad=np.zeros((4, 2, nc)), constant=np.zeros(nc, np.int32), vlo=np.zeros((4, nc)),
                 vhi=np.zeros((4, nc)), wall_values=np.zeros((4, 4, nc)), wall_ready=np.zeros((4, nc), np.int32),
                 face_value=np.zeros((4, 2, nf)), trace=np.zeros((10, nf)), kind=np.zeros(nf, np.int32),
                 rstatus=np.zeros(nf, np.int32), local=np.zeros((8, nf)), closed=np.zeros(nf, np.int32),
                 riemann=np.zeros((18, nf)), astatus=np.zeros(nf, np.int32), fl=np.zeros((3, nf)),
                 fr=np.zeros((3, nf)), speed=np.zeros(nf), fstatus=np.zeros(nf, np.int32), rate=np.zeros((3, nc)))
        self.call("reconstruction", "reconstruction_primitive", nc, q, self.z, g["owner"], g["neighbour"], g["bid"],
                  g["offset"], g["faces"], g["signs"], LL(nc), self.dry, o["v"], o["active"], o["pstatus"], launch=True)
        self.call("reconstruction", "reconstruction_cells", nc, q, o["v"], g["xy"], g["mid"], g["normal"],
                  g["owner"], g["neighbour"], g["bid"], g["boundary_mode"], g["offset"], g["faces"], g["signs"],
                  o["active"], g["ls_matrix"], g["ls_weight"], g["ls_delta"], g["rectangle"], g["weno"],
                  g["displacement"], g["triangle"], g["wall_ids"], g["wall_kind"], g["stencil_normal"],
                  g["wall_slot"], g["wall_normal"], g["wall_mean_distance"], g["wall_box_center"],
                  LL(nc), LL(nf), LL(nadj), self.dry, self.grav, 1.0, 0,
                  o["grad"], o["vlo"], o["vhi"], o["wall_values"], o["wall_ready"], o["constant"], launch=True)
        bt = np.zeros((3, nf)) if boundary_trace is None else np.ascontiguousarray(boundary_trace)
        self.call("reconstruction", "reconstruction_faces", nf, q, o["v"], o["grad"], o["vlo"], o["vhi"],
                  o["wall_values"], o["wall_ready"], o["constant"], g["owner"], g["neighbour"], g["bid"],
                  g["wall_slot"], g["weno"], g["displacement"], bt, 0, LL(nc), LL(nf), self.dry,
                  o["face_value"], o["trace"], o["kind"], o["rstatus"], launch=True)
        if boundary_trace is not None:
            o["trace"][:3, self.open_idx] = bt[:, self.open_idx]
        self.faces_flux(q, o)
        self.call("gather", "implicit_full_rate_from_faces", nc, q, g["area"], g["length"], g["normal"],
                  o["fl"], o["fr"], g["offset"], g["faces"], g["signs"], o["active"], LL(nc), LL(nf),
                  self.grav, o["rate"], launch=True)
        return o

    def faces_flux(self, q, o):
        m, g = self.m, self.g
        nc, nf = m.nc, m.nf
        self.call("update", "resident_prepare_faces", nf, o["trace"], q, self.z, g["normal"], g["distance"],
                  g["owner"], g["neighbour"], o["kind"], LL(nc), LL(nf), self.grav, self.dry,
                  o["local"], o["closed"], launch=True)
        self.call("update", "augmented_fwave_local", nf, o["local"], LL(nf), self.grav, self.dry,
                  o["riemann"], o["astatus"], launch=True)
        self.call("update", "resident_assemble_flux", nf, o["trace"], o["local"], o["riemann"], q, self.z,
                  g["normal"], g["owner"], g["neighbour"], o["kind"], g["boundary_mode"], g["sampled"],
                  g["bedoffset"], o["constant"], o["closed"], LL(nc), LL(nf), self.grav, self.dry,
                  o["fl"], o["fr"], o["speed"], o["fstatus"], launch=True)

    def fwave(self, states):
        states = np.ascontiguousarray(states, dtype=np.float64)
        n = states.shape[1]
        out = np.zeros((18, n))
        status = np.zeros(n, np.int32)
        self.call("update", "augmented_fwave_local", n, states, LL(n), self.grav, self.dry, out, status, launch=True)
        return out, status

    # -- exterior boundary owner ----------------------------------------------
    def _reduce(self, values, fields, result):
        nb, nf, tiles = self.nb, self.m.nf, self.tiles
        n = nb * fields
        partial = np.zeros(n * tiles)
        self.call("exterior", "exterior_partial", 0, n * tiles, nf, nb, tiles, fields,
                  self.g["boffset"], self.g["bfaces"], values, partial)
        self.call("exterior", "exterior_totals", 0, n, tiles, partial, result)

    def exterior(self, q):
        m, g = self.m, self.g
        nf, n, nb = m.nf, m.nc, self.nb
        terms = np.zeros((2, nf))
        stage = np.zeros(2 * nb)
        weights = np.zeros(nf)
        total = np.zeros(nb)
        trace = np.zeros((3, nf))
        flux = np.zeros((3, nf))
        status = np.zeros(nf, np.int32)
        # reference lines of the critical / normal inlets (river_exterior_bed.py:199-200)
        if self.case.get("inlet"):
            self._inlet_lines()
        self.call("exterior", "exterior_stage_terms", 0, nf, n, self.dry, g["owner"], g["selected"], q, self.z,
                  g["length"], terms)
        self._reduce(terms, 2, stage)
        rmode = min(self.rmode, 3)
        self.call("exterior", "exterior_weights", 0, nf, n, nb, self.dry, self.grav, rmode, self.dry,
                  int(self.rmode == 4), g["owner"], g["bid"], g["selected"], self.seg_mode, q, self.z,
                  self.exterior_bed, g["length"], self.roughness, stage, self.forcing, weights)
        self._reduce(weights, 1, total)
        self.call("exterior", "exterior_flux", 0, nf, n, nb, self.grav, self.dry, self.speed_limit,
                  g["owner"], g["bid"], g["selected"], self.seg_mode, self.stage_policy, q, self.z,
                  self.exterior_bed, g["normal"], g["length"], self.forcing, weights, total, trace, flux, status)
        # section owners after exterior_flux (ExteriorBed.evaluate, river_exterior_bed.py:213-217)
        if np.any(self.seg_mode[:nb] == 9):
            self._compatible_inlet(q, trace, flux, status)
        if np.any(self.seg_mode[:nb] == 4):
            self._critical_outlet(q, trace, flux, status)
        if np.any(self.seg_mode[:nb] == 5):
            from braids_hkt_gb300.solver import weir_parameters
            if "ref_outlet" not in self.libs:
                self.libs["ref_outlet"] = C.CDLL(str(REF / "libref_outlet.so"))
                self.libs["ref_outlet"].mobile_threads(C.c_int(os.cpu_count() or 1))
            control = np.ascontiguousarray((self.seg_mode[:nb] == 5).astype(np.int32))
            sec = np.zeros(nb, np.int32)
            self.call("ref_outlet", "exterior_free_weir", 0, nf, n, nb, self.grav, self.dry, self.speed_limit, control,
                      weir_parameters([self.case]), g["boffset"], g["bfaces"], g["owner"], q, self.z, self.exterior_bed,
                      g["normal"], g["length"], np.zeros(nf, np.int32), np.zeros(nf), np.zeros(nb), np.zeros((3, nb)),
                      trace, flux, status, sec)
            if np.any(sec):
                raise Rejected("free-weir outlet has no admissible subcritical control")
        if np.any(self.seg_mode[:nb] == 10):
            from braids_core.sediment.river_boundary_components import connected_opening_chains
            if "ref_normal" not in self.libs:
                self.libs["ref_normal"] = C.CDLL(str(REF / "libref_normal.so"))
                self.libs["ref_normal"].mobile_threads(C.c_int(os.cpu_count() or 1))
            m = self.m
            data = dict(owner=m.owner, neighbour=m.neighbour, bid=m.bid, mid=m.mid, normal=m.normal, length=m.length)
            chains, slopes = [], []
            for b in range(nb):
                if self.seg_mode[b] == 10:
                    for chain in connected_opening_chains(data, b):
                        chains.append(chain)
                        slopes.append(self.case["outlet"][b]["bed_slope"])
            off = np.ascontiguousarray(np.cumsum([0] + [len(c) for c in chains]), dtype=np.int32)
            cf = np.ascontiguousarray([f for c in chains for f in c], dtype=np.int32)
            cnt = len(chains)
            sec, trans = np.zeros(cnt, np.int32), np.zeros(cnt, np.int32)
            self.call("ref_normal", "normal_outlet", 0, nf, n, cnt, self.grav, self.dry, self.speed_limit, int(self.rmode),
                      off, cf, g["owner"], q, self.z, self.exterior_bed, g["normal"], g["length"], self.roughness,
                      np.ascontiguousarray(slopes, dtype=np.float64), np.zeros(cnt), np.zeros((2, cnt)), trace, flux,
                      status, sec, trans)
            if np.any(sec):
                raise Rejected("normal-depth outlet has no admissible subcritical section root")
        if np.any(self.seg_mode[:nb] == 11):
            from braids_hkt_gb300.solver import rating_tables
            if "ref_rating" not in self.libs:
                self.libs["ref_rating"] = C.CDLL(str(REF / "libref_rating.so"))
                self.libs["ref_rating"].mobile_threads(C.c_int(os.cpu_count() or 1))
            off, rq, re_ = rating_tables([self.case])
            control = np.ascontiguousarray((self.seg_mode[:nb] == 11).astype(np.int32))
            sec = np.zeros(nb, np.int32)
            self.call("ref_rating", "rating_outlet", 0, nf, n, nb, self.grav, self.dry, self.speed_limit, control,
                      g["boffset"], g["bfaces"], g["owner"], q, self.z, self.exterior_bed, g["normal"], g["length"],
                      off, rq, re_, np.zeros(nb), np.zeros(nb), trace, flux, status, sec)
            if np.any(sec):
                raise Fatal("Q-H outlet has no admissible subcritical solution within the supplied curve")
        return trace, flux, status

    def _inlet_lines(self):
        """The reference's own CriticalSection and NormalSection owners
        (river_exterior_section.py, river_exterior_normal.py) on a stand-in
        exterior owner, their kernels the host builds of their headers."""
        from braids_core.sediment import river_exterior_section as RS
        from braids_core.sediment import river_exterior_normal as RN
        from braids_core.sediment.bend_methods_v1 import BendTrialRejected
        m, g, nb = self.m, self.g, self.nb
        if not hasattr(self, "_lines"):
            from braids_support.sediment.river_morphodynamics.sediment_wave import WaveEngine

            def make(lib):
                def engine(backend, threads, source=None, names=None):
                    e = WaveEngine.__new__(WaveEngine)
                    e.backend, e.threads = "cpu", threads
                    e.lib, e.fn = lib, {n: getattr(lib, n) for n in names}
                    for fn in e.fn.values():
                        fn.restype = None
                    e.identity = {}
                    return e
                return engine
            libs = {}
            for name in ("ref_section", "ref_section_normal"):
                libs[name] = C.CDLL(str(REF / f"lib{name}.so"))
                libs[name].mobile_threads(C.c_int(os.cpu_count() or 1))

            def normal_engine(backend, threads, source=None, names=None):
                lib = libs["ref_section" if Path(str(source)).name == "river_exterior_section.h" else "ref_section_normal"]
                return make(lib)(backend, threads, source, names)
            RS.WaveEngine = make(libs["ref_section"])
            RN.WaveEngine = normal_engine
            ns = SimpleNamespace
            from braids_core.sediment.river_roughness import KEYS
            method = {1: "roughness.chezy", 2: "roughness.manning"}.get(int(self.rmode), "roughness.white_colebrook")
            params = {KEYS[method]: float(self.rvalue)}
            if method == "roughness.white_colebrook":
                params["white_colebrook_relation"] = "flow_log_layer" if int(self.rmode) == 3 else "classical_2d"
            data = dict(owner=m.owner, neighbour=m.neighbour, bid=m.bid, mid=m.mid, normal=m.normal, length=m.length,
                        mode=self.seg_mode[:nb])
            p = ns(g=dict(bid=g["bid"], length=g["length"]), nf=m.nf, n=m.nc,
                   parameters=ns(gravity=self.grav, dry=self.dry), exterior_bed=self.exterior_bed,
                   flow=ns(threads=1), identity=dict(river_roughness=dict(method=method, parameters=params)))
            self._lines_ext = ns(p=p, xp=np, nb=nb, tiles=self.tiles, a=ns(backend="cpu", data=data),
                                 offset=g["boffset"], faces=g["bfaces"], selected=g["selected"], bedforms=None)
            methods = {"stage": "inlet.stage_discharge", "critical": "inlet.critical_discharge",
                       "normal": "inlet.normal_discharge"}
            controls = {}
            for b in range(nb):
                row = (self.case.get("inlet") or {}).get(b, {})
                if self.seg_mode[b] == 9:
                    controls[str(b)] = {"method": methods[row.get("line", "stage")]}
                    if row.get("line") == "normal":
                        controls[str(b)]["energy_slope"] = float(row["energy_slope"])
                else:
                    controls[str(b)] = {"method": "outlet.stage"}
            self._lines = []
            if any(v["method"] == "inlet.critical_discharge" for v in controls.values()):
                self._lines.append(RS.CriticalSection(self._lines_ext, controls))
            if any(v["method"] == "inlet.normal_discharge" for v in controls.values()):
                self._lines.append(RN.NormalSection(self._lines_ext, controls))
        self._lines_ext.forcing = self.forcing
        try:
            for owner in self._lines:
                owner.solve()
        except BendTrialRejected as exc:
            raise Rejected(str(exc))

    def _compatible_inlet(self, q, trace, flux, status):
        """The reference's own CompatibleInlet owner (river_exterior_inlet.py:7-38)
        on a stand-in exterior owner, its kernel the host build of river_exterior_inlet.h."""
        from braids_core.sediment import river_exterior_inlet as RI
        from braids_core.sediment.bend_methods_v1 import BendTrialRejected
        m, g, nb = self.m, self.g, self.nb
        if not hasattr(self, "_inlet"):
            from braids_support.sediment.river_morphodynamics.sediment_wave import WaveEngine
            lib = C.CDLL(str(REF / "libref_inlet.so"))
            lib.mobile_threads(C.c_int(os.cpu_count() or 1))

            def engine(backend, threads, source=None, names=None):
                e = WaveEngine.__new__(WaveEngine)
                e.backend, e.threads = "cpu", threads
                e.lib, e.fn = lib, {n: getattr(lib, n) for n in names}
                for fn in e.fn.values():
                    fn.restype = None
                e.identity = {}
                return e
            RI.WaveEngine = engine
            ns = SimpleNamespace
            p = ns(g=dict(owner=g["owner"], normal=g["normal"], length=g["length"]), nf=m.nf, n=m.nc,
                   parameters=ns(gravity=self.grav, dry=self.dry), exterior_bed=self.exterior_bed, flow=ns(threads=1))
            self._inlet_ext = ns(p=p, xp=np, nb=nb, a=ns(backend="cpu", data=dict(speed_limit=self.speed_limit)),
                                 offset=g["boffset"], faces=g["bfaces"])
            controls = {str(b): {"method": "inlet.stage_discharge" if self.seg_mode[b] == 9 else "outlet.stage"}
                        for b in range(nb)}
            self._inlet = RI.CompatibleInlet(self._inlet_ext, controls)
        e = self._inlet_ext
        e.forcing, e.trace, e.flux, e.status = self.forcing, trace, flux, status
        try:
            self._inlet.evaluate(np.ascontiguousarray(q), self.z)
        except BendTrialRejected as exc:
            raise Rejected(str(exc))

    def _critical_outlet(self, q, trace, flux, status):
        """The reference's own CriticalOutlet owner (river_exterior_outlet.py:10-72)
        on a stand-in exterior owner, its kernel the host build of river_exterior_outlet.h."""
        from braids_core.sediment import river_exterior_outlet as RO
        from braids_core.sediment.bend_methods_v1 import BendTrialRejected
        m, g, nb = self.m, self.g, self.nb
        if not hasattr(self, "_crit"):
            from braids_support.sediment.river_morphodynamics.sediment_wave import WaveEngine
            lib = C.CDLL(str(REF / "libref_outlet.so"))

            def engine(backend, threads, source=None, names=None):
                e = WaveEngine.__new__(WaveEngine)
                e.backend, e.threads = "cpu", threads
                e.lib, e.fn = lib, {n: getattr(lib, n) for n in names}
                for fn in e.fn.values():
                    fn.restype = None
                e.identity = {}
                return e
            RO.WaveEngine = engine
            ns = SimpleNamespace
            data = dict(owner=m.owner, neighbour=m.neighbour, bid=m.bid, mid=m.mid, normal=m.normal, length=m.length,
                        speed_limit=self.speed_limit)
            p = ns(g=dict(owner=g["owner"], normal=g["normal"], length=g["length"]), nf=m.nf, n=m.nc,
                   parameters=ns(gravity=self.grav, dry=self.dry), exterior_bed=self.exterior_bed, flow=ns(threads=1))
            self._crit_ext = ns(p=p, xp=np, nb=nb, a=ns(backend="cpu", data=data), offset=g["boffset"],
                                faces=g["bfaces"])
            controls = {str(b): {"method": "outlet.critical" if self.seg_mode[b] == 4 else "outlet.stage"}
                        for b in range(nb)}
            self._crit = RO.CriticalOutlet(self._crit_ext, controls)
        self._crit_ext.trace, self._crit_ext.flux, self._crit_ext.status = trace, flux, status
        try:
            self._crit.evaluate(np.ascontiguousarray(q), self.z)
        except BendTrialRejected as exc:
            raise Rejected(str(exc))

    # -- one spatial residual --------------------------------------------------
    def rate(self, q, dt, time, base):
        m, g = self.m, self.g
        n, nf = m.nc, m.nf
        q = np.ascontiguousarray(q)
        if not np.all(np.isfinite(q)) or np.any(q[0] < 0):
            raise Rejected("spatial")
        if self.nb:
            ext_trace, ext_flux, ext_status = self.exterior(q)
            if np.any(ext_status):
                raise Rejected("spatial")
            self._ext_stub.flux, self._ext_stub.trace = ext_flux, ext_trace
            self._budget.allocate(base, dt)
        else:
            ext_trace = np.zeros((3, nf))
            ext_flux = np.zeros((3, nf))
            ext_status = np.zeros(nf, np.int32)
        o = self.kernels(q, boundary_trace=ext_trace if self.nb else None)
        fl, fr = o["fl"], o["fr"]
        if self.nb:
            idx = self.open_idx
            fl[:, idx] = ext_flux[:, idx]
            fr[:, idx] = ext_flux[:, idx]
            o["fstatus"][idx] = ext_status[idx]
            # the gather ran inside kernels() before the exterior flux replaced the open faces: redo it
            o["rate"][:] = 0
            self.call("gather", "implicit_full_rate_from_faces", n, q, g["area"], g["length"], g["normal"],
                      fl, fr, g["offset"], g["faces"], g["signs"], o["active"], LL(n), LL(nf),
                      self.grav, o["rate"], launch=True)
        if any(np.any(o[k]) for k in ("pstatus", "rstatus", "astatus", "fstatus")):
            raise Rejected("spatial")
        rate = o["rate"]
        water = fl[0].copy()
        theta = np.ones(n)
        correction = np.zeros((2, nf))
        status = np.zeros(nf, np.int32)
        self.call("midpoint", "midpoint_inventory", 0, n, float(dt), base, g["area"], g["length"],
                  g["offset"], g["faces"], g["signs"], water, theta)
        saved = None
        limiter_bid = g["bid"]
        if self.nb:
            saved = self._budget.reserve(base, dt, water, theta)
            limiter_bid = np.ascontiguousarray(self._budget.limiter_bid, dtype=np.int32)
        self.call("midpoint", "midpoint_faces", 0, nf, n, self.dry, q, theta, g["owner"], g["neighbour"],
                  limiter_bid, water, correction, status)
        if self.nb:
            self._budget.restore(water, correction, saved)
        if np.any(status):
            raise Rejected("budget")
        self.call("midpoint", "midpoint_gather", 0, n, nf, g["area"], g["length"], g["offset"], g["faces"],
                  g["signs"], water, correction, rate)
        if self.rotors:
            self.turbine_momentum(q, o, rate)
        if not np.all(np.isfinite(rate)):
            raise Rejected("spatial")
        freq = np.zeros(n)
        mask = g["selected"] if self.nb else np.zeros(nf, np.int32)
        self.call("explicit", "explicit_frequency", 0, n, nf, self.grav, self.dry, q, o["speed"],
                  np.ascontiguousarray(ext_trace), mask, g["owner"], g["normal"], g["area"], g["length"],
                  g["offset"], g["faces"], freq)
        frequency = float(np.max(freq))
        self.frequency_peak = max(self.frequency_peak, frequency)
        if not np.isfinite(frequency) or dt * frequency > self.cfl * (1 + 1e-12):
            raise Rejected("cfl")
        return rate, water, frequency

    # -- HLLC / MUSCL-Hancock option: the reference's own operator ---------------
    def _hllc_engine(self, source, names):
        """A WaveEngine (sediment_wave.py:22-56) bound to the host build of ``source``."""
        from braids_support.sediment.river_morphodynamics.sediment_wave import WaveEngine
        lib = C.CDLL(str(REF / ("libref_hllc_turbines.so" if Path(source).name == "hllc_turbines.h"
                                else "libref_hllc.so")))
        e = WaveEngine.__new__(WaveEngine)
        e.backend, e.threads = "cpu", os.cpu_count() or 1
        e.lib, e.fn = lib, {name: getattr(lib, name) for name in names}
        for fn in e.fn.values():
            fn.restype = None
        e.identity = dict(backend="cpu", source=str(source))
        return e

    def hllc_operator(self, cfl=None):
        """The reference's HLLCHydraulics on this mesh, hooked as RiverHLLC / the
        HLLC rotor install hook it (river_hllc.py:14-55, river_turbines.py:27-51)."""
        from braids_core.hydraulics import hllc as H
        from braids_core.hydraulics.outlet_feasibility import OutletFeasibility
        from braids_core.sediment.bend_methods_v1 import BendTrialRejected
        m, g = self.m, self.g
        H.WaveEngine = lambda backend, threads, source=None, names=None: self._hllc_engine(source, names)
        inlet = {6, 9}
        cells = [SimpleNamespace(centroid_xy=(float(m.xy[0, i]), float(m.xy[1, i])), area_m2=float(m.area[i]))
                 for i in range(m.nc)]
        faces = []
        for f in range(m.nf):
            mid = (float(m.mid[0, f]), float(m.mid[1, f]))   # (mid + mid) / 2 == mid exactly
            kind = "interior" if m.neighbour[f] >= 0 else "wall"
            if self.openf[f]:
                kind = "inlet" if int(self.seg_mode[m.bid[f]]) in inlet else "outlet"
            faces.append(SimpleNamespace(start_xy=np.array(mid), end_xy=np.array(mid),
                                         outward_normal=(float(m.normal[0, f]), float(m.normal[1, f])),
                                         owner=int(m.owner[f]), neighbour=int(m.neighbour[f]),
                                         length_m=float(m.length[f]), kind=kind))
        mesh = SimpleNamespace(cells=cells, faces=faces)

        def exterior(q, z, time):
            trace, flux, status = self.exterior(np.ascontiguousarray(q))
            if np.any(status):
                raise BendTrialRejected("Exterior hydraulic boundary rejected")
            return flux, trace
        feasibility = OutletFeasibility(self._ext_stub) if self.nb else None
        inlet_feasibility = None
        if self.nb and self._ext_stub.inlet_compatibility is not None:
            from braids_core.hydraulics.inlet_feasibility import InletFeasibility
            inlet_feasibility = InletFeasibility(self._ext_stub)

        def boundary_correction(q, dt, flux, trace):
            # feasible_boundary (river_hllc.py:31-33): outlet allocation, then inlet allocation
            feasibility(q, dt, flux, trace)
            if inlet_feasibility is not None:
                inlet_feasibility(q, dt, flux, trace)

        momentum = correct = None
        if self.rotors:
            def momentum(q, water, rate):
                saved, self.hkt_pressure = self.hkt_pressure, False
                try:
                    self.turbine_momentum(q, None, rate)
                finally:
                    self.hkt_pressure = saved
            pressure = self._hllc_engine("hllc_turbines.h", ("hllc_turbine_pressure",))

            def correct(op):
                k = op.g
                pressure.launch("hllc_turbine_pressure", op.nf, op.n, op.nf, op.gravity, op.dry, op.half, op.grad,
                                k["xy"], k["mid"], k["normal"], k["owner"], k["neighbour"], op.fl, op.fr)
        return H.HLLCHydraulics(mesh, backend="cpu", threads=os.cpu_count() or 1, gravity=self.grav, dry=self.dry,
                                cfl=self.cfl if cfl is None else cfl, exterior=exterior if self.nb else None,
                                friction=self.friction, check=None, integration="hancock", momentum=momentum,
                                boundary_correction=boundary_correction if self.nb else None,
                                face_correction=correct)

    def friction(self, q, dt):
        chezy = np.zeros(self.m.nc)
        comps = np.zeros(1)
        self.call("drag", "river_cell_drag", 0, self.m.nc, float(dt), self.grav, self.dry, self.rmode,
                  self.rvalue, 0, comps, q, chezy)

    def single(self, base, dt, time):
        dry = self.dry
        work = base.copy()
        self.frequency_peak = 0.0
        self.friction(work, .5 * dt)
        r, w, _ = self.rate(work, dt, time, work)
        q1 = work + dt * r
        if np.any(q1[0] < 0):
            raise Rejected("spatial")
        q1[1:, q1[0] <= dry] = 0.
        q1 = np.ascontiguousarray(q1)
        r2, w2, _ = self.rate(q1, dt, time + dt, q1)
        q2 = .5 * work + .5 * (q1 + dt * r2)
        if not np.all(np.isfinite(q2)) or np.any(q2[0] < 0):
            raise Rejected("spatial")
        q2[1:, q2[0] <= dry] = 0.
        q2 = np.ascontiguousarray(q2)
        self.friction(q2, .5 * dt)
        return q2, .5 * (w + w2), self.frequency_peak

    def advance(self, base, dt, time):
        q = base
        water = None
        used, rejected, freqs = [], [], []
        elapsed = 0.
        floor = dt * 2 ** -20
        hint = dt if self.step_hint is None else self.step_hint
        while not used or elapsed < dt - 1e-13 * max(1., dt):
            trial = min(hint, dt - elapsed)
            truncated = trial < hint * (1 - 1e-12)
            try:
                nextq, w, frequency = self.single(q, trial, time + elapsed)
            except Rejected:
                rejected.append(trial)
                hint = min(.5 * trial, .98 * self.cfl / self.frequency_peak) if self.frequency_peak > 0 else .5 * trial
                if hint < floor or len(rejected) > 100:
                    raise
                continue
            q = nextq
            water = trial * w if water is None else water + trial * w
            elapsed += trial
            used.append(trial)
            freqs.append(trial * frequency)
            growth = hint if truncated else 2 * trial
            hint = min(growth, .98 * self.cfl / frequency) if frequency > 0 else growth
            if len(used) > 4096:
                raise Rejected("limit")
        self.step_hint = float(hint)
        return q, water / dt, dict(substeps=len(used), rejections=len(rejected), min_dt=min(used),
                                   max_dt=max(used), accepted_cfl_max=max(freqs), hint=self.step_hint)
