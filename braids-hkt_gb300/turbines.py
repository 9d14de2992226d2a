"""Rotor arrays: host-side geometry, validation and packing of the actuator-disk sink.

A rotor is a dict with the keys of the reference's turbine rows
(src/braids_core/sediment/river_turbine_flow.py:46-52,
river_turbine_thetis.py:90-149):

  name                          identifier reported with the diagnostics
  X, Y                          rotor centre [m]
  D                             rotor diameter [m]
  hub_elevation_m               fixed absolute hub elevation [m]
  minimum_bed_clearance_m       required gap between rotor bottom and bed [m]
  minimum_surface_clearance_m   required gap between rotor top and surface [m]
  control                       one of
      {"mode": "constant_ct", "thrust_coefficient": Ct, "power_coefficient": Cp or None}
      {"mode": "thetis_speed_table" | "incident_speed_table", "model_name": ...,
       "performance": [{"speed_m_s", "thrust_coefficient", "power_coefficient"}, ...]}
      {"mode": "incident_speed_curves", "model_name": ...,
       "thrust_curve": [{"speed_m_s", "thrust_coefficient"}, ...],
       "power_curve": [{"speed_m_s", "power_coefficient"}, ...]}
  nu                            ambient eddy viscosity [m2/s], shared by a
                                scenario's rotors (0: no ambient stress)

The source is Thetis' discrete turbine: a D-by-D axis-aligned bump
exp(2 - 1/(1-x^2) - 1/(1-y^2)) (x, y scaled to [-1, 1]) integrated exactly
over each cell's part of the footprint (river_turbine_geometry.py:27-60),
density = integral / ((D/2)^2 * 1.45661) (river_turbine_thetis.py:263).
The coverage gate samples the surface and bed where the rotor line x = X
crosses the cells (river_turbine_flow.py:69-76).

Everything here runs once per mesh; the per-stage work is in the CUDA
kernels (support sums, gate, Thetis cell terms, sink, balanced pressure).
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

MODES = {"constant_ct": 0, "thetis_speed_table": 1, "incident_speed_table": 2, "incident_speed_curves": 3}
# per-rotor parameter record (doubles)
P_D, P_HUB, P_BEDCLEAR, P_SURFCLEAR, P_TOL, P_MODE, P_CT, P_CP, P_N = range(9)
# diagnostic record fields (doubles per rotor)
DIAG_FIELDS = ("active", "reason", "minimum_coverage_margin_m", "minimum_bed_clearance_m",
               "local_velocity_m_s", "upstream_velocity_m_s", "mean_depth_m",
               "thrust_coefficient", "power_coefficient", "force_per_density_m4_s2",
               "useful_power_per_density_m5_s3", "hydraulic_power_removed_per_density_m5_s3",
               "minimum_surface_m", "maximum_bed_m", "error", "reserved")
NDIAG = len(DIAG_FIELDS)
REASONS = ("covered", "insufficient_depth", "bed_intersection", "insufficient_surface_clearance",
           "insufficient_bed_clearance", "dry_numerical_support", "reverse_flow", "no_incoming_flow",
           "below_cut_in_speed")
ERRORS = {1: "Thetis induction correction is outside its real domain: Ct*A exceeds rotor diameter "
             "times local water depth.",
          2: "Incident-speed device curves require a fully covered rotor (local depth at least D)."}
WATER_DENSITY = 1000.0     # kg/m3, the reference's output scaling of per-density quantities
BUMP_NORMALIZER = 1.45661  # Thetis' bump integral over [-1, 1]^2, as published


# ---------------------------------------------------------------------------
# Controls
# ---------------------------------------------------------------------------
def _number(v):
    return type(v) in (int, float) and math.isfinite(v)


def validate_control(control):
    """The reference's control checks (river_turbine_thetis.py:90-149)."""
    if not isinstance(control, dict):
        raise ValueError("Choose Thetis constant coefficients or a speed / Ct / Cp table.")
    c = dict(control)
    mode = c.get("mode")
    if mode == "constant_ct":
        if set(c) != {"mode", "thrust_coefficient", "power_coefficient"}:
            raise ValueError("Constant input requires Ct and Cp (null or zero selects Thetis ideal-disk Cp).")
        pairs = [(c["thrust_coefficient"], c["power_coefficient"])]
    elif mode == "incident_speed_curves":
        if set(c) != {"mode", "model_name", "thrust_curve", "power_curve"} or not str(c.get("model_name", "")).strip():
            raise ValueError("Name the device curves and supply separate thrust_curve and power_curve tables.")
        for key, field, label in (("thrust_curve", "thrust_coefficient", "Ct"), ("power_curve", "power_coefficient", "Cp")):
            rows = c[key]
            if not isinstance(rows, list) or len(rows) < 2:
                raise ValueError(f"{label} curve requires at least two speed / {label} rows.")
            speeds = []
            for row in rows:
                if not isinstance(row, dict) or set(row) != {"speed_m_s", field}:
                    raise ValueError(f"{label} rows require only speed_m_s and {field}.")
                u, value = row["speed_m_s"], row[field]
                if not _number(u) or u < 0:
                    raise ValueError(f"{label} speeds must be finite and nonnegative.")
                if not _number(value) or value < 0 or (value >= 1 if label == "Ct" else value > 1):
                    raise ValueError(f"{label} must satisfy " + ("0 <= Ct < 1." if label == "Ct" else "0 <= Cp <= 1."))
                speeds.append(u)
            if any(b <= a for a, b in zip(speeds, speeds[1:])):
                raise ValueError(f"{label} speeds must be strictly increasing.")
        if (c["power_curve"][0]["speed_m_s"] > c["thrust_curve"][0]["speed_m_s"]
                or c["power_curve"][-1]["speed_m_s"] < c["thrust_curve"][-1]["speed_m_s"]):
            raise ValueError("The Cp speed range must cover the entire Ct operating range.")
        pairs = []
    elif mode in ("thetis_speed_table", "incident_speed_table"):
        if set(c) != {"mode", "model_name", "performance"} or not str(c.get("model_name", "")).strip():
            raise ValueError("Name the turbine speed table and provide speed, Ct and Cp rows.")
        rows = c["performance"]
        if not isinstance(rows, list) or len(rows) < 2:
            raise ValueError("Thetis needs at least two speed / Ct / Cp rows.")
        speeds = []
        for r in rows:
            if not isinstance(r, dict) or set(r) != {"speed_m_s", "thrust_coefficient", "power_coefficient"}:
                raise ValueError("Each table row requires speed_m_s, thrust_coefficient and power_coefficient.")
            if not _number(r["speed_m_s"]) or r["speed_m_s"] < 0:
                raise ValueError("Table speeds must be finite and nonnegative.")
            speeds.append(r["speed_m_s"])
        if any(b <= a for a, b in zip(speeds, speeds[1:])):
            raise ValueError("Table speeds must be strictly increasing.")
        pairs = [(r["thrust_coefficient"], r["power_coefficient"]) for r in rows]
    else:
        raise ValueError("Choose constant Ct/Cp or an explicitly referenced speed / Ct / Cp table.")
    for ct, cp in pairs:
        if not _number(ct) or not 0 <= ct < 1:
            raise ValueError("Ct must be finite, with 0 <= Ct < 1.")
        if cp is None and mode == "constant_ct":
            continue
        if not _number(cp) or not 0 <= cp <= 1:
            raise ValueError("Cp must be finite and between 0 and 1.")
    if mode in ("incident_speed_table", "incident_speed_curves"):
        rows = _curve_rows(c, "thrust_coefficient")
        for left, right in zip(rows, rows[1:]):
            slope = (right["thrust_coefficient"] - left["thrust_coefficient"]) / (right["speed_m_s"] - left["speed_m_s"])
            for row in (left, right):
                root = math.sqrt(1 - math.pi / 4 * row["thrust_coefficient"])
                derivative = .5 * (1 + root) - row["speed_m_s"] * math.pi / 4 * slope / (4 * root)
                if derivative <= 0:
                    raise ValueError("Incident-speed Ct table gives a nonunique induction-corrected operating point.")
    return c


def _curve_rows(control, field):
    if control["mode"] == "incident_speed_curves":
        return control["thrust_curve" if field == "thrust_coefficient" else "power_curve"]
    return control["performance"]


def rated_power_curve(diameter, ct, cp0, rated_power_w, max_speed=10.0, points=64):
    """Incident-speed curves for a constant Ct and Cp(U) = min(Cp0, P_rated / (1/2 rho A U^3))."""
    area = math.pi * diameter ** 2 / 4
    speeds = np.linspace(0.0, max_speed, points)
    cps = [cp0 if u <= 0 else min(cp0, rated_power_w / (.5 * WATER_DENSITY * area * u ** 3)) for u in speeds]
    return {"mode": "incident_speed_curves", "model_name": f"constant Ct {ct}, rated {rated_power_w:g} W",
            "thrust_curve": [{"speed_m_s": float(u), "thrust_coefficient": float(ct)} for u in speeds],
            "power_curve": [{"speed_m_s": float(u), "power_coefficient": float(c)} for u, c in zip(speeds, cps)]}


# ---------------------------------------------------------------------------
# Footprint quadrature
# ---------------------------------------------------------------------------
@lru_cache(maxsize=8)
def _gauss(order):
    x, w = np.polynomial.legendre.leggauss(order)
    s = (x + 1) / 2
    w = w / 2
    s.setflags(write=False)
    w.setflags(write=False)
    return s, w


def triangle_bump(vertices, diameter, order):
    """Bump integral over one triangle (rotor-local coordinates), collapsed
    Gauss-Legendre (Duffy) rule of the given order in each direction."""
    s, w = _gauss(order)
    a, b, d = np.asarray(vertices, dtype=float)[:3]
    v = b - a
    t = d - a
    xy = a + s[:, None, None] * v + (1 - s[:, None, None]) * s[None, :, None] * t
    z = 2 * xy / diameter
    inside = np.all(abs(z) < 1, axis=2)
    value = np.zeros(inside.shape)
    zz = z[inside]
    value[inside] = np.exp(2 - 1 / (1 - zz[:, 0] ** 2) - 1 / (1 - zz[:, 1] ** 2))
    return abs(np.linalg.det(np.array([v, t]))) * np.sum(value * (1 - s)[:, None] * w[:, None] * w[None, :])


def _clip_square(poly, half):
    """Sutherland-Hodgman clip of a convex polygon to |x| <= half, |y| <= half."""
    for axis, sign in ((0, 1.0), (0, -1.0), (1, 1.0), (1, -1.0)):
        if len(poly) == 0:
            return poly
        out = []
        n = len(poly)
        for i in range(n):
            p, q = poly[i], poly[(i + 1) % n]
            fp, fq = sign * p[axis] - half, sign * q[axis] - half
            if fp <= 0:
                out.append(p)
            if (fp < 0 < fq) or (fq < 0 < fp):
                t = fp / (fp - fq)
                out.append(p + t * (q - p))
        poly = out
    return poly


def _area(poly):
    if len(poly) < 3:
        return 0.0
    x = np.array([p[0] for p in poly])
    y = np.array([p[1] for p in poly])
    return 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))


def bump_integrals(mesh, X, Y, D):
    """Per-cell integrals of the rotor bump over each cell's part of the D-by-D
    footprint (quadrature orders 16, 32, 64, 128 until two agree to 2e-12 D^2).

    Returns (cells, values). Raises if the cells do not cover the footprint or
    the integrals do not add up to the bump's own integral.
    """
    half = D / 2
    pts = mesh.points[mesh.tri] - np.array([X, Y])            # (nc, 3, 2) rotor-local
    lo, hi = pts.min(axis=1), pts.max(axis=1)
    cand = np.flatnonzero((hi[:, 0] > -half) & (lo[:, 0] < half) & (hi[:, 1] > -half) & (lo[:, 1] < half))
    cells, values = [], []
    area = 0.0
    for i in cand:
        poly = _clip_square([p for p in pts[i]], half)
        a = _area(poly)
        if a <= 0:
            continue
        area += a
        tris = [(poly[0], poly[k], poly[k + 1]) for k in range(1, len(poly) - 1)]
        previous = sum(triangle_bump(t, D, 16) for t in tris)
        for order in (32, 64, 128):
            value = sum(triangle_bump(t, D, order) for t in tris)
            if abs(value - previous) <= 2e-12 * D ** 2:
                break
            previous = value
        else:
            raise ValueError("Polygon bump quadrature did not converge")
        if value > 0:
            cells.append(int(i))
            values.append(value)
    if not math.isclose(area, D * D, rel_tol=1e-10, abs_tol=1e-13):
        raise ValueError("Turbine footprint intersects a wall or is not covered exactly")
    expected = bump_integral_1d() ** 2 * half * half
    total = float(np.sum(values))
    if abs(total - expected) > 1e-9 * expected:
        raise ValueError("Polygon partition changes the physical bump integral")
    return np.asarray(cells, dtype=np.int64), np.asarray(values)


@lru_cache(maxsize=1)
def bump_integral_1d():
    """Integral of exp(1 - 1/(1-s^2)) over (-1, 1)."""
    from scipy.integrate import quad
    return quad(lambda s: math.exp(1 - 1 / (1 - s * s)), -1., 1., epsabs=1e-13, epsrel=1e-13)[0]


def rotor_plane(mesh, X, Y, D):
    """Cells crossed by the rotor line x = X, |y - Y| <= D/2, with the
    displacement of both ends of each crossing from the cell centroid."""
    a = np.array([X, Y - D / 2])
    b = np.array([X, Y + D / 2])
    pts = mesh.points[mesh.tri]
    lo, hi = pts.min(axis=1), pts.max(axis=1)
    cand = np.flatnonzero((lo[:, 0] <= X) & (hi[:, 0] >= X) & (hi[:, 1] >= a[1]) & (lo[:, 1] <= b[1]))
    rows, disp = [], []
    for i in cand:
        # parametric clip of the segment a + t (b - a), t in [0, 1], to the CCW triangle
        t0, t1 = 0.0, 1.0
        tri = pts[i]
        dirv = b - a
        ok = True
        for k in range(3):
            p, q = tri[k], tri[(k + 1) % 3]
            e = q - p
            nrm = np.array([e[1], -e[0]])                 # outward normal of a CCW triangle
            num = np.dot(nrm, p - a)
            den = np.dot(nrm, dirv)
            if den == 0:
                if num < 0:
                    ok = False
                    break
                continue
            t = num / den
            if den > 0:
                t1 = min(t1, t)
            else:
                t0 = max(t0, t)
        if not ok or t1 - t0 <= 0:
            continue
        p0, p1 = a + t0 * dirv, a + t1 * dirv
        if np.hypot(*(p1 - p0)) <= 1e-12:
            continue
        for p in (p0, p1):
            rows.append(int(i))
            disp.append(p - mesh.xy[:, i])
    if not rows:
        raise ValueError("Rotor plane is not represented")
    return np.asarray(rows, dtype=np.int64), np.asarray(disp).T.copy()


def flow_geometry(mesh):
    """The unweighted least-squares metric of the flow engines
    (bend_methods_v1.py:100-128): centre offsets per CSR entry, the
    pseudo-inverse of sum d d^T / |d|^2 per cell, and face-midpoint
    displacements (owner x, y; neighbour x, y)."""
    nc, nadj = mesh.nc, mesh.nadj
    cell = np.repeat(np.arange(nc), np.diff(mesh.offset))
    f = mesh.faces
    other = np.where(mesh.signs < 0, mesh.owner[f], mesh.neighbour[f])
    has = other >= 0
    delta = np.zeros((2, nadj))
    delta[:, has] = mesh.xy[:, other[has]] - mesh.xy[:, cell[has]]
    rr = np.vecdot(delta.T, delta.T)      # d @ d as the reference forms it (numpy's dot, contracted)
    a = np.zeros((nc, 2, 2))
    outer = np.where(has, delta[:, None, :] * delta[None, :, :] / np.where(has, rr, 1.0), 0.0)   # (2, 2, nadj)
    for i in range(2):
        for j in range(2):
            a[:, i, j] = np.bincount(cell, weights=outer[i, j], minlength=nc)
    v = np.linalg.pinv(a)
    inverse = np.stack((v[:, 0, 0], v[:, 0, 1], v[:, 1, 1]))
    disp = np.zeros((4, mesh.nf))
    disp[:2] = mesh.mid - mesh.xy[:, mesh.owner]
    inside = mesh.neighbour >= 0
    disp[2:, inside] = mesh.mid[:, inside] - mesh.xy[:, mesh.neighbour[inside]]
    return delta, inverse, disp


# ---------------------------------------------------------------------------
# One scenario's rotor array
# ---------------------------------------------------------------------------
class RotorArray:
    """Packed geometry of one scenario's rotors (cell ids local to its mesh)."""

    def __init__(self, mesh, rows):
        if not rows:
            raise ValueError("empty rotor array")
        if len({float(r.get("nu", 0.0)) for r in rows}) != 1:
            raise ValueError("A turbine array requires one explicitly shared ambient viscosity.")
        self.rows = [dict(r) for r in rows]
        self.names = [str(r.get("name", i)) for i, r in enumerate(rows)]
        self.nu = float(rows[0].get("nu", 0.0))
        params, curves, cx, cy = [], [], [], []
        self.support, self.plane = [], []
        for r in rows:
            for key in ("X", "Y", "D", "hub_elevation_m", "minimum_bed_clearance_m", "minimum_surface_clearance_m"):
                if key not in r or not _number(r[key]):
                    raise ValueError(f"rotor {r.get('name')}: finite {key} required")
            if r["minimum_bed_clearance_m"] < 0 or r["minimum_surface_clearance_m"] < 0:
                raise ValueError("Explicit nonnegative turbine clearance limits required")
            control = validate_control(r["control"])
            D = float(r["D"])
            top, bottom = r["hub_elevation_m"] + D / 2, r["hub_elevation_m"] - D / 2
            tol = max(1e-9, 64 * np.finfo(float).eps * max(1., abs(top), abs(bottom)))
            mode = MODES[control["mode"]]
            ct = cp = 0.0
            if mode == 0:
                ct = float(control["thrust_coefficient"])
                cp = float(control["power_coefficient"] or .5 * ct * (1 + math.sqrt(1 - ct)))
            start = len(cx)
            trows = [] if mode == 0 else _curve_rows(control, "thrust_coefficient")
            prows = [] if mode == 0 else _curve_rows(control, "power_coefficient")
            cx += [float(t["speed_m_s"]) for t in trows]
            cy += [float(t["thrust_coefficient"]) for t in trows]
            pstart = len(cx)
            cx += [float(t["speed_m_s"]) for t in prows]
            cy += [float(t["power_coefficient"]) for t in prows]
            curves.append((start, len(trows), pstart, len(prows)))
            params.append((D, float(r["hub_elevation_m"]), float(r["minimum_bed_clearance_m"]),
                           float(r["minimum_surface_clearance_m"]), tol, float(mode), ct, cp))
            cells, values = bump_integrals(mesh, float(r["X"]), float(r["Y"]), D)
            # the footprint must be resolved across the rotor (river_turbine_flow.py:59-61)
            ext = np.ptp(mesh.points[mesh.tri[cells]][:, :, 1], axis=1)
            if np.any(ext > D * (1 + 1e-9)):
                raise ValueError("Merged turbine footprint is unresolved across the rotor; reduce the mesh size.")
            weight = values / values.sum()
            density = values / ((D / 2) ** 2 * BUMP_NORMALIZER)
            self.support.append((cells, weight, density))
            self.plane.append(rotor_plane(mesh, float(r["X"]), float(r["Y"]), D))
        self.param = np.asarray(params, dtype=np.float64)
        self.curve = np.asarray(curves, dtype=np.int32)
        self.curve_x = np.asarray(cx if cx else [0.0])
        self.curve_y = np.asarray(cy if cy else [0.0])


def pack(cases, cell_offsets):
    """Concatenate the rotor arrays of a batch (global cell ids). Returns None
    without rotors, else a dict of contiguous arrays for the C ABI."""
    arrays = [(i, case.get("_rotors") or (RotorArray(case["mesh"], case["turbines"]) if case.get("turbines") else None))
              for i, case in enumerate(cases)]
    for (i, ra), case in zip(arrays, cases):
        if ra is not None:
            case["_rotors"] = ra
    if not any(ra is not None for _, ra in arrays):
        return None
    scen, param, curve, cx, cy = [], [], [], [], []
    soff, scell, sw, sden = [0], [], [], []
    poff, pcell, pdx, pdy = [0], [], [], []
    dxdy, inverse, xy, mdisp, nu, hkt = [], [], [], [], [], []
    names = []
    for (i, ra), case in zip(arrays, cases):
        m = case["mesh"]
        base = int(cell_offsets[i])
        if ra is None:
            dxdy.append(np.zeros((2, m.nadj))); inverse.append(np.zeros((3, m.nc)))
            mdisp.append(np.zeros((4, m.nf))); xy.append(m.xy); nu.append(np.zeros(m.nc)); hkt.append(0)
            continue
        if getattr(ra, "flow", None) is None:
            ra.flow = flow_geometry(m)              # once per mesh (the rotor array travels with the case)
        d, inv, disp = ra.flow
        dxdy.append(d); inverse.append(inv); mdisp.append(disp); xy.append(m.xy)
        nu.append(np.full(m.nc, ra.nu)); hkt.append(1)
        shift = len(cx)
        for k in range(len(ra.rows)):
            scen.append(i)
            names.append(ra.names[k])
            param.append(ra.param[k])
            t0, tn, p0, pn = ra.curve[k]
            curve.append((t0 + shift, tn, p0 + shift, pn))
            cells, w, den = ra.support[k]
            scell.append(cells + base); sw.append(w); sden.append(den)
            soff.append(soff[-1] + len(cells))
            rows, disp2 = ra.plane[k]
            pcell.append(rows + base); pdx.append(disp2[0]); pdy.append(disp2[1])
            poff.append(poff[-1] + len(rows))
        cx.extend(ra.curve_x.tolist()); cy.extend(ra.curve_y.tolist())
    cat = np.concatenate
    return dict(
        nrotor=len(scen), names=names,
        scenario=np.asarray(scen, dtype=np.int32),
        param=np.ascontiguousarray(np.asarray(param, dtype=np.float64)),
        curve=np.ascontiguousarray(np.asarray(curve, dtype=np.int32)),
        curve_x=np.asarray(cx if cx else [0.0]), curve_y=np.asarray(cy if cy else [0.0]),
        support_offset=np.asarray(soff, dtype=np.int32), support_cell=cat(scell).astype(np.int32),
        support_weight=cat(sw), support_density=cat(sden),
        plane_offset=np.asarray(poff, dtype=np.int32), plane_cell=cat(pcell).astype(np.int32),
        plane_delta=np.ascontiguousarray(np.stack((cat(pdx), cat(pdy)))),
        dxdy=np.ascontiguousarray(cat(dxdy, axis=1)), inverse=np.ascontiguousarray(cat(inverse, axis=1)),
        xy=np.ascontiguousarray(cat(xy, axis=1)), mid_disp=np.ascontiguousarray(cat(mdisp, axis=1)),
        nu=cat(nu), hkt=np.asarray(hkt, dtype=np.int32))


def diagnostics_rows(diag, names, water_density=WATER_DENSITY):
    """Per-rotor dicts from a (nrotor, NDIAG) record, with the reference's
    output scaling to thrust [N] and power [W]."""
    out = []
    for k, name in enumerate(names):
        d = {f: float(diag[k, j]) for j, f in enumerate(DIAG_FIELDS)}
        d["turbine_id"] = name
        d["active"] = bool(d["active"])
        d["inactive_reason"] = None if d["active"] else REASONS[int(d["reason"])]
        d["thrust_N"] = d["force_per_density_m4_s2"] * water_density
        d["power_W"] = d["useful_power_per_density_m5_s3"] * water_density
        d["useful_power_W"] = d["power_W"]
        d["hydraulic_work_W"] = d["hydraulic_power_removed_per_density_m5_s3"] * water_density
        out.append(d)
    return out
