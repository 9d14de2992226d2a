"""Seeded synthetic river scenarios: mesh, bed, initial state, boundaries, controls.

Every scenario is a plain dict ("case") that both the CUDA solver and the CPU
oracle consume:

  mesh          Mesh (topology, geometry records)
  z             (nc,) bed elevation
  q             (3,nc) initial h, hu, hv
  seg_mode      (nb,) hydraulic mode per open segment (2 stage, 6 total Q)
  stage_policy  (nb,) 0 outflow only, 1 subcritical backflow
  forcing       (2,nb) row 0 discharge Q [m3/s], row 1 stage [m]
  exterior_bed  (nf,) exterior bed elevation on open faces (0 elsewhere)
  controls      dict(grav, dry, cfl, speed_limit, roughness_mode, roughness_value)
  turbines      list of rotor dicts (optional)

Constants follow the reference's physical parameters: g = 9.81, dry = 1e-6
(src/braids_core/sediment/bend_methods_v1.py:64-66), speed limit 50 m/s
(src/braids_core/sediment/river_exterior_bed.py:210).
"""
from __future__ import annotations

import numpy as np

from . import mesh as M

GRAVITY = 9.81
DRY = 1e-6
SPEED_LIMIT = 50.0


def controls(cfl=0.9, manning=0.03):
    return dict(grav=GRAVITY, dry=DRY, cfl=float(cfl), speed_limit=SPEED_LIMIT,
                roughness_mode=2, roughness_value=float(manning))


def _exterior_bed(mesh, z):
    """Exterior bed on open faces = owner cell bed (no artificial step)."""
    ext = np.zeros(mesh.nf)
    openf = (mesh.neighbour < 0) & (mesh.bid >= 0)
    ext[openf] = z[mesh.owner[openf]]
    return ext


def channel(length=2000.0, width=200.0, spacing=4.0, jitter=1.0, seed=1, sigma=0.2, corr=25.0,
            slope=1e-3, outlet_bed=-5.0, stage=3.0, discharge=400.0, manning=0.03, cfl=0.9,
            refine=(), field_resolution=1.0, apron=3.0):
    """Straight channel of the 50k-cell class: jittered-grid Delaunay, sloped bed + Gaussian field.

    Lake at rest at ``stage``; inflow ``discharge`` (mode 6, conveyance
    weighted) at x=0, stage outlet (mode 2) at x=L. The bed datum puts the
    outlet bed at ``outlet_bed`` so a 5 m rotor is covered.

    The last ``apron`` grid spacings before the outlet are a flat bed at
    ``outlet_bed``. The reconstruction lets a subcritical stage outlet keep its
    cell's bed slope towards the outlet face (the face is left out of the
    limiter); on jittered triangles with a sloping bed that leaves an
    odd-even transverse mode of the outlet cells undamped, which grows from
    round-off within seconds even in a lake at rest. On a flat apron the bed
    gradient there is zero and the outlet is stable.
    """
    mesh = M.channel_mesh(length, width, spacing, jitter, seed, refine)
    rng = np.random.default_rng(seed + 1000003)
    grid = M.gaussian_field(length, width, sigma, corr, rng, field_resolution) if sigma > 0 else None
    x, y = mesh.xy
    z = outlet_bed + slope * (length - x)
    if grid is not None:
        z = z + M.sample_field(grid, x, y)
    if apron > 0:
        z = np.where(x > length - apron * spacing, outlet_bed, z)
    z = np.ascontiguousarray(z)
    h = np.maximum(stage - z, 0.0)
    q = np.ascontiguousarray(np.stack((h, np.zeros_like(h), np.zeros_like(h))))
    return dict(mesh=mesh, z=z, q=q,
                seg_mode=np.array([M.MODE_TOTAL_Q, M.MODE_STAGE], np.int32),
                stage_policy=np.zeros(2, np.int32),
                forcing=np.array([[discharge, 0.0], [0.0, stage]]),
                exterior_bed=_exterior_bed(mesh, z),
                controls=controls(cfl, manning), name=f"channel_{length:g}x{width:g}_s{spacing:g}")


def config1(seed=1):
    """Plain method, straight channel 2000 m x 200 m, 4 m jittered grid, about 50k triangles."""
    return channel(seed=seed)


def rotor_rows(case, centres, diameter=5.0, control=None, bed_clearance=0.5, surface_clearance=0.5, nu=0.0):
    """Rotor dicts at the given centres with the hub fixed D/2 + bed_clearance
    above the highest bed in each footprint (the reference's explicit fixed
    hub elevation and clearance limits, river_turbine_flow.py:46-52)."""
    from . import turbines as TB
    mesh, z = case["mesh"], case["z"]
    control = control or {"mode": "constant_ct", "thrust_coefficient": 0.8, "power_coefficient": None}
    rows = []
    for k, (x, y) in enumerate(centres):
        cells, _ = TB.bump_integrals(mesh, x, y, diameter)
        hub = float(np.max(z[cells])) + bed_clearance + 0.5 * diameter + 0.25
        rows.append(dict(name=f"T{k + 1}", X=float(x), Y=float(y), D=float(diameter), hub_elevation_m=round(hub, 3),
                         minimum_bed_clearance_m=0.2, minimum_surface_clearance_m=float(surface_clearance),
                         control=control, nu=float(nu)))
    return rows


def config2(seed=2, refine_spacing=1.0, control=None):
    """Config-1 channel with 3 tandem rotors on the centreline 150 m apart and
    the mesh refined to 1 m across the channel from 5 m upstream to 60 m
    downstream of each rotor (about 120k cells).

    Rotors: D = 5 m, Ct = 0.8 with Cp(U) = min(0.4, 500 kW / (1/2 rho A U^3))
    referenced to the incident speed (rated near 5.0 m/s), hub 0.75 m above
    D/2 over the highest bed in the footprint.
    """
    from . import turbines as TB
    length, width = 2000.0, 200.0
    xs = [700.0, 850.0, 1000.0]
    boxes = [(x - 5.0, x + 60.0, 0.0, width, refine_spacing) for x in xs]
    case = channel(length, width, seed=seed, refine=boxes)
    control = control or TB.rated_power_curve(5.0, 0.8, 0.4, 500e3)
    case["turbines"] = rotor_rows(case, [(x, 0.5 * width) for x in xs], control=control)
    case["name"] = "channel_3_rotors"
    return case


def small_rotor_channel(length=150.0, width=30.0, spacing=1.5, seed=21, discharge=150.0, rotors=2, control=None,
                        nu=0.0, sigma=0.1, corr=6.0):
    """A 150 m x 30 m channel resolved for 5 m rotors (about 4k cells) with
    ``rotors`` rotors on the centreline, 40 m apart, starting in uniform flow."""
    case = channel(length=length, width=width, spacing=spacing, jitter=0.25 * spacing, seed=seed, sigma=sigma,
                   corr=corr, discharge=discharge, field_resolution=min(1.0, spacing))
    q = case["q"]
    q[1] = np.where(q[0] > 0.0, discharge / width, 0.0)
    xs = [50.0 + 40.0 * k for k in range(rotors)]
    case["turbines"] = rotor_rows(case, [(x, 0.5 * width) for x in xs], control=control, nu=nu)
    case["name"] = "small_rotor_channel"
    return case


def config3(length=10000.0, width=1500.0, spacing=3.87, channels=5, seed=3, amplitude=200.0,
            channel_depth=(2.0, 4.0), sigma=0.5, corr=50.0, slope=1e-3, rotors=12, rotor_d=2.0,
            q_low=200.0, q_high=2000.0, rise_s=3600.0, stage_above=0.5, grain=0.02):
    """Braided river (config 3): ``channels`` seeded sinuous channels
    (amplitude ``amplitude`` m, depth U(channel_depth)) cut into a floodplain
    of slope ``slope`` carrying a Gaussian field (sigma, corr), stage outlet
    ``stage_above`` m over the floodplain at the outlet (extensive wet/dry),
    inlet hydrograph q_low -> q_high m3/s over rise_s seconds (forcing
    table), MPM bed update (d50 = grain, porosity 0.4) and ``rotors``
    staggered rotors of diameter rotor_d on the deepest channels, their
    footprints refined. The full size (10 km x 1.5 km, 3.87 m) is about 2M
    triangles; tests use a scaled-down copy."""
    rng = np.random.default_rng(seed)
    ys = (np.arange(channels) + 1.0) / (channels + 1.0) * width
    wl = rng.uniform(0.8, 1.6, channels) * 10.0 * width / 1.5 / channels * 1.5   # meander wavelengths
    phase = rng.uniform(0.0, 2 * np.pi, channels)
    half = rng.uniform(0.02, 0.04, channels) * width
    depth = rng.uniform(channel_depth[0], channel_depth[1], channels)
    amp = amplitude * width / 1500.0

    def centre(k, x):
        return ys[k] + amp * np.sin(2 * np.pi * x / wl[k] + phase[k])

    # rotors: staggered along the deepest channels, away from the ends
    order = np.argsort(-depth)
    centres = []
    for j in range(rotors):
        k = int(order[j % max(1, min(channels, 3))])
        x = length * (0.3 + 0.5 * (j + 0.5) / rotors)
        centres.append((float(x), float(centre(k, x))))
    fine = min(spacing, 0.35 * rotor_d)
    boxes = [(x - 3 * rotor_d, x + 3 * rotor_d, y - 3 * rotor_d, y + 3 * rotor_d, fine) for x, y in centres]
    mesh = M.channel_mesh(length, width, spacing, 0.25 * spacing, seed, refine=boxes)
    grid = M.gaussian_field(length, width, sigma, corr, rng, min(spacing, 5.0))
    x, y = mesh.xy
    floodplain = slope * (length - x) + M.sample_field(grid, x, y)
    cut = np.zeros_like(x)
    for k in range(channels):
        d = np.abs(y - centre(k, x))
        cut = np.maximum(cut, depth[k] * np.clip(1.0 - (d / half[k]) ** 2, 0.0, None))
    z = floodplain - cut
    apron = x > length - 3 * spacing
    z = np.where(apron, np.minimum(z, -max(channel_depth)), z)
    # inlet forebay: a flat pool across the inlet, filled to the floodplain
    # level there, so the total-discharge inlet sees a wet cross-section
    level = float(slope * length)
    forebay = x < 4 * spacing
    z = np.where(forebay, level - max(channel_depth), z)
    z = np.ascontiguousarray(z)
    stage = stage_above
    h = np.maximum(np.maximum(stage - z, 0.0), np.where(cut > 0, floodplain - z, 0.0))
    h = np.where(forebay, level - z, h)
    q = np.ascontiguousarray(np.stack((h, np.zeros_like(h), np.zeros_like(h))))
    case = dict(mesh=mesh, z=z, q=q, seg_mode=np.array([M.MODE_TOTAL_Q, M.MODE_STAGE], np.int32),
                stage_policy=np.zeros(2, np.int32), forcing=np.array([[q_low, 0.0], [0.0, stage]]),
                exterior_bed=_exterior_bed(mesh, z), controls=controls(0.9, 0.03),
                name=f"braided_{length:g}x{width:g}")
    times = np.array([0.0, rise_s, 10 * rise_s])
    value = np.zeros((2, 2, 3))
    value[0, 0] = [q_low, q_high, q_high]
    value[1, 1] = stage
    case["table_time"], case["table_value"] = times, value
    case["exner"] = exner_params(case, diameter=grain, chezy=40.0, erodible=2.0)
    control = {"mode": "constant_ct", "thrust_coefficient": 0.8, "power_coefficient": None}
    rows = []
    for k, (cx, cy) in enumerate(centres):
        cells, _ = __import__("braids_hkt_gb300.turbines", fromlist=["x"]).bump_integrals(mesh, cx, cy, rotor_d)
        hub = float(np.max(z[cells])) + 0.3 + 0.5 * rotor_d
        rows.append(dict(name=f"R{k + 1}", X=cx, Y=cy, D=float(rotor_d), hub_elevation_m=round(hub, 3),
                         minimum_bed_clearance_m=0.1, minimum_surface_clearance_m=0.2, control=control, nu=0.0))
    case["turbines"] = rows
    return case


def exner_params(case, diameter=0.002, porosity=0.4, chezy=44.0, morfac=1.0, sediment_depth=0.001,
                 erodible=2.0, inlet_bc=3, outlet_bc=2, feed=0.0):
    """Bed-update parameters of one scenario: a single grain size, porosity,
    Chezy coefficient of the transport formula, morphological factor, the
    sediment working depth, a non-erodible layer ``erodible`` metres below the
    bed, and per-face bed boundaries (0 wall, 1 prescribed feed, 2 open
    outflow, 3 transport capacity) on the inlet and outlet segments."""
    m = case["mesh"]
    bedbc = np.zeros(m.nf, np.int32)
    feeds = np.zeros(m.nf)
    openf = (m.neighbour < 0) & (m.bid >= 0)
    bedbc[openf & (m.bid == 0)] = inlet_bc
    bedbc[openf & (m.bid == 1)] = outlet_bc
    feeds[openf & (m.bid == 0)] = feed
    return dict(diameter=float(diameter), porosity=float(porosity), chezy=float(chezy), morfac=float(morfac),
                sediment_depth=float(sediment_depth), bedbc=bedbc, feed=feeds,
                rock=np.ascontiguousarray(case["z"] - erodible))


def small_channel(length=120.0, width=24.0, spacing=4.0, seed=7, sigma=0.15, corr=8.0,
                  discharge=20.0, stage=3.0, outlet_bed=-1.0, slope=2e-3, cfl=0.9):
    """A few hundred cells with the same physics as config 1 (for parity tests)."""
    return channel(length, width, spacing, 1.0, seed, sigma, corr, slope, outlet_bed, stage,
                   discharge, 0.03, cfl, field_resolution=0.5)


def rating_channel(discharge=20.0, knots=((0.0, 2.0), (10.0, 2.6), (20.0, 3.0), (40.0, 3.6), (80.0, 4.5)),
                   **kw):
    """The small channel with its outlet controlled by a Q-H rating curve
    (mode 11) instead of a fixed stage: `knots` are (Q [m3/s], water
    elevation [m]); the default passes through the inflow at the initial
    stage of 3.0 m."""
    case = small_channel(discharge=discharge, **kw)
    case["seg_mode"] = np.array([M.MODE_TOTAL_Q, 11], np.int32)
    case["rating"] = {1: [tuple(map(float, k)) for k in knots]}
    case["name"] = "rating_channel"
    return case


def critical_channel(discharge=20.0, **kw):
    """The small channel ending in a critical outlet (mode 4): the outgoing
    characteristic discharge of the controlled faces equals sqrt(g A^3 / B)."""
    case = small_channel(discharge=discharge, **kw)
    case["seg_mode"] = np.array([M.MODE_TOTAL_Q, 4], np.int32)
    case["name"] = "critical_channel"
    return case


def weir_channel(discharge=20.0, crest=2.0, coefficient=1.7, width=24.0, **kw):
    """The small channel ending in a free weir (mode 5): discharge =
    coefficient x width x (stage - crest)^1.5 at the common subcritical
    stage of the opening."""
    case = small_channel(discharge=discharge, **kw)
    case["seg_mode"] = np.array([M.MODE_TOTAL_Q, 5], np.int32)
    case["outlet"] = {1: {"crest_m": float(crest), "coefficient_m_half_s": float(coefficient),
                          "effective_width_m": float(width)}}
    case["name"] = "weir_channel"
    return case


def normal_channel(discharge=20.0, bed_slope=2e-3, **kw):
    """The small channel with a normal-depth outlet (mode 10): per connected
    chain of outlet faces, the level of uniform flow at `bed_slope` with the
    channel's Manning roughness."""
    case = small_channel(discharge=discharge, **kw)
    case["seg_mode"] = np.array([M.MODE_TOTAL_Q, 10], np.int32)
    case["outlet"] = {1: {"bed_slope": float(bed_slope)}}
    case["name"] = "normal_channel"
    return case


def cartesian_channel(length=120.0, width=24.0, spacing=3.0, seed=7, sigma=0.15, corr=8.0, discharge=20.0,
                      stage=3.0, outlet_bed=-1.0, slope=2e-3, cfl=0.9):
    """The small channel on Cartesian square cells (four faces per cell, the
    shape of the reference's uncut Cartesian cells): sloped bed plus a
    Gaussian field, total-discharge inlet, stage outlet, lake at rest at
    `stage` initially."""
    mesh = M.cartesian_mesh(length, width, spacing)
    M.geometry_records(mesh)
    rng = np.random.default_rng(seed + 1000003)
    x, y = mesh.xy
    z = outlet_bed + slope * (length - x)
    if sigma > 0:
        z = z + M.sample_field(M.gaussian_field(length, width, sigma, corr, rng, 0.5), x, y)
    z = np.ascontiguousarray(np.where(x > length - 3 * spacing, outlet_bed, z))
    h = np.maximum(stage - z, 0.0)
    q = np.ascontiguousarray(np.stack((h, np.zeros_like(h), np.zeros_like(h))))
    return dict(mesh=mesh, z=z, q=q, seg_mode=np.array([M.MODE_TOTAL_Q, M.MODE_STAGE], np.int32),
                stage_policy=np.zeros(2, np.int32), forcing=np.array([[discharge, 0.0], [0.0, stage]]),
                exterior_bed=_exterior_bed(mesh, z), controls=controls(cfl, 0.03), name="cartesian_channel")


def stage_discharge_channel(discharge=20.0, reference_stage=3.05, **kw):
    """The small channel fed through an exact-discharge inlet (mode 9): the
    inflow `discharge` is imposed exactly through boundary Riemann solutions
    against a virtual reservoir whose water line is `reference_stage` [m]; the
    outlet keeps its fixed stage."""
    case = small_channel(discharge=discharge, **kw)
    case["seg_mode"] = np.array([9, M.MODE_STAGE], np.int32)
    case["forcing"] = case["forcing"].copy()
    case["forcing"][1, 0] = float(reference_stage)
    case["name"] = "stage_discharge_channel"
    return case


def critical_inlet_channel(discharge=20.0, **kw):
    """The small channel fed through an exact-discharge inlet whose reference
    water line is the section's critical-depth level for the inflow
    (inlet.critical_discharge: Q^2 W / (g A^3) = 1 on the exterior face beds,
    minimum specific energy among the wet-width branches)."""
    case = stage_discharge_channel(discharge=discharge, **kw)
    case["inlet"] = {0: {"line": "critical"}}
    case["name"] = "critical_inlet_channel"
    return case


def normal_inlet_channel(discharge=20.0, energy_slope=2e-3, **kw):
    """The small channel fed through an exact-discharge inlet whose reference
    water line is the section's normal-depth level (inlet.normal_discharge:
    uniform flow at `energy_slope` with the channel's roughness, wetted
    vertical steps between neighbouring faces in the perimeter)."""
    case = stage_discharge_channel(discharge=discharge, **kw)
    case["inlet"] = {0: {"line": "normal", "energy_slope": float(energy_slope)}}
    case["name"] = "normal_inlet_channel"
    return case


def lake_at_rest(length=80.0, width=40.0, spacing=4.0, seed=11, islands=True):
    """Variable bed with emerged islands, flat surface at 1.0 m, closed walls (no open segments)."""
    mesh = M.channel_mesh(length, width, spacing, 1.0, seed)
    mesh.bid[:] = -1
    mesh.boundary_offset = np.zeros(1, np.int32)
    mesh.boundary_faces = np.zeros(0, np.int32)
    x, y = mesh.xy
    z = 0.4 * np.sin(x / 9.0) * np.cos(y / 7.0)
    if islands:
        z = z + 1.6 * np.exp(-((x - 0.3 * length) ** 2 + (y - 0.5 * width) ** 2) / 40.0)
        z = z + 1.3 * np.exp(-((x - 0.7 * length) ** 2 + (y - 0.3 * width) ** 2) / 25.0)
    z = np.ascontiguousarray(z)
    h = np.maximum(1.0 - z, 0.0)
    q = np.ascontiguousarray(np.stack((h, np.zeros_like(h), np.zeros_like(h))))
    return dict(mesh=mesh, z=z, q=q, seg_mode=np.zeros(0, np.int32), stage_policy=np.zeros(0, np.int32),
                forcing=np.zeros((2, 1)), exterior_bed=np.zeros(mesh.nf),
                controls=controls(0.9, 0.03), name="lake_at_rest")


def hydraulic_jump(length=60.0, width=3.0, spacing=0.5, seed=17, froude=2.5, h1=0.4, cfl=0.9):
    """A stationary hydraulic jump on a flat frictionless channel.

    Supercritical inflow of depth h1 at Froude number `froude` through a
    mode-9 inlet (the exact discharge Q with reference water line h1); the
    outlet stage at the conjugate depth h2 = h1 (sqrt(1 + 8 Fr^2) - 1) / 2
    (Belanger); the initial state is the two conjugate states either side of
    mid-channel with the unit discharge q = h1 u1 throughout.
    """
    mesh = M.channel_mesh(length, width, spacing, 0.2, seed)
    g = 9.81
    u1 = froude * np.sqrt(g * h1)
    qx = h1 * u1
    h2 = 0.5 * h1 * (np.sqrt(1.0 + 8.0 * froude ** 2) - 1.0)
    x = mesh.xy[0]
    h = np.where(x < 0.5 * length, h1, h2)
    q = np.ascontiguousarray(np.stack((h, np.full_like(h, qx), np.zeros_like(h))))
    ctl = controls(cfl, 0.03)
    ctl["roughness_mode"] = 1
    ctl["roughness_value"] = 1e12          # Chezy -> infinity: frictionless
    forcing = np.array([[qx * width, 0.0], [h1, h2]])
    return dict(mesh=mesh, z=np.zeros(mesh.nc), q=q, seg_mode=np.array([9, 2], np.int32),
                stage_policy=np.zeros(2, np.int32), forcing=forcing, exterior_bed=np.zeros(mesh.nf),
                controls=ctl, name="hydraulic_jump", jump=dict(h1=h1, h2=h2, q=qx, froude=froude))


def dam_break(length=200.0, width=8.0, spacing=2.0, seed=13, h_left=2.0, h_right=0.0):
    """Dam break on a flat frictionless bed; h_right = 0 gives the dry-bed (Ritter) case."""
    mesh = M.channel_mesh(length, width, spacing, 0.4, seed)
    mesh.bid[:] = -1
    mesh.boundary_offset = np.zeros(1, np.int32)
    mesh.boundary_faces = np.zeros(0, np.int32)
    x = mesh.xy[0]
    z = np.zeros(mesh.nc)
    h = np.where(x < 0.5 * length, h_left, h_right)
    q = np.ascontiguousarray(np.stack((h, np.zeros_like(h), np.zeros_like(h))))
    ctl = controls(0.9, 0.03)
    ctl["roughness_mode"] = 1
    ctl["roughness_value"] = 1e12          # Chezy -> infinity: frictionless
    return dict(mesh=mesh, z=z, q=q, seg_mode=np.zeros(0, np.int32), stage_policy=np.zeros(0, np.int32),
                forcing=np.zeros((2, 1)), exterior_bed=np.zeros(mesh.nf), controls=ctl, name="dam_break")


def perturbed_state(case, seed, amplitude=0.3, velocity=0.6, dry_fraction=0.0):
    """A random but physical state on the case's bed: surface waves, currents and optional dry cells."""
    rng = np.random.default_rng(seed)
    z = case["z"]
    eta = case["q"][0] + z
    eta = eta + amplitude * rng.uniform(-1, 1, eta.shape)
    h = np.maximum(eta - z, 0.0)
    if dry_fraction > 0:
        h[rng.random(h.shape) < dry_fraction] = 0.0
    u = velocity * rng.uniform(-1, 1, h.shape)
    v = velocity * rng.uniform(-1, 1, h.shape)
    return np.ascontiguousarray(np.stack((h, h * u, h * v)))


# ---------------------------------------------------------------------------
# (De)serialisation: a case as flat arrays, so fixtures do not depend on the
# Delaunay implementation of the machine that reads them.
# ---------------------------------------------------------------------------
_MESH_FIELDS = ("points", "tri", "owner", "neighbour", "bid", "normal", "length", "mid", "area", "xy",
                "offset", "faces", "signs", "boundary_offset", "boundary_faces")


def case_arrays(case):
    m = case["mesh"]
    out = {f"mesh_{k}": getattr(m, k) for k in _MESH_FIELDS}
    out.update({f"rec_{k}": v for k, v in m.records.items()})
    for k in ("z", "q", "seg_mode", "stage_policy", "forcing", "exterior_bed"):
        out[k] = np.asarray(case[k])
    for k, v in case["controls"].items():
        out[f"ctl_{k}"] = np.asarray(v)
    for b, knots in (case.get("rating") or {}).items():
        out[f"rating_{int(b)}"] = np.asarray(knots, dtype=np.float64)
    for b, params in (case.get("outlet") or {}).items():
        for name, value in params.items():
            out[f"outlet_{int(b)}_{name}"] = np.asarray(value, dtype=np.float64)
    for b, params in (case.get("inlet") or {}).items():
        out[f"inletline_{int(b)}"] = np.asarray(params.get("line", "stage"))
        out[f"inletslope_{int(b)}"] = np.asarray(float(params.get("energy_slope", 0.0)))
    return out


def case_from_arrays(arrs):
    mesh = M.Mesh(**{k: np.asarray(arrs[f"mesh_{k}"]) for k in _MESH_FIELDS})
    mesh.records = {k[4:]: np.asarray(v) for k, v in arrs.items() if k.startswith("rec_")}
    ctl = {k[4:]: arrs[k].item() for k in arrs if k.startswith("ctl_")}
    ctl["roughness_mode"] = int(ctl["roughness_mode"])
    case = dict(mesh=mesh, controls=ctl, name="fixture")
    for k in ("z", "q", "seg_mode", "stage_policy", "forcing", "exterior_bed"):
        case[k] = np.asarray(arrs[k])
    rating = {int(k[7:]): [tuple(r) for r in np.asarray(v)] for k, v in arrs.items() if k.startswith("rating_")}
    if rating:
        case["rating"] = rating
    outlet = {}
    for k, v in arrs.items():
        if k.startswith("outlet_"):
            seg, name = k[7:].split("_", 1)
            outlet.setdefault(int(seg), {})[name] = float(np.asarray(v))
    if outlet:
        case["outlet"] = outlet
    inlet = {int(k[10:]): {"line": str(np.asarray(v)), "energy_slope": float(np.asarray(arrs[f"inletslope_{k[10:]}"]))}
             for k, v in arrs.items() if k.startswith("inletline_")}
    if inlet:
        case["inlet"] = inlet
    return case


# ---------------------------------------------------------------------------
# Batched scenarios (64 channels of mixed size)
# ---------------------------------------------------------------------------

def config4_params(count=64, seed=4):
    """Per-scenario draws: cells ~ logU(1e4, 5e5), width ~ U(100, 400) m, Q ~ U(100, 1500) m3/s.

    Channels keep the config-1 construction (jittered-grid Delaunay, 1e-3 slope
    plus a Gaussian field, stage outlet at 3 m, conveyance inlet). The length
    is ten widths and the grid spacing follows from the drawn cell count
    (spacing = sqrt(2 L W / cells)), which keeps every Delaunay domain compact.
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        cells = float(np.exp(rng.uniform(np.log(1e4), np.log(5e5))))
        width = float(rng.uniform(100.0, 400.0))
        q = float(rng.uniform(100.0, 1500.0))
        length = 10.0 * width
        spacing = float(np.sqrt(2.0 * length * width / cells))
        out.append(dict(index=i, cells=cells, width=width, length=length, spacing=spacing, discharge=q,
                        seed=int(rng.integers(1, 2**31 - 1))))
    for p in out:
        p["rotors"] = rotor_layout(p["length"], p["width"], p["seed"])
    return out


def rotor_layout(length, width, seed, diameter=5.0, most=8, spacing_d=5.0):
    """0..most rotor centres, uniform over the downstream channel reach
    (x in [0.4, 0.85] L, y in [0.3, 0.7] W), at least spacing_d diameters apart.
    Drawn from a stream derived from the scenario seed, so the hydraulic draws
    of a scenario do not depend on its rotors."""
    rng = np.random.default_rng([seed, 0x7E57])
    count = int(rng.integers(0, most + 1))
    centres = []
    for _ in range(200 * max(count, 1)):
        if len(centres) == count:
            break
        x = float(rng.uniform(0.4 * length, 0.85 * length))
        y = float(rng.uniform(0.3 * width, 0.7 * width))
        if all(np.hypot(x - a, y - b) >= spacing_d * diameter for a, b in centres):
            centres.append((x, y))
    return centres


def config4_case(p, rotors=True):
    """One batch scenario, started in uniform flow (unit discharge Q/W along the channel),
    with its rotors (rated 500 kW, Ct 0.8) in 16 m boxes refined to 1.5 m.

    Starting a 100 m channel from rest under its full discharge drives a
    startup bore past 30 m/s; the batch configuration prescribes no initial
    state, so each channel starts already carrying its discharge.
    """
    from . import turbines as TB
    centres = p.get("rotors", []) if rotors else []
    fine = min(p["spacing"], 1.5)
    boxes = [(x - 8.0, x + 8.0, y - 8.0, y + 8.0, fine) for x, y in centres]
    case = channel(length=p["length"], width=p["width"], spacing=p["spacing"], jitter=0.25 * p["spacing"],
                   seed=p["seed"], discharge=p["discharge"], field_resolution=min(1.0, p["spacing"]), refine=boxes)
    q = case["q"]
    q[1] = np.where(q[0] > 0.0, p["discharge"] / p["width"], 0.0)
    if centres:
        case["turbines"] = rotor_rows(case, centres, control=TB.rated_power_curve(5.0, 0.8, 0.4, 500e3))
        TB.RotorArray(case["mesh"], case["turbines"])        # validate the layout while building
    case["name"] = f"batch_{p['index']:02d}"
    return case


def build_cases(params, workers=None):
    """Build scenario cases in a spawn-context process pool (safe before any CUDA use)."""
    import multiprocessing as mp
    import os
    workers = workers or min(len(params), os.cpu_count() or 1)
    # A spawned child re-imports an unguarded __main__; never start a pool from
    # inside a pool worker (it would respawn forever): build serially there.
    if workers <= 1 or mp.parent_process() is not None:
        return [config4_case(p) for p in params]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(config4_case, params, chunksize=1)
