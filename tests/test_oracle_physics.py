"""Known-answer checks of the oracle (the reference's runtime invariants and
analytic solutions), the same cases later run through the CUDA path.

  lake at rest with emerged islands        reconstruction_oracle.py:30-31 ("cutcell_lake")
  water budget per step                    shoreline_solver.py:29-39, 354-360
  dry-bed dam break (Ritter)               reconstruction_oracle.py:30-31 ("dry_dam_break")
  stationary hydraulic jump (Belanger)     reconstruction_oracle.py:30-31 ("hydraulic_jump")
"""
import numpy as np

import braids_hkt_gb300.scenarios as S
from oracle import Oracle


def test_lake_at_rest_round_off():
    case = S.lake_at_rest()
    o = Oracle(case, threads=2)
    q = case["q"].copy()
    st, _, stats = o.advance(q, 5.0, 0.0)
    assert st == 0 and stats["substeps"] > 20
    assert np.abs(q[0] - case["q"][0]).max() < 1e-12
    assert np.abs(q[1:]).max() < 1e-11


def test_closed_basin_mass_conserved():
    case = S.lake_at_rest()
    q = S.perturbed_state(case, 9, 0.4, 0.6, 0.05)
    o = Oracle(case, threads=2)
    area = case["mesh"].area
    v0 = float(np.sum(q[0] * area))
    st, _, stats = o.advance(q, 3.0, 0.0)
    assert st == 0
    v1 = float(np.sum(q[0] * area))
    assert abs(v1 - v0) <= max(1e-10, 64 * np.finfo(float).eps * v0)
    assert q[0].min() >= 0


def test_open_channel_budget():
    """Volume change equals the integrated boundary water flux (stage outlet, Q inlet)."""
    case = S.small_channel()
    m = case["mesh"]
    o = Oracle(case, threads=2)
    q = case["q"].copy()
    v0 = float(np.sum(q[0] * m.area))
    dt = 2.0
    st, water_mean, _ = o.advance(q, dt, 0.0)
    assert st == 0
    openf = (m.neighbour < 0) & (m.bid >= 0)
    outflow = float(np.sum(water_mean[openf] * m.length[openf])) * dt
    v1 = float(np.sum(q[0] * m.area))
    assert abs((v1 - v0) + outflow) <= 1e-9 * max(1.0, v0)
    inflow = -float(np.sum((water_mean * m.length)[openf & (m.bid == 0)])) * dt
    assert 0.9 * 20.0 * dt < inflow < 1.1 * 20.0 * dt       # Q = 20 m3/s imposed


def ritter_depth(x, t, h0, x0, g=9.81):
    c0 = np.sqrt(g * h0)
    xi = (x - x0) / t
    h = np.where(xi <= -c0, h0, np.where(xi >= 2 * c0, 0.0, (2 * c0 - xi) ** 2 / (9 * g)))
    return h


def test_dry_dam_break_matches_ritter():
    case = S.dam_break()
    o = Oracle(case, threads=2)
    q = case["q"].copy()
    t = 4.0
    st, _, _ = o.advance(q, t, 0.0)
    assert st == 0
    x = case["mesh"].xy[0]
    exact = ritter_depth(x, t, 2.0, 100.0)
    inner = (x > 60) & (x < 140)
    err = np.abs(q[0] - exact)[inner]
    assert err.mean() < 0.03          # first-order-limited scheme on a 2 m mesh
    front = x[(q[0] > 1e-3)].max()
    assert abs(front - (100.0 + 2 * np.sqrt(9.81 * 2.0) * t)) < 12.0


def test_hydraulic_jump_holds_conjugate_depths():
    """Supercritical inflow (Fr 2.5, 0.4 m) against the conjugate outlet stage: after 20 s
    the jump stays near mid-channel, the depths either side are Belanger's conjugate pair,
    the unit discharge is uniform and the momentum function q^2/h + g h^2/2 is continuous."""
    case = S.hydraulic_jump()
    j = case["jump"]
    o = Oracle(case, threads=2)
    q = case["q"].copy()
    for k in range(4):
        st, _, _ = o.advance(q, 5.0, 5.0 * k)
        assert st == 0
    x, y = case["mesh"].xy
    up, dn = (x > 5) & (x < 20), (x > 40) & (x < 55)
    h_up, h_dn = q[0][up].mean(), q[0][dn].mean()
    assert abs(h_up - j["h1"]) <= 0.01 * j["h1"]
    assert abs(h_dn - j["h2"]) <= 0.02 * j["h2"]
    for region in (up, dn):
        assert abs(q[1][region].mean() - j["q"]) <= 0.01 * j["q"]
    momentum = lambda h, qq: qq * qq / h + 9.81 * h * h / 2
    m_up, m_dn = momentum(h_up, q[1][up].mean()), momentum(h_dn, q[1][dn].mean())
    assert abs(m_up - m_dn) <= 0.02 * m_up
    band = np.abs(y - 1.5) < 1.0
    x_jump = x[band & (q[0] > 0.5 * (j["h1"] + j["h2"]))].min()
    assert 25.0 < x_jump < 35.0


def _rating_q(knots, eta):
    e = np.array([k[1] for k in knots])
    qv = np.array([k[0] for k in knots])
    return float(np.interp(eta, e, qv))


def test_rating_outlet_follows_its_curve():
    """Q-H outlet (mode 11): the discharge through the opening is the rating
    curve at the opening's water level (within 3% of it, the face level
    differing from the owner cells' mean), through a seiche of the channel."""
    case = S.rating_channel()
    o = Oracle(case, threads=2)
    q = case["q"].copy()
    m = case["mesh"]
    outlet = (m.neighbour < 0) & (m.bid == 1)
    owners = m.owner[outlet]
    t = 0.0
    for k in range(6):
        st, _, _ = o.advance(q, 5.0, t)
        t += 5.0
        stage = float(np.mean(q[0][owners] + case["z"][owners]))
        st2, water, _ = o.advance(q, 0.1, t)      # the discharge over a short window at that level
        t += 0.1
        assert st == 0 and st2 == 0
        out = float(np.sum(water[outlet] * m.length[outlet]))
        assert abs(out - _rating_q(case["rating"][1], stage)) <= 0.03 * max(out, 1.0)


def test_rating_outlet_without_a_bracket_fails():
    """A curve whose elevations lie below any admissible level: the reference
    raises (no retry); the oracle's interval fails."""
    case = S.rating_channel(knots=((0.0, -5.0), (1.0, -4.0)))
    o = Oracle(case, threads=2)
    st, _, _ = o.advance(case["q"].copy(), 1.0, 0.0)
    assert st == 4


def test_normal_depth_outlet_drains_towards_uniform_flow():
    """Normal-depth outlet (mode 10): the channel, filled to 3 m over its
    uniform-flow depth for the inflow, drains through the outlet with a
    discharge falling towards the inflow while staying above it."""
    case = S.normal_channel()
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    m = case["mesh"]
    outlet = (m.neighbour < 0) & (m.bid == 1)
    st, _, _ = o.advance(q, 30.0, 0.0)          # past the first drawdown wave
    assert st == 0
    flows = []
    for k in range(3):
        st, water, _ = o.advance(q, 10.0, 30.0 + 10.0 * k)
        assert st == 0
        flows.append(float(np.sum(water[outlet] * m.length[outlet])))
    assert flows[0] > flows[1] > flows[2] > 20.0


def test_free_weir_outlet_discharges_by_the_weir_law():
    """Free weir (mode 5): the discharge over a short window equals
    coefficient x width x (stage - crest)^1.5 at the outlet cells' stage to
    2%, through the channel's seiche."""
    case = S.weir_channel()
    w_ = case["outlet"][1]
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    m = case["mesh"]
    outlet = (m.neighbour < 0) & (m.bid == 1)
    owners = m.owner[outlet]
    t = 0.0
    for k in range(4):
        st, _, _ = o.advance(q, 5.0, t)
        t += 5.0
        stage = float(np.mean(q[0][owners] + case["z"][owners]))
        st2, water, _ = o.advance(q, 0.1, t)
        t += 0.1
        assert st == 0 and st2 == 0
        out = float(np.sum(water[outlet] * m.length[outlet]))
        law = w_["coefficient_m_half_s"] * w_["effective_width_m"] * max(stage - w_["crest_m"], 0.0) ** 1.5
        assert abs(out - law) <= 0.02 * law


def test_critical_outlet_passes_critical_flow():
    """Critical outlet (mode 4): the discharge over a short window equals the
    critical flow sum(len sqrt(g) (2E/3)^1.5) of the outlet cells' specific
    energy E = h + un^2 / 2g to 3%, while the channel drains through it."""
    case = S.critical_channel()
    o = Oracle(case, threads=4)
    q = case["q"].copy()
    m = case["mesh"]
    g = case["controls"]["grav"]
    outlet = (m.neighbour < 0) & (m.bid == 1)
    owners = m.owner[outlet]
    t = 0.0
    for k in range(3):
        st, _, _ = o.advance(q, 10.0, t)
        t += 10.0
        h = q[0][owners]
        un = (q[1][owners] * m.normal[0, outlet] + q[2][owners] * m.normal[1, outlet]) / h
        energy = h + un * un / (2 * g)
        critical = float(np.sum(m.length[outlet] * np.sqrt(g) * (2 * energy / 3) ** 1.5))
        st2, water, _ = o.advance(q, 0.1, t)
        t += 0.1
        assert st == 0 and st2 == 0
        out = float(np.sum(water[outlet] * m.length[outlet]))
        assert abs(out - critical) <= 0.03 * critical
