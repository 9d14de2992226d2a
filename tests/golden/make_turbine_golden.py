"""Golden vectors for the rotor array, from the reference's own turbine code.

Run where the reference checkout is present ($BRAIDS_REFERENCE, else a
``reference`` folder beside this repository):

    python oracle/ref_build.py && python tests/golden/make_turbine_golden.py

The reference's ThetisRotor.sample / cell_terms and the coverage gate run on
numpy (src/braids_core/sediment/river_turbine_thetis.py,
river_turbine_flow.py); the wet gradients, surface pack, balanced pressure,
ambient stress and momentum gather are the reference's host-compiled kernels
(river_turbine_flow.h, river_hydrokinetic_stress.h,
flow2dh_fixed_bed_kernels.h), orchestrated as the reference's
install.add (oracle/ref_driver.py). The footprint integrals and rotor-plane
rows come from the product's host geometry (braids_hkt_gb300.turbines).

Outputs (tests/golden/turbines/):
  rotor_steps.npz  one 4k-cell channel with two rotors; for four control
                   modes: one residual, one SSPRK(2,2) substep, a 1 s
                   adaptive advance and the rotor diagnostics after it
  rotor_gate.npz   rotor diagnostics for gate outcomes (coverage, clearances,
                   dry support, no flow, cut-in)
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import braids_hkt_gb300.scenarios as S  # noqa: E402
import braids_hkt_gb300.turbines as TB  # noqa: E402
from ref_driver import Ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "turbines"
FIELDS = ("active", "minimum_coverage_margin_m", "minimum_bed_clearance_m", "local_velocity_m_s",
          "upstream_velocity_m_s", "mean_depth_m", "thrust_coefficient", "power_coefficient",
          "force_per_density_m4_s2", "useful_power_per_density_m5_s3",
          "hydraulic_power_removed_per_density_m5_s3")


def controls():
    table = {"mode": "thetis_speed_table", "model_name": "three-point table", "performance": [
        {"speed_m_s": 0.3, "thrust_coefficient": 0.7, "power_coefficient": 0.35},
        {"speed_m_s": 1.0, "thrust_coefficient": 0.8, "power_coefficient": 0.4},
        {"speed_m_s": 3.0, "thrust_coefficient": 0.6, "power_coefficient": 0.3}]}
    return {
        "constant": ({"mode": "constant_ct", "thrust_coefficient": 0.8, "power_coefficient": None}, 0.0),
        "curves": (TB.rated_power_curve(5.0, 0.8, 0.4, 500e3), 0.005),
        "table": (table, 0.0),
        "incident_table": (dict(table, mode="incident_speed_table"), 0.0),
    }


def diag_rows(samples):
    """(nrotor, fields) values and reason strings of reference samples."""
    vals = np.array([[float(s[0][f]) for f in FIELDS] for s in samples])
    reasons = [s[0]["inactive_reason"] or "covered" for s in samples]
    return vals, reasons


def steps():
    arrs = {}
    base = None
    for name, (control, nu) in controls().items():
        case = S.small_rotor_channel(control=control, nu=nu)
        if base is None:
            base = case
            arrs.update(S.case_arrays(case))
        q = np.ascontiguousarray(case["q"])
        ref = Ref(case, threads=1)
        rate, water, freq = ref.rate(q, 0.005, 0.0, q)
        q2, w2, peak = ref.single(q, 0.01, 0.0)
        qa, wa, stats = ref.advance(q.copy(), 1.0, 0.0)
        vals, reasons = diag_rows(ref.turbine_sample(qa))
        arrs[f"{name}_rows"] = np.array(json.dumps(case["turbines"]))
        arrs.update({f"{name}_rate": rate, f"{name}_single": q2, f"{name}_advance": qa,
                     f"{name}_substeps": np.asarray(stats["substeps"]), f"{name}_diag": vals,
                     f"{name}_reasons": np.array(reasons)})
        print(name, "substeps", stats["substeps"], "power", vals[:, FIELDS.index("useful_power_per_density_m5_s3")])
    np.savez_compressed(OUT / "rotor_steps.npz", **arrs)


def gate():
    case = S.small_rotor_channel(rotors=1)
    row = case["turbines"][0]
    q0 = np.ascontiguousarray(case["q"])
    dry = q0.copy()
    cells, _ = TB.bump_integrals(case["mesh"], row["X"], row["Y"], row["D"])
    dry[0, cells[0]] = 0.0
    dry[1:, cells[0]] = 0.0
    still = q0.copy()
    still[1:] = 0.0
    cutin = {"mode": "thetis_speed_table", "model_name": "late cut-in", "performance": [
        {"speed_m_s": 2.0, "thrust_coefficient": 0.8, "power_coefficient": 0.4},
        {"speed_m_s": 4.0, "thrust_coefficient": 0.8, "power_coefficient": 0.4}]}
    variants = {
        "covered": (dict(row), q0),
        "insufficient_depth": (dict(row, hub_elevation_m=row["hub_elevation_m"] + 4.0), q0),
        "bed_intersection": (dict(row, hub_elevation_m=row["hub_elevation_m"] - 1.5), q0),
        "insufficient_surface_clearance": (dict(row, minimum_surface_clearance_m=3.5), q0),
        "insufficient_bed_clearance": (dict(row, minimum_bed_clearance_m=2.0), q0),
        "dry_numerical_support": (dict(row), dry),
        "no_incoming_flow": (dict(row), still),
        "below_cut_in_speed": (dict(row, control=cutin), q0),
    }
    arrs = dict(S.case_arrays(case))
    arrs.update(dry_q=dry, still_q=still)
    for name, (r, q) in variants.items():
        c = dict(case, turbines=[r])
        c.pop("_rotors", None)
        ref = Ref(c, threads=1)
        vals, reasons = diag_rows(ref.turbine_sample(q))
        assert reasons[0] == name, (name, reasons)
        arrs[f"{name}_rows"] = np.array(json.dumps([r]))
        arrs[f"{name}_state"] = np.array("dry" if q is dry else ("still" if q is still else "initial"))
        arrs[f"{name}_diag"] = vals
        print(name, reasons[0])
    np.savez_compressed(OUT / "rotor_gate.npz", **arrs)


if __name__ == "__main__":
    OUT.mkdir(exist_ok=True)
    steps()
    gate()
