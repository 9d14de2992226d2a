"""Generate the boundary-allocation fixtures from the reference's own classes.

Run where the reference checkout is present ($BRAIDS_REFERENCE, else a
``reference`` folder beside this repository):

    python tests/golden/make_feasibility_golden.py

The reference's OutletFeasibility and InletFeasibility
(src/braids_core/hydraulics/outlet_feasibility.py,
src/braids_core/hydraulics/inlet_feasibility.py) are applied in the order of
ExplicitBoundaryBudget.allocate (src/braids_core/sediment/
river_explicit_boundary_budget.py:37-39) to seeded open-boundary fluxes and
traces on the exact-discharge inlet channel: outward inlet debits larger than
the owners' stock (the cap and its in-section rebalance), sections where no
rebalance exists, and ordinary fluxes that pass unchanged. Each fixture holds
the case, the inputs and the reference's outputs; tests/test_oracle_inlet.py
checks the C oracle against them bit for bit.
"""
import os
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
REFERENCE = Path(os.environ.get("BRAIDS_REFERENCE") or ROOT.parent / "reference")
sys.path.insert(0, str(REFERENCE / "src"))

import braids_hkt_gb300.scenarios as S  # noqa: E402

OUT = Path(__file__).resolve().parent / "feasibility"


def reference_allocation(case, base, dt, flux, trace):
    from braids_core.hydraulics.inlet_feasibility import InletFeasibility
    from braids_core.hydraulics.outlet_feasibility import OutletFeasibility
    m = case["mesh"]
    nb = len(case["seg_mode"])
    data = dict(boundary_faces=np.asarray(m.boundary_faces, np.int32), owner=np.asarray(m.owner, np.int32),
                bid=np.asarray(m.bid, np.int32))
    p = SimpleNamespace(g=dict(length=np.asarray(m.length, np.float64), area=np.asarray(m.area, np.float64)))
    inlet = SimpleNamespace(control=(np.asarray(case["seg_mode"]) == 9).astype(np.int32))
    ext = SimpleNamespace(xp=np, p=p, a=SimpleNamespace(data=data), inlet_compatibility=inlet, nb=nb,
                          hydraulic_mode=np.asarray(case["seg_mode"], np.int32))
    OutletFeasibility(ext)(base, dt, flux, trace)
    InletFeasibility(ext)(base, dt, flux, trace)


def main():
    OUT.mkdir(exist_ok=True)
    case = S.stage_discharge_channel()
    m = case["mesh"]
    nf = m.nf
    openf = np.asarray(m.boundary_faces)
    rng = np.random.default_rng(40)
    seg = np.asarray(case["seg_mode"])[m.bid[openf]]
    inlet = seg == 9
    owners = m.owner[openf]
    # name: (depth factor on the inlet owners, outward excess over the owner's stock, incoming inflow)
    for name, (shallow, excess, inflow, dt) in {"cap": (0.01, 1.5, 3.0, 1.0), "infeasible": (0.001, 40.0, 0.2, 1.0),
                                                "pass": (1.0, 0.0, 1.0, 0.05)}.items():
        base = np.ascontiguousarray(S.perturbed_state(case, 11, 0.2, 0.4, 0.0))
        base[0, np.unique(owners[inlet])] *= shallow
        flux = np.zeros((3, nf))
        trace = np.zeros((3, nf))
        stock = base[0, owners] * m.area[owners] / dt
        water = -rng.uniform(0.5, 1.0, openf.size) * inflow
        out = inlet & (np.arange(openf.size) % 2 == 1) if excess > 0 else np.zeros(openf.size, bool)
        water[out] = stock[out] * excess / m.length[openf[out]]
        water[~inlet] = rng.uniform(-0.5, 1.0, int((~inlet).sum()))
        flux[0, openf] = water
        flux[1:, openf] = rng.normal(0.0, 2.0, (2, openf.size))
        trace[0, openf] = rng.uniform(0.1, 2.0, openf.size)
        trace[0, openf[rng.random(openf.size) < 0.15]] = 0.0
        trace[1:, openf] = rng.normal(0.0, 1.5, (2, openf.size))
        f_out, t_out = flux.copy(), trace.copy()
        reference_allocation(case, base, dt, f_out, t_out)
        arrs = S.case_arrays(case)
        arrs.update(base=base, flux=flux, trace=trace, dt=np.float64(dt), flux_out=f_out, trace_out=t_out)
        np.savez_compressed(OUT / f"{name}.npz", **arrs)
        print(name, "changed flux / trace entries:", int(np.sum(f_out != flux)), int(np.sum(t_out != trace)))


if __name__ == "__main__":
    main()
