"""Golden vectors for the HLLC / MUSCL-Hancock option, from the reference's own operator.

Run where the reference checkout is present ($BRAIDS_REFERENCE, else a
``reference`` folder beside this repository):

    python oracle/ref_build.py && python tests/golden/make_hllc_golden.py [case ...]

The reference's ``HLLCHydraulics`` class (src/braids_core/hydraulics/hllc.py)
runs unchanged: its substep controller, its Hancock step and its own kernels
(hllc.h, hllc_turbines.h, host-compiled by oracle/ref_build.py). Its hooks are
the ones the reference's river owner installs (river_hllc.py:14-55,
river_turbines.py:27-51): the exterior boundary owner and the reference's
OutletFeasibility and InletFeasibility classes, the reference's drag kernel, and for rotors the
reference's wet gradients / Thetis sink. Geometry is the product's channel
meshes (braids_hkt_gb300.scenarios); the operator builds its own incidence
and least-squares inverse from them.

Outputs (tests/golden/hllc/<case>.npz): the initial state, the bed, the
state after each of three 1 s intervals with the controller's substep and
retry counts and the interval-mean water flux, and the internals of one
Hancock step from the initial state (gradients, predicted state, limited
face fluxes, speeds, budget factors, frequencies, the update).
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import braids_hkt_gb300.scenarios as S  # noqa: E402
from ref_driver import Ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "hllc"
INTERVALS = 3
DT = 1.0


def cases():
    return {
        "channel": S.small_channel(),              # inlet (mode 6) and stage outlet (mode 2)
        "lake": S.lake_at_rest(),                  # closed basin, emerged islands
        "dam_break": S.dam_break(),                # dry bed downstream
        "rotors": S.small_rotor_channel(),         # two rotors: sink + HLLC rotor pressure
        "stage_discharge": S.stage_discharge_channel(),   # exact-discharge inlet (mode 9) and its allocation
    }


def main():
    OUT.mkdir(parents=True, exist_ok=True)
    only = sys.argv[1:]                           # case names to (re)generate; all when empty
    for name, case in cases().items():
        if only and name not in only:
            continue
        ref = Ref(case)
        op = ref.hllc_operator()
        q0 = np.ascontiguousarray(case["q"], dtype=np.float64)
        out = dict(q0=q0, z=ref.z.copy())
        # internals of one Hancock step from the initial state
        _, _, f0 = op._spatial_step(q0.copy(), ref.z, 1e-4, 0.0)
        hint = float(0.5 * op.cfl / f0)          # half the admissible step
        q1, w1, f1 = op._spatial_step(q0.copy(), ref.z, hint, 0.0)
        out.update(step_dt=np.float64(hint), step_q=q1, step_water=w1, step_frequency=np.float64(f1),
                   step_grad=op.grad.copy(), step_half=op.half.copy(), step_qhalf=op.qhalf.copy(),
                   step_fl=op.fl.copy(), step_fr=op.fr.copy(), step_speed=op.speed.copy(),
                   step_theta=op.theta.copy(), step_freq=op.frequency.copy(), step_next=op.next.copy())
        op = ref.hllc_operator()
        q = q0.copy()
        qs, subs, retries, waters, hints = [], [], [], [], []
        for k in range(INTERVALS):
            q, water, info = op.advance(q, ref.z, DT, k * DT)
            qs.append(q.copy())
            subs.append(info["hydraulic_substeps"])
            retries.append(info["hydraulic_retries"])
            waters.append(water.copy())
            hints.append(op.step_hint)
        out.update(q=np.stack(qs), substeps=np.array(subs), retries=np.array(retries), water=np.stack(waters),
                   hint=np.array(hints), dt=np.float64(DT))
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(name, case["mesh"].nc, "cells, substeps", subs, "retries", retries)


if __name__ == "__main__":
    main()
