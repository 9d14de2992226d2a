"""Generate the golden fixtures from the reference's own kernels.

Run where the reference checkout is present ($BRAIDS_REFERENCE, else a
``reference`` folder beside this repository):

    python oracle/ref_build.py && python tests/golden/make_golden.py

Each fixture holds one small case (mesh, geometry records, bed, boundaries,
controls), an input state, and the outputs of the reference's host-compiled
kernels driven through one spatial residual, one SSPRK(2,2) substep and an
adaptive advance (oracle/ref_driver.py). tests/test_oracle_golden.py checks
the C oracle against them without the reference present.
"""
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import braids_hkt_gb300.scenarios as S  # noqa: E402
from ref_driver import Ref  # noqa: E402

OUT = Path(__file__).resolve().parent

ONLY = sys.argv[1:]          # case names to (re)generate; all when empty

CASES = {
    "channel_wet": (S.small_channel, lambda c: S.perturbed_state(c, 3, 0.3, 0.6, 0.0), 0.01, 1.0),
    "channel_wetdry": (S.small_channel, lambda c: S.perturbed_state(c, 4, 1.5, 0.8, 0.2), 0.01, 1.0),
    "lake_islands": (S.lake_at_rest, lambda c: c["q"], 0.05, 2.0),
    "lake_perturbed": (S.lake_at_rest, lambda c: S.perturbed_state(c, 5, 0.5, 0.5, 0.1), 0.01, 1.0),
    "dam_break_dry": (S.dam_break, lambda c: c["q"], 0.02, 1.0),
    "rating_outlet": (S.rating_channel, lambda c: S.perturbed_state(c, 6, 0.2, 0.4, 0.0), 0.01, 1.0),
    "normal_outlet": (S.normal_channel, lambda c: S.perturbed_state(c, 7, 0.2, 0.4, 0.0), 0.01, 1.0),
    "weir_outlet": (S.weir_channel, lambda c: S.perturbed_state(c, 8, 0.2, 0.4, 0.0), 0.01, 1.0),
    "critical_outlet": (S.critical_channel, lambda c: S.perturbed_state(c, 9, 0.2, 0.4, 0.0), 0.01, 1.0),
    "stage_discharge_inlet": (S.stage_discharge_channel, lambda c: S.perturbed_state(c, 10, 0.2, 0.4, 0.0),
                              0.01, 1.0),
    "critical_inlet": (S.critical_inlet_channel, lambda c: S.perturbed_state(c, 13, 0.2, 0.4, 0.0), 0.01, 1.0),
    "normal_inlet": (S.normal_inlet_channel, lambda c: S.perturbed_state(c, 14, 0.2, 0.4, 0.0), 0.01, 1.0),
    "cartesian_channel": (S.cartesian_channel, lambda c: S.perturbed_state(c, 15, 0.3, 0.5, 0.1), 0.01, 1.0),
}


def main():
    for name, (make, state, dt, interval) in CASES.items():
        if ONLY and name not in ONLY:
            continue
        case = make()
        q = np.ascontiguousarray(state(case))
        ref = Ref(case, threads=1)
        k = ref.kernels(q)
        rate, water, freq = ref.rate(q, dt, 0.0, q)
        q2, w2, peak = ref.single(q, dt, 0.0)
        qa, wa, stats = ref.advance(q.copy(), interval, 0.0)
        arrs = S.case_arrays(case)
        arrs.update(input_q=q, dt=np.float64(dt), interval=np.float64(interval))
        for key in ("v", "active", "grad", "constant", "trace", "kind", "local", "closed", "riemann",
                    "astatus", "fl", "fr", "speed", "fstatus"):
            arrs[f"k_{key}"] = k[key]
        arrs.update(rate=rate, water=water, freq=np.float64(freq), single_q=q2, single_water=w2,
                    single_peak=np.float64(peak), advance_q=qa, advance_water=wa)
        for key, val in stats.items():
            arrs[f"advance_{key}"] = np.asarray(val)
        np.savez_compressed(OUT / f"{name}.npz", **arrs)
        print(name, case["mesh"].nc, "cells", stats)


if __name__ == "__main__":
    main()
