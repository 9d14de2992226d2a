"""Golden vectors for the Exner bed update, from the reference's own kernels.

Run where the reference checkout is present ($BRAIDS_REFERENCE, else a
``reference`` folder beside this repository):

    python oracle/ref_build.py && python tests/golden/make_exner_golden.py

The reference's mixture / mpm (river_mpm.h), bend gradients / donor
factors / flux limiter / divergence (bend_methods_v1_kernels.h), mobile-bed
face inputs and bed flux (flow2dh_mobile_kernels.h) and the Koch-Flokstra
slope kernel (src/braids_gpu/flow_bed_slope_runtime.cu), host-compiled,
orchestrated as ShorelinePhysics.finish / bed_faces (oracle/ref_driver.py).
Each case: a scenario, an accepted state after an adaptive advance, and the
reference's trial bed and checks.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import braids_hkt_gb300.scenarios as S  # noqa: E402
from ref_driver import Ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "exner"


def cases():
    a = S.small_channel(length=200.0, width=30.0, spacing=3.0, discharge=150.0)
    a["exner"] = S.exner_params(a, diameter=0.002)
    b = S.small_channel(length=200.0, width=30.0, spacing=3.0, discharge=150.0, seed=9)
    b["exner"] = S.exner_params(b, diameter=0.002, erodible=2e-5, inlet_bc=1, feed=2e-5)   # donor-limited, fed
    c = S.lake_at_rest()
    c["exner"] = S.exner_params(c, diameter=0.002, chezy=30.0, erodible=0.5)
    return {"channel": (a, 20.0, None), "channel_limited_fed": (b, 20.0, None),
            "lake_wetdry": (c, 1.0, lambda k: S.perturbed_state(k, 5, 0.5, 0.5, 0.1))}


def main():
    OUT.mkdir(exist_ok=True)
    for name, (case, interval, state) in cases().items():
        ref = Ref(case, threads=1)
        q = np.ascontiguousarray(state(case) if state else case["q"])
        qa, _, stats = ref.advance(q.copy(), interval, 0.0)
        zt, info = ref.exner(qa, case["z"], interval)
        arrs = S.case_arrays(case)
        for key, val in case["exner"].items():
            arrs[f"ex_{key}"] = np.asarray(val)
        arrs.update(input_q=qa, interval=np.float64(interval), z_trial=zt, flux=info["flux"],
                    ok=np.asarray(info["ok"]), residual=np.float64(info["residual"]),
                    boundary=np.float64(info["boundary"]), donor=np.float64(info["donor"]),
                    change=np.float64(info["change"]))
        np.savez_compressed(OUT / f"{name}.npz", **arrs)
        print(name, {k: v for k, v in info.items() if not isinstance(v, np.ndarray)},
              "max dz", float(np.abs(zt - case["z"]).max()))


if __name__ == "__main__":
    main()
