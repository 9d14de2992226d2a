"""Golden vectors for the conservative wet-bank viscosity, from the reference's own code.

Run where the reference checkout is present ($BRAIDS_REFERENCE, else a
``reference`` folder beside this repository):

    python oracle/ref_build.py && python tests/golden/make_viscosity_golden.py

The reference's wet-bank viscosity owner (src/braids_core/sediment/
shoreline_viscosity.py:57-72) adds to the momentum rate: its safe state
(secondary_vector_ops.safe), the flow engines' least-squares velocity
gradients on the reference's own prepared geometry (bend_methods_v1_kernels.h
``gradients``, bend_methods_v1.prepared_geometry), the shared-face stresses of
shoreline_viscosity.h and flow_momentum_gather (flow2dh_fixed_bed_kernels.h),
all host-compiled by oracle/ref_build.py and driven by oracle/ref_driver.py.
Each fixture holds a case, a state with dry banks and moving water, the
coefficient, and the reference's rate increment, gradients and face
stresses; tests/test_oracle_viscosity.py checks the C oracle against them.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import braids_hkt_gb300.scenarios as S  # noqa: E402
from ref_driver import Ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "viscosity"


def cases():
    a = S.small_channel(length=200.0, width=30.0, spacing=3.0, discharge=150.0)
    qa = S.perturbed_state(a, 31, 0.3, 0.8, 0.12)
    b = S.lake_at_rest()
    qb = S.perturbed_state(b, 32, 0.4, 0.6, 0.1)
    return {"channel_banks": (a, qa, 0.05), "lake_islands": (b, qb, 0.5)}


def main():
    OUT.mkdir(exist_ok=True)
    for name, (case, q, nu) in cases().items():
        ref = Ref(case, threads=1)
        rate = np.zeros((3, case["mesh"].nc))
        grad, face = ref.viscosity_momentum(q, nu, rate)
        np.savez_compressed(OUT / f"{name}.npz", **S.case_arrays(case), state=q, nu=nu, rate=rate,
                            grad=grad[:4], face=face)
        print(name, case["mesh"].nc, "cells; max |rate|", float(np.abs(rate).max()),
              "wet faces", int((face[0] != 0).sum()))


if __name__ == "__main__":
    main()
