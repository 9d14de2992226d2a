"""Build the reference's own hot-path kernels for the host, into oracle/_ref/.

TEST INFRASTRUCTURE ONLY. This recipe reads the reference checkout
($BRAIDS_REFERENCE, else a ``reference`` folder beside this repository), runs the reference's own source
transforms exactly as its GPU owner does before compiling, and compiles the
result as host C++ with the reference's CPU flags (``-O3 -fopenmp
-ffp-contract=off``, src/braids_support/sediment/river_morphodynamics/
sediment_wave.py:28). Nothing is copied into the repository: every output
(generated sources and shared libraries) lands in the git-ignored
``oracle/_ref/`` folder.

Generated CUDA C (run on the host through a 10-line shim of the CUDA
built-ins and a loop over the launch grid):
  reconstruction.cu  + wall_bed_hydraulics.cuda_source
                       (src/braids_core/sediment/wall_bed_hydraulics.py:32-36)
  augmented_fwave.cu + face_activity.cuda_transform(resident_update.cu)
                       (src/braids_support/sediment/river_morphodynamics/face_activity.py:30-37,
                        install_hydraulic :76)
  implicit_midpoint_fwave.cu (src/braids_gpu/implicit_midpoint_fwave.cu)
Dual-compiled OpenMP headers (their ENTRY/LOOP macros select the host form):
  river_midpoint.h, river_explicit.h, river_exterior_bed.h,
  river_hydraulic_drag.source() (src/braids_core/sediment/river_hydraulic_drag.py:11-15),
  river_turbine_flow.h, river_hydrokinetic_stress.h (turbine momentum terms),
  river_mpm.h, flow2dh_mobile_kernels.h, bend_methods_v1_kernels.h (Exner / MPM, and the
  flow engines' least-squares gradients), shoreline_viscosity.h (wet-bank viscosity),
  hllc.h, hllc_turbines.h (src/braids_core/hydraulics, the HLLC option),
  river_rating_outlet.h, river_normal_outlet.h, river_exterior_outlet.h (rating,
  normal-depth, critical and free-weir outlets), river_exterior_inlet.h
  (exact-discharge inlets), river_exterior_section.h and
  river_exterior_normal.h (their critical and normal reference lines)
Generated CUDA C also: flow_bed_slope_runtime.cu (src/braids_gpu, Koch-Flokstra slope)

Usage: python oracle/ref_build.py   (exits non-zero when the reference is absent)
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference checkout: $BRAIDS_REFERENCE, else a `reference` folder beside this repository
REFERENCE = Path(os.environ.get("BRAIDS_REFERENCE") or HERE.parent.parent / "reference")
FLAGS = ["-x", "c++", "-std=c++17", "-O3", "-fopenmp", "-shared", "-fPIC", "-ffp-contract=off"]
DECLSPEC = '-D__declspec(x)=__attribute__((visibility("default")))'

SHIM = r"""
// Host shim for CUDA C kernels: built-in indices become thread-local structs
// and every kernel is driven by a loop over its 1-D launch grid.
#include <cmath>
#include <cstdint>
using std::sqrt; using std::fabs; using std::fmin; using std::fmax; using std::isfinite;
using std::hypot; using std::copysign; using std::pow; using std::log1p; using std::log10; using std::exp;
struct brx_dim3 { unsigned x, y, z; };
static thread_local brx_dim3 blockIdx, threadIdx, blockDim, gridDim;
#define __device__
#define __global__
#define __forceinline__ inline
static inline double atomicAdd(double *a, double v) { double o;
    _Pragma("omp atomic capture") { o = *a; *a += v; } return o; }
template <class F> static void brx_launch(long long n, F body) {
    const long long blocks = (n + 127) / 128;
    #pragma omp parallel for schedule(static)
    for (long long b = 0; b < blocks; ++b) {
        blockDim.x = 128; gridDim.x = (unsigned)blocks; blockIdx.x = (unsigned)b;
        for (unsigned t = 0; t < 128; ++t) { threadIdx.x = t; body(); }
    }
}
"""


def _kernel_wrappers(code):
    """extern "C" L_<name>(long long count, <params>) launching each kernel over count threads."""
    out = []
    for name, params in re.findall(r'extern "C" __global__ void (\w+)\s*\((.*?)\)\s*\{', code, re.S):
        plist = [p.strip() for p in params.replace("\n", " ").split(",") if p.strip()]
        names = [re.findall(r"(\w+)\s*$", p)[0] for p in plist]
        out.append(f'extern "C" void L_{name}(long long brx_count, {", ".join(plist)}) '
                   f'{{ brx_launch(brx_count, [&]{{ {name}({", ".join(names)}); }}); }}')
    return "\n".join(out)


def generate():
    src = REFERENCE / "src"
    if not src.is_dir():
        raise SystemExit(f"reference checkout not found at {REFERENCE}")
    sys.path.insert(0, str(src))
    from braids_core.sediment import wall_bed_hydraulics
    from braids_support.sediment.river_morphodynamics import face_activity
    from braids_core.sediment import river_hydraulic_drag
    gpu = src / "braids_support/gpu_fwave"
    reconstruction = wall_bed_hydraulics.cuda_source((gpu / "reconstruction.cu").read_text())
    update = (gpu / "augmented_fwave.cu").read_text() + "\n" + \
        face_activity.cuda_transform((gpu / "resident_update.cu").read_text())
    gather = (src / "braids_gpu/implicit_midpoint_fwave.cu").read_text()
    OUT.mkdir(exist_ok=True)
    slope = (src / "braids_gpu/flow_bed_slope_runtime.cu").read_text()
    units = {"ref_reconstruction": reconstruction, "ref_update": update, "ref_gather": gather,
             "ref_slope": slope}
    for name, code in units.items():
        (OUT / f"{name}.cpp").write_text(SHIM + "\n" + code + "\n" + _kernel_wrappers(code) + "\n")
    headers = {
        "ref_midpoint": (src / "braids_core/sediment/river_midpoint.h").read_text(),
        "ref_explicit": (src / "braids_core/sediment/river_explicit.h").read_text(),
        "ref_exterior": (src / "braids_core/sediment/river_exterior_bed.h").read_text(),
        "ref_drag": river_hydraulic_drag.source(False),
        # turbine momentum terms (river_turbine_flow.h, river_hydrokinetic_stress.h)
        "ref_hkt": (src / "braids_core/sediment/river_turbine_flow.h").read_text(),
        "ref_stress": (src / "braids_core/sediment/river_hydrokinetic_stress.h").read_text(),
        "ref_flow": (src / "braids_core/sediment/flow2dh_fixed_bed_kernels.h").read_text(),
        # Exner bed update with MPM transport
        "ref_mpm": (src / "braids_core/sediment/river_mpm.h").read_text(),
        "ref_mobile": (src / "braids_core/sediment/flow2dh_mobile_kernels.h").read_text(),
        "ref_bend": (src / "braids_core/sediment/bend_methods_v1_kernels.h").read_text(),
        # conservative wet-bank viscosity (shoreline_viscosity.py)
        "ref_visc": (src / "braids_core/sediment/shoreline_viscosity.h").read_text(),
        # HLLC / MUSCL-Hancock option and its rotor pressure correction
        "ref_hllc": (src / "braids_core/hydraulics/hllc.h").read_text(),
        "ref_hllc_turbines": (src / "braids_core/hydraulics/hllc_turbines.h").read_text(),
        # section owners of the remaining outlet modes
        "ref_rating": (src / "braids_core/sediment/river_rating_outlet.h").read_text(),
        "ref_normal": (src / "braids_core/sediment/river_normal_outlet.h").read_text(),
        "ref_outlet": (src / "braids_core/sediment/river_exterior_outlet.h").read_text(),
        # exact-discharge inlets (mode 9)
        "ref_inlet": (src / "braids_core/sediment/river_exterior_inlet.h").read_text(),
        # their critical-depth and normal-depth reference lines
        "ref_section": (src / "braids_core/sediment/river_exterior_section.h").read_text(),
        "ref_section_normal": (src / "braids_core/sediment/river_exterior_normal.h").read_text(),
    }
    for name, code in headers.items():
        (OUT / f"{name}.h").write_text(code)
    return list(units) + list(headers)


def compile_all(names):
    jobs = []
    for name in names:
        src = OUT / (f"{name}.cpp" if (OUT / f"{name}.cpp").exists() else f"{name}.h")
        cmd = ["g++", *FLAGS, DECLSPEC, str(src), "-o", str(OUT / f"lib{name}.so")]
        jobs.append(subprocess.Popen(cmd, stderr=subprocess.PIPE, text=True))
    failed = []
    for name, job in zip(names, jobs):
        _, err = job.communicate()
        if job.returncode:
            failed.append((name, err[-2000:]))
    if failed:
        raise SystemExit("reference host build failed: " + repr(failed))


def main():
    names = generate()
    compile_all(names)
    print("built", ", ".join(f"lib{n}.so" for n in names), "in", OUT)


if __name__ == "__main__":
    main()
