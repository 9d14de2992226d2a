"""Compile the CUDA library in-tree for sm_103a (Blackwell Ultra / GB300).

Output: braids-hkt_gb300/_build/libbraids_gb300.so (git-ignored). Translation
units compile in parallel; each is a single -gencode for sm_103a.

The FP64 form is compiled with -fmad=false so that its arithmetic keeps the
reference's operation order (the reference builds its CUDA with
--fmad=false --prec-div=true --prec-sqrt=true --ftz=false,
src/braids_support/gpu_fwave/resident_update.py:27).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIBRARY = BUILD / "libbraids_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-diag-suppress", "1444"]
# (source, extra flags)
UNITS = [
    ("brx_api.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    ("brx_mixed.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build braids_gb300")
    return path


def sources():
    return (sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) +
            [HERE.parent / "include" / "braids_gb300.h"])


def up_to_date():
    if not LIBRARY.exists():
        return False
    t = LIBRARY.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources())


def build(force=False, verbose=False):
    """Build the shared library if any source is newer. Returns its path."""
    if not force and up_to_date():
        return LIBRARY
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    objs, jobs = [], []
    for src, flags in UNITS:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *ARCH, *COMMON, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(str(obj))
    errors = []
    for cmd, job in jobs:
        out, _ = job.communicate()
        if job.returncode:
            errors.append(" ".join(cmd) + "\n" + out)
    if errors:
        raise RuntimeError("CUDA build failed:\n" + "\n".join(errors))
    tmp = LIBRARY.with_suffix(".tmp.so")
    link = [cc, *ARCH, "-shared", *objs, "-o", str(tmp), "-lcudart"]
    res = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode:
        raise RuntimeError("link failed:\n" + res.stdout)
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force=True, verbose=True))
