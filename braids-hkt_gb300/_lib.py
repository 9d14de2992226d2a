"""ctypes binding of include/braids_gb300.h.

The library is the only compute path: if it cannot be loaded this module
raises, it never falls back to Python or CPU arithmetic.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import LIBRARY, build

P = C.c_void_p
I = C.c_int
D = C.c_double

# Every symbol declared in include/braids_gb300.h with (restype, argtypes).
SIGNATURES = {
    "brx_last_error": (C.c_char_p, []),
    "brx_version": (I, []),
    "brx_solver_create": (I, [I, P, P, I, I, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, I, P, P, P, I,
                              C.POINTER(P)]),
    "brx_solver_destroy": (I, [P]),
    "brx_controls_set": (I, [P, I, D, D, D, D, I, D]),
    "brx_boundary_set": (I, [P, P, P, P, P]),
    "brx_forcing_table_set": (I, [P, I, P, P]),
    "brx_forcing_set": (I, [P, P]),
    "brx_viscosity_set": (I, [P, P, P, P, P]),
    "brx_state_bind": (I, [P, P, P]),
    "brx_advance": (I, [P, D, D, P]),
    "brx_advance_batch": (I, [P, P, P, P]),
    "brx_advance_chain": (I, [P, P, P, I, P, P, P]),
    "brx_tile_set": (I, [P, I]),
    "brx_tile_get": (I, [P, P, P]),
    "brx_substep": (I, [P, D, D, P, P]),
    "brx_rate": (I, [P, D, D, P, P, P, P]),
    "brx_scenarios_activate": (I, [P, P]),
    "brx_turbines_set": (I, [P, I, P, P, P, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
    "brx_turbines_diagnose": (I, [P, P]),
    "brx_turbines_last": (I, [P, P]),
    "brx_exner_set": (I, [P, P, P, P, P, P, P, P, P]),
    "brx_exner": (I, [P, P, P]),
    "brx_advance_start": (I, [P, P, P]),
    "brx_advance_poll": (I, [P, P, P]),
    "brx_solver_bytes": (C.c_longlong, [P]),
    "brx_totals": (I, [P, P]),
    "brx_rating_set": (I, [P, P, P, P]),
    "brx_outlet_chains_set": (I, [P, I, P, P, P]),
    "brx_weir_set": (I, [P, P]),
    "brx_critical_chains_set": (I, [P, P, P, P]),
    "brx_inlet_lines_set": (I, [P, P, P, P, P]),
    "brx_forcing_get": (I, [P, P]),
    "brx_ledger_get": (I, [P, P]),
    "brx_ledger_gross_get": (I, [P, P]),
    "brx_hllc_set": (I, [P, P, P, P, P]),
    "brx_method_set": (I, [P, I]),
    "brx_launch_shape_set": (I, [P, I, I, I]),
    "brx_launch_shape_get": (I, [P, I, P, P, P]),
    "brx_hint_get": (I, [P, P]),
    "brx_hint_set": (I, [P, P]),
    "brx_graph_chunk_set": (I, [P, I]),
    "brx_profile_substep": (I, [P, D, D, I, P, P, P]),
    "brx_fma_rate": (I, [I, P, P]),
    "brx_rate_noalloc": (I, [I, I, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, D, D, D, D, P, P, P, P,
                             P]),
    "brx_launch_count": (C.c_longlong, [P]),
    "brx_stream": (P, [P]),
}

ERRORS = {1: "argument", 2: "cuda", 3: "state", 4: "rejected", 5: "unsupported"}


class BrxError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"braids_gb300 error {code} ({ERRORS.get(code, '?')}): {message}")
        self.code = code


class AdvanceStats(C.Structure):
    _fields_ = [("substeps", I), ("rejections", I), ("failed", I), ("pad", I),
                ("min_dt", D), ("max_dt", D), ("accepted_cfl_max", D), ("hint", D)]


_lib = None


def load(path: Path | None = None, build_if_missing=True):
    """Load (building first if needed) and type the library."""
    global _lib
    if _lib is not None:
        return _lib
    lib_path = Path(path) if path else LIBRARY
    if build_if_missing:
        build()
    if not lib_path.exists():
        raise OSError(f"braids_gb300 library missing at {lib_path}; run __graft_entry__.build()")
    lib = C.CDLL(str(lib_path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code):
    if code != 0:
        raise BrxError(code, _lib.brx_last_error().decode())
    return code
