"""The C-ABI library loads and exports every symbol include/braids_gb300.h declares.

No compute call is made here (there is no GPU in the CPU suite); argument
validation that happens before any CUDA call is exercised.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np

import braids_hkt_gb300._lib as L

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(brx_\w+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported():
    lib = L.load()
    names = declared()
    assert names, "no declarations found"
    for name in names:
        assert hasattr(lib, name), name
    assert names == set(L.SIGNATURES)


def test_version_and_error_string():
    lib = L.load()
    assert lib.brx_version() >= 1
    assert isinstance(lib.brx_last_error(), bytes)


def test_create_rejects_bad_topology_without_cuda():
    lib = L.load()
    h = C.c_void_p()
    one = np.array([0, 1], np.int32)
    bad_owner = np.array([5], np.int32)      # out of range
    z = np.zeros(8)
    i = np.zeros(4, np.int32)
    p = lambda a: C.c_void_p(a.ctypes.data)
    rc = lib.brx_solver_create(1, p(one), p(one), 1, 1, 1, p(bad_owner), p(np.array([-1], np.int32)),
                               p(np.array([-1], np.int32)), p(one), p(np.array([0], np.int32)),
                               p(np.array([1], np.int32)), p(z), p(z), p(z), p(z), p(z), p(z), p(z), None, p(z),
                               0, None, None, None, 0, C.byref(h))
    assert rc == 1 and b"out of range" in lib.brx_last_error()
    rc = lib.brx_solver_create(1, p(one), p(one), 1, 1, 1, p(i), p(i), p(i), p(one), p(i), p(i),
                               p(z), p(z), p(z), p(z), p(z), p(z), p(z), None, p(z), 0, None, None, None, 7, C.byref(h))
    assert rc == 1 and b"precision" in lib.brx_last_error()
    assert not h.value
