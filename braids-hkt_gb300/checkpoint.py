"""Checkpoint format of a resident solver: authenticated, validated, atomic.

The layout follows the reference owner's checkpoint
(ShorelineSolver.checkpoint_bytes / restart, src/braids_core/sediment/
shoreline_solver.py:374-408, with arrays_to_bytes / write_bytes_atomic,
src/braids_gpu/atomic_output.py:93-114):

  * one uncompressed NPZ archive (numpy.savez) of the state arrays and a
    0-d string array ``metadata`` holding a JSON header;
  * the header carries the solver identity, the clock (time, steps) and a
    SHA-256 of every array's bytes;
  * restart checks the identity, the array inventory, every shape, dtype and
    hash before it changes anything (no partial restart);
  * the file is written to a temporary beside the target and moved over it
    (os.replace), so a reader sees the old or the new checkpoint, never a
    torn one.

The state arrays of a RiverSolver are its accepted state q (3, nc), the bed
z (nc) and the per-scenario step hints (nscen). The identity names the
format, the arithmetic form, the hydraulic method and digests of the packed
geometry and boundary set-up, so a checkpoint restarts only into a solver
built from the same scenarios.
"""
from __future__ import annotations

import hashlib
import io
import json
import os
from pathlib import Path

import numpy as np

FORMAT = "braids_gb300.river_checkpoint.v1"


def digest(*arrays):
    """SHA-256 over the bytes of the arrays (C order), shapes and dtypes."""
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str((a.shape, a.dtype.str)).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def encode(identity, arrays, time=0.0, steps=0):
    """The checkpoint bytes: arrays plus the JSON header (identity, clock, hashes)."""
    arrays = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
    if "metadata" in arrays:
        raise ValueError("'metadata' is reserved for the checkpoint header")
    header = dict(format=FORMAT, identity=identity, time=float(time), steps=int(steps),
                  hashes={k: hashlib.sha256(v.tobytes()).hexdigest() for k, v in arrays.items()})
    stream = io.BytesIO()
    np.savez(stream, metadata=np.array(json.dumps(header, sort_keys=True)), **arrays)
    return stream.getvalue()


def decode(payload, identity, expected):
    """Validate checkpoint bytes against the expected identity and arrays.

    expected: {name: (shape, dtype)}. Returns (arrays, header); raises
    ValueError on any difference, before the caller mutates anything.
    """
    with np.load(io.BytesIO(payload), allow_pickle=False) as saved:
        if "metadata" not in saved.files:
            raise ValueError("checkpoint has no header")
        header = json.loads(str(saved["metadata"]))
        if header.get("format") != FORMAT:
            raise ValueError("checkpoint format differs")
        if header.get("identity") != identity:
            raise ValueError("checkpoint identity differs (another solver set-up)")
        if set(saved.files) != set(expected) | {"metadata"} or set(header.get("hashes", {})) != set(expected):
            raise ValueError("checkpoint array inventory differs")
        arrays = {}
        for name, (shape, dtype) in expected.items():
            a = saved[name]
            if a.shape != tuple(shape) or a.dtype != np.dtype(dtype):
                raise ValueError(f"checkpoint array {name} has another shape or dtype")
            if hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest() != header["hashes"][name]:
                raise ValueError(f"checkpoint array {name} fails its hash")
            arrays[name] = np.array(a, copy=True)
    return arrays, header


def write_atomic(path, payload):
    """Publish the bytes at path through a temporary in the same folder."""
    path = Path(path)
    tmp = path.with_name(f".{path.name}.{os.getpid()}.tmp")
    try:
        with open(tmp, "xb") as f:
            f.write(payload)
            f.flush()
            os.fsync(f.fileno())
        os.replace(tmp, path)
    finally:
        if tmp.exists():
            tmp.unlink()
