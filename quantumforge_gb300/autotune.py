"""Execution autotuner for gate sweeps.

``autotune_exec`` times a gate list on a device state under candidate
execution options — per-gate tile passes on 12- or 13-qubit tiles, and dense
k-qubit fusion (``block_qubits`` 2..5, the fusion width) — and returns the
fastest, so a caller that applies the same circuit structure many times (a
training loop, a parameter sweep) runs it the best way for its own circuit.
Every candidate is timed with CUDA events on the engine's stream after one
untimed call (which plans and compiles); the state is overwritten.
"""
from __future__ import annotations

import ctypes as C

from ._native import load
from .core import StateVector, default_backend

DEFAULT_CANDIDATES = (
    {},
    {"tile_qubits": 13},
    {"block_qubits": 2},
    {"block_qubits": 3},
    {"block_qubits": 4},
    {"block_qubits": 5},
)


def autotune_exec(ops, qubits: int, dtype: str = "c64", candidates=DEFAULT_CANDIDATES, reps: int = 2, backend=None):
    """Returns (best exec_opts dict, {index: seconds per application}) for the
    gate list ``ops`` (a ``qf_op`` record array) on a ``qubits``-qubit state."""
    import torch

    backend = backend or default_backend()
    sp = C.c_void_p()
    load().qf_ctx_stream(backend.handle, C.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    sv = StateVector.zero(qubits, dtype=dtype, backend=backend)
    times = {}
    for i, eo in enumerate(candidates):
        try:
            sv.apply_ops(ops, exec_opts=eo)
        except Exception:  # an option this state or circuit cannot take
            continue
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            sv.apply_ops(ops, exec_opts=eo)
        e1.record(stream)
        e1.synchronize()
        times[i] = e0.elapsed_time(e1) / 1000.0 / reps
    del sv
    if not times:
        raise RuntimeError("no candidate execution ran")
    best = min(times, key=times.get)
    return dict(candidates[best]), times
