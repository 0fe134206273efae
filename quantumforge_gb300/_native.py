"""Loader and typed bindings for ``libqf_gb300.so`` (the C ABI of include/qf.h).

There is no fallback: if the library is missing, importing the engine raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _abi

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libqf_gb300.so"
_lib = None


class QuantumError(Exception):
    """Error raised for a non-zero ``qf_status``; ``kind`` is the reference's variant name."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.kind = _abi.STATUS_NAMES.get(status, f"Status{status}")
        super().__init__(f"{self.kind}: {message}")


def lib_path() -> Path:
    return Path(os.environ.get("QF_GB300_LIB", str(_LIB_PATH)))


P = C.c_void_p
U32, U64, I32, F64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_double
PU64, PU32, PF64 = C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_double)

# name -> argtypes (every entry point of include/qf.h)
SIGNATURES = {
    "qf_last_error": [],
    "qf_status_name": [C.c_int],
    "qf_abi_version": [],
    "qf_ctx_create": [C.c_int, C.POINTER(P)],
    "qf_ctx_destroy": [P],
    "qf_ctx_synchronize": [P],
    "qf_ctx_stream": [P, C.POINTER(P)],
    "qf_sv_create": [P, U32, C.c_int, U64, C.POINTER(P)],
    "qf_sv_destroy": [P],
    "qf_sv_qubits": [P, PU32],
    "qf_sv_dtype": [P, C.POINTER(C.c_int)],
    "qf_sv_device_ptr": [P, C.POINTER(P)],
    "qf_sv_set_zero": [P],
    "qf_sv_upload": [P, P, U64],
    "qf_sv_download": [P, P, U64],
    "qf_sv_upload_raw": [P, P, U64],
    "qf_sv_download_raw": [P, P, U64],
    "qf_sv_copy_from": [P, P],
    "qf_sv_apply_gate": [P, C.c_int, F64, U32],
    "qf_sv_apply_cnot": [P, U32, U32],
    "qf_sv_apply_cz": [P, U32, U32],
    "qf_sv_apply_swap": [P, U32, U32],
    "qf_sv_apply_ops": [P, P, U64, P, U64, P, U64, P],
    "qf_sv_norm_sqr": [P, PF64],
    "qf_sv_probabilities": [P, P, U64],
    "qf_sv_expectation_z_all": [P, P, U64],
    "qf_sv_expectation": [P, C.c_int, U32, PF64],
    "qf_sv_expectation_pauli_sum": [P, P, U64, P],
    "qf_sv_measure": [P, U32, PU64, C.POINTER(C.c_uint8)],
    "qf_run_circuit": [P, U32, C.c_int, P, U64, P, P, U64, P],
    "qf_run_shots": [P, U32, C.c_int, P, U64, P, U64, U64, F64, P, PU32, PU64, P],
    "qf_run_shots_with_noise": [P, U32, C.c_int, P, U64, P, U64, U64, F64, P, PU32, PU64, P],
    "qf_sv_normalize": [P],
    "qf_sv_apply_channel_trajectory": [P, P, PU64, C.POINTER(C.c_int)],
    "qf_batch_create": [P, U32, C.c_int, U64, C.POINTER(P)],
    "qf_batch_destroy": [P],
    "qf_batch_qubits": [P, PU32],
    "qf_batch_size": [P, PU64],
    "qf_batch_upload": [P, P, U64],
    "qf_batch_download": [P, P, U64],
    "qf_batch_copy_from": [P, P],
    "qf_batch_apply_ops": [P, P, U64, P],
    "qf_batch_measure": [P, U32, PU64, P],
    "qf_run_circuit_batch": [P, U32, C.c_int, P, U64, P, U64, P, U64, P],
    "qf_dm_create": [P, U32, C.c_int, C.POINTER(P)],
    "qf_dm_destroy": [P],
    "qf_dm_qubits": [P, PU32],
    "qf_dm_upload": [P, P, U64],
    "qf_dm_download": [P, P, U64],
    "qf_dm_from_state": [P, P],
    "qf_dm_set_maximally_mixed": [P],
    "qf_dm_apply_ops": [P, P, U64, P],
    "qf_dm_trace": [P, P],
    "qf_dm_purity": [P, PF64],
    "qf_dm_expectation": [P, C.c_int, U32, PF64],
    "qf_dm_probability_one": [P, U32, PF64],
    "qf_dm_probabilities": [P, P, U64],
    "qf_dm_measure": [P, U32, PU64, P],
    "qf_run_density_circuit": [P, U32, C.c_int, P, U64, P, P, U64, P],
    "qf_expectation_density": [P, U32, C.c_int, P, U64, P, U64, P, U64, C.c_int, U32, P, PF64],
    "qf_parameter_shift_gradient_density": [P, U32, C.c_int, P, U64, P, U64, P, U64, C.c_int, U32, P, PF64, P],
    "qf_expectation_shots": [P, U32, C.c_int, P, U64, P, U64, P, U64, C.c_int, U32, U64, U64, F64, P, PF64, PU64, PU64],
    "qf_parameter_shift_gradient_shots": [P, U32, C.c_int, P, U64, P, U64, P, U64, C.c_int, U32, U64, U64, F64, P, P, PU64],
    "qf_sample_expectation": [F64, U64, U64, PF64, PU64],
    "qf_parameter_shift_gradient_density_shots": [P, U32, C.c_int, P, U64, P, U64, P, U64, C.c_int, U32, U64, U64, P, P],
    "qf_parse_qasm": [C.c_char_p, U64, P, U64, PU64, PU32, PU32, PU64],
    "qf_circuit_from_json": [C.c_char_p, U64, P, U64, PU64, PU32, PU32],
    "qf_circuit_to_json": [P, U64, P, U64, PU64],
    "qf_circuit_to_qasm": [P, U64, C.c_int64, P, U64, PU64],
    "qf_sv_sample": [P, P, P, U32, U64, U64, F64, P, PU64],
    "qf_gradient": [P, U32, P, U64, P, U64, P, U64, P, U64, P, P, P, P],
    "qf_expectation": [P, U32, C.c_int, P, U64, P, U64, P, U64, P, U64, P, PF64],
    "qf_plan_stats": [U32, C.c_int, P, U64, P, U64, P, U64, P, PU64, PU64],
    "qf_adjoint_plan_stats": [U32, C.c_int, P, U64, P, U64, P, U64, P, U64, P, P],
    "qf_qaoa_maxcut_batch": [P, P, U64, P, U64, U32, P, P, P, P, P],
    "qf_rng_jump": [U64, U64],
    "qf_expectation_z_all_noalloc": [C.c_int, P, U32, C.c_int, P, P, U64],
}
RESTYPES = {"qf_last_error": C.c_char_p, "qf_status_name": C.c_char_p, "qf_rng_jump": U64}


def load():
    """Load the engine library once; raise if it is missing or incomplete."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not path.exists():
        raise ImportError(
            f"the GB300 engine library is missing ({path}); build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (requires nvcc)"
        )
    lib = C.CDLL(str(path))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError = incomplete library
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != 0:
        msg = load().qf_last_error().decode(errors="replace")
        raise QuantumError(status, msg)


def ptr(a: np.ndarray | None):
    """Data pointer of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the engine must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)
