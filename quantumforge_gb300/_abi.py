"""ctypes mirror of ``include/qf.h``: constants, record layouts and numpy dtypes.

Only layouts live here; ``_native`` binds the functions.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# status codes (QuantumError / CudaError variants)
STATUS_NAMES = {
    0: "Ok",
    1: "ZeroQubits",
    2: "MemoryBudgetExceeded",
    3: "SimulationSizeOverflow",
    4: "MemoryAllocationFailed",
    5: "StateSizeNotPowerOfTwo",
    6: "QubitOutOfRange",
    7: "InvalidQubitPair",
    8: "InvalidProbability",
    9: "OperationRequiresDensityMatrix",
    10: "OperationRequiresShotExecution",
    11: "InvalidShotCount",
    12: "ClassicalBitOutOfRange",
    13: "InvalidParameterCount",
    14: "InvalidInputCount",
    15: "NonFiniteParameter",
    16: "InvalidFiniteDifferenceStep",
    17: "UnsupportedOperation",
    18: "Timeout",
    19: "Cuda",
    20: "InvalidArgument",
    21: "EmptyBatch",
    22: "IncompatibleBatch",
    23: "StateTooLarge",
    24: "IncompatibleDeviceState",
}
STATUS_CODES = {v: k for k, v in STATUS_NAMES.items()}

# enum qf_gate (order of `enum Gate`, src/lib.rs:2239-2264)
GATE_I, GATE_X, GATE_Y, GATE_Z, GATE_H, GATE_S, GATE_SDG, GATE_T, GATE_TDG, GATE_RX, GATE_RY, GATE_RZ = range(12)
GATE_NAMES = ["I", "X", "Y", "Z", "H", "S", "Sdg", "T", "Tdg", "Rx", "Ry", "Rz"]

# enum qf_pauli1
PAULI_X, PAULI_Y, PAULI_Z = 0, 1, 2

# enum qf_op_kind
OP_GATE, OP_CNOT, OP_CZ, OP_SWAP, OP_CHANNEL, OP_MEASURE, OP_COND, OP_ROTATION, OP_ENCODING = range(9)

# enum qf_channel (order of `enum NoiseChannel`, src/lib.rs:1561-1600)
CHANNEL_DEPOLARIZING, CHANNEL_AMPLITUDE_DAMPING, CHANNEL_PHASE_DAMPING, CHANNEL_THERMAL_DAMPING = range(4)

# enum qf_dtype
C64, C128 = 0, 1

# enum qf_exec_mode
EXEC_AUTO, EXEC_UNFUSED, EXEC_FUSED = 0, 1, 2

# enum qf_gradient_strategy
GRAD_PARAMETER_SHIFT, GRAD_ADJOINT, GRAD_BACKPROP, GRAD_FINITE_DIFFERENCE, GRAD_AUTO = range(5)


class Op(C.Structure):
    _fields_ = [
        ("kind", C.c_uint8),
        ("gate", C.c_uint8),
        ("flags", C.c_uint16),
        ("q0", C.c_uint32),
        ("q1", C.c_uint32),
        ("param", C.c_uint32),
        ("theta", C.c_double),
    ]


class PauliTerm(C.Structure):
    _fields_ = [
        ("xmask", C.c_uint64),
        ("zmask", C.c_uint64),
        ("coeff_re", C.c_double),
        ("coeff_im", C.c_double),
    ]


class ExecOpts(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("tile_qubits", C.c_int32),
        ("block_qubits", C.c_int32),
        ("flags", C.c_int32),
    ]


EXEC_FLAG_SMEM_TILES = 1
EXEC_FLAG_JIT = 2
EXEC_FLAG_NO_JIT = 4
EXEC_FLAG_SHOTS_TREE = 8
EXEC_FLAG_SHOTS_TRAJECTORIES = 16
EXEC_FLAG_PLAN_FIRST_COME = 32
EXEC_FLAG_BLOCKS_SIMT = 64
_MODES = {"auto": EXEC_AUTO, "unfused": EXEC_UNFUSED, "fused": EXEC_FUSED}


def exec_opts(opts) -> "ExecOpts":
    """qf_exec_opts from a dict {mode, tile_qubits, block_qubits, smem_tiles, jit,
    shots_engine ("tree" | "trajectories"), blocks_engine ("auto" | "simt")}."""
    if isinstance(opts, ExecOpts):
        return opts
    opts = opts or {}
    flags = EXEC_FLAG_SMEM_TILES if opts.get("smem_tiles") else 0
    if opts.get("jit") is True:
        flags |= EXEC_FLAG_JIT
    elif opts.get("jit") is False:
        flags |= EXEC_FLAG_NO_JIT
    if opts.get("plan") == "first_come":
        flags |= EXEC_FLAG_PLAN_FIRST_COME
    elif opts.get("plan", "lookahead") != "lookahead":
        raise ValueError("plan must be 'lookahead' or 'first_come'")
    blocks = opts.get("blocks_engine")
    if blocks == "simt":
        flags |= EXEC_FLAG_BLOCKS_SIMT
    elif blocks not in (None, "auto"):
        raise ValueError("blocks_engine must be 'auto' or 'simt'")
    engine = opts.get("shots_engine")
    if engine == "tree":
        flags |= EXEC_FLAG_SHOTS_TREE
    elif engine == "trajectories":
        flags |= EXEC_FLAG_SHOTS_TRAJECTORIES
    elif engine is not None:
        raise ValueError("shots_engine must be 'tree' or 'trajectories'")
    return ExecOpts(_MODES[opts.get("mode", "auto")], int(opts.get("tile_qubits", 0)), int(opts.get("block_qubits", 0)),
                    flags)


class GradientOpts(C.Structure):
    _fields_ = [
        ("strategy", C.c_int32),
        ("dtype", C.c_int32),
        ("finite_difference_step", C.c_double),
        ("shots", C.c_uint64),
        ("checkpoint_every", C.c_int32),
        ("reserved", C.c_int32),
        ("exec", ExecOpts),
    ]


class AdjointStats(C.Structure):
    """qf_adjoint_stats: launches and algorithmic HBM bytes of one adjoint gradient."""
    _fields_ = [("forward_passes", C.c_uint64), ("backward_passes", C.c_uint64), ("pauli_passes", C.c_uint64),
                ("state_copies", C.c_uint64), ("hbm_bytes", C.c_double)]


class GradientInfo(C.Structure):
    _fields_ = [("strategy", C.c_int32), ("reserved", C.c_int32), ("evaluations", C.c_uint64)]


assert C.sizeof(Op) == 24, C.sizeof(Op)
assert C.sizeof(PauliTerm) == 32

OP_DTYPE = np.dtype(
    [("kind", "u1"), ("gate", "u1"), ("flags", "<u2"), ("q0", "<u4"), ("q1", "<u4"), ("param", "<u4"), ("theta", "<f8")],
    align=True,
)
TERM_DTYPE = np.dtype([("xmask", "<u8"), ("zmask", "<u8"), ("coeff_re", "<f8"), ("coeff_im", "<f8")])
assert OP_DTYPE.itemsize == 24 and TERM_DTYPE.itemsize == 32


def ops_array(records) -> np.ndarray:
    """Build a contiguous ``qf_op`` array from (kind, gate, q0, q1, param, theta[, flags]) tuples."""
    rows = [(r[0], r[1], r[6] if len(r) > 6 else 0, r[2], r[3], r[4], r[5]) for r in records]
    return np.array(rows, dtype=OP_DTYPE) if rows else np.zeros(0, dtype=OP_DTYPE)


def aux_fields(value: float) -> tuple[int, int]:
    """(q1, param) of a channel record whose second parameter is `value`:
    the float64 bits split as q1 = low 32, param = high 32 (qf_op_set_aux)."""
    bits = int(np.float64(value).view(np.uint64))
    return bits & 0xFFFFFFFF, bits >> 32


def channel_record(kind: int, target: int, p: float, beta_delta: float = 0.0) -> tuple:
    """A QF_OP_CHANNEL record: channel `kind` on `target`, theta = probability
    / gamma / gamma_down, beta_delta (thermal channel) in the aux fields."""
    q1, param = aux_fields(beta_delta)
    return (OP_CHANNEL, int(kind), int(target), q1, param, float(p))


def terms_array(terms) -> np.ndarray:
    """Build a ``qf_pauli_term`` array from (xmask, zmask, coeff) tuples (coeff real or complex)."""
    arr = np.zeros(len(terms), dtype=TERM_DTYPE)
    for i, (x, z, c) in enumerate(terms):
        c = complex(c)
        arr[i] = (x, z, c.real, c.imag)
    return arr
