"""GB300-native state-vector engine for QuantumForge.

A drop-in for the reference's dense state-vector path: gate sweeps,
probabilities, seeded sampling, Pauli-sum expectations and adjoint /
parameter-shift gradients, executed by hand-written sm_103a CUDA kernels
behind the C ABI of ``include/qf.h``. Importing the package does not touch the
GPU; the first call that needs the device loads ``_lib/libqf_gb300.so`` and
raises if it is missing (there is no CPU fallback).
"""
from ._native import QuantumError, load as load_library
from .core import (
    Circuit,
    CudaBackend,
    DensityMatrix,
    Gate,
    NoiseChannel,
    ParameterizedCircuit,
    PauliSum,
    RotationAxis,
    ShotConfig,
    ShotResult,
    SingleQubitObservable,
    SmallRng,
    StateVector,
    StateVectorBatch,
    default_backend,
    export_qasm,
    export_qasm_with_qubits,
    parse_qasm,
    sample_expectation,
    wilson_ci,
)
from . import gradients

__all__ = [
    "Circuit", "CudaBackend", "DensityMatrix", "Gate", "NoiseChannel", "ParameterizedCircuit", "PauliSum", "QuantumError", "RotationAxis",
    "ShotConfig", "ShotResult", "SingleQubitObservable", "SmallRng", "StateVector", "StateVectorBatch", "default_backend", "export_qasm",
    "export_qasm_with_qubits", "parse_qasm", "sample_expectation", "wilson_ci", "gradients",
    "load_library",
]
