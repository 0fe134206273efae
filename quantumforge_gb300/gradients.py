"""Gradient strategies — the reference's ``src/gradients.rs`` over the GB300 engine.

``GradientStrategy``, ``CircuitProfile``, ``GradientOptions`` and
``GradientEstimate`` keep the reference's names, defaults and selection rule
(src/gradients.rs:48-178). The observable is a Pauli sum; the reference's
``SingleQubitObservable`` on one qubit is the one-term case.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._native import QuantumError, check, load, ptr
from .core import PauliSum, _as_terms, _dtype_code, default_backend


class GradientStrategy(enum.IntEnum):
    """`enum GradientStrategy` (src/gradients.rs:48-73)."""

    ParameterShift = _abi.GRAD_PARAMETER_SHIFT
    Adjoint = _abi.GRAD_ADJOINT
    Backprop = _abi.GRAD_BACKPROP
    FiniteDifference = _abi.GRAD_FINITE_DIFFERENCE
    Auto = _abi.GRAD_AUTO

    @staticmethod
    def select(profile: "CircuitProfile"):
        """GradientStrategy::select (src/gradients.rs:81-89)."""
        if profile.has_channel:
            return None
        if profile.shots > 0:
            return GradientStrategy.ParameterShift
        return GradientStrategy.Adjoint

    def name_str(self) -> str:
        return {0: "parameter-shift", 1: "adjoint", 2: "backprop", 3: "finite-difference", 4: "auto"}[int(self)]

    def is_exact(self) -> bool:
        return self != GradientStrategy.FiniteDifference

    @staticmethod
    def parse(name: str):
        table = {
            "parameter-shift": GradientStrategy.ParameterShift, "shift": GradientStrategy.ParameterShift,
            "adjoint": GradientStrategy.Adjoint, "backprop": GradientStrategy.Backprop,
            "backpropagation": GradientStrategy.Backprop, "finite-difference": GradientStrategy.FiniteDifference,
            "finite-diff": GradientStrategy.FiniteDifference, "fd": GradientStrategy.FiniteDifference,
            "auto": GradientStrategy.Auto,
        }
        return table.get(name)


@dataclass
class CircuitProfile:
    """`CircuitProfile` (src/gradients.rs:126-139)."""

    operations: int = 0
    parameters: int = 0
    parameterized_operations: int = 0
    has_channel: bool = False
    shots: int = 0


@dataclass
class GradientOptions:
    """`GradientOptions` (src/gradients.rs:144-165) plus engine knobs."""

    strategy: GradientStrategy = GradientStrategy.Auto
    finite_difference_step: float = 1e-3
    shots: int = 0


@dataclass
class GradientEstimate:
    """`GradientEstimate` (src/gradients.rs:167-178); `expectation` is <H> at the parameters."""

    gradient: np.ndarray
    strategy: GradientStrategy
    evaluations: int
    expectation: float = float("nan")


def gradient_with_inputs(circuit, options: GradientOptions, inputs, parameters, qubits: int, hamiltonian,
                         dtype="c128", checkpoint_every: int = 0, exec_opts=None, backend=None) -> GradientEstimate:
    """ParameterizedCircuit::gradient_with_inputs (src/gradients.rs:232-330) on the device."""
    i, p = circuit._values(inputs, parameters)
    backend = backend or default_backend()
    terms = _as_terms(hamiltonian)
    ops = circuit.ops()
    o = _abi.GradientOpts()
    o.strategy = int(options.strategy)
    o.dtype = _dtype_code(dtype)
    o.finite_difference_step = float(options.finite_difference_step)
    o.shots = int(options.shots)
    o.checkpoint_every = int(checkpoint_every)
    if exec_opts:
        o.exec = _abi.exec_opts(exec_opts)
    grad = np.zeros(p.size, dtype=np.float64)
    e = C.c_double(float("nan"))
    info = _abi.GradientInfo()
    check(load().qf_gradient(backend.handle, int(qubits), ptr(ops), len(ops), ptr(p), p.size, ptr(i), i.size, ptr(terms),
                             len(terms), C.byref(o), C.byref(e), ptr(grad), C.byref(info)))
    return GradientEstimate(grad, GradientStrategy(info.strategy), int(info.evaluations), e.value)


def finite_difference_gradient_with_inputs(circuit, inputs, parameters, qubits, observable, observable_qubit, step,
                                           **kw) -> np.ndarray:
    """finite_difference_gradient_with_inputs (src/gradients.rs:344-375)."""
    opts = GradientOptions(strategy=GradientStrategy.FiniteDifference, finite_difference_step=step)
    return gradient_with_inputs(circuit, opts, inputs, parameters, qubits, PauliSum.single(observable, observable_qubit),
                                **kw).gradient


def backprop_gradient_with_inputs(circuit, inputs, parameters, qubits, observable, observable_qubit, **kw) -> np.ndarray:
    """backprop_gradient_with_inputs (src/gradients.rs:392-506): same reverse-mode sweep as the adjoint."""
    opts = GradientOptions(strategy=GradientStrategy.Backprop)
    return gradient_with_inputs(circuit, opts, inputs, parameters, qubits, PauliSum.single(observable, observable_qubit),
                                **kw).gradient
