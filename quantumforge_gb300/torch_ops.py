"""PyTorch binding of the adjoint gradient.

``QFExpectation`` is a ``torch.autograd.Function`` for E(θ) = <ψ(θ)|H|ψ(θ)>
of a ``ParameterizedCircuit`` and a Pauli-sum H (the reference's
``PyParameterizedCircuit.gradient``, src/python.rs:611-638, with the adjoint
rule). One engine call computes E and dE/dθ (forward state sweep, costate,
reverse sweep on the GPU); ``backward`` scales the stored gradient.
"""
from __future__ import annotations

import numpy as np
import torch

from .gradients import GradientOptions, GradientStrategy, gradient_with_inputs


class QFExpectation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, circuit, qubits, hamiltonian, dtype="c64", backend=None, checkpoint_every=0, inputs=None):
        p = params.detach().to("cpu", torch.float64).numpy()
        est = gradient_with_inputs(circuit, GradientOptions(strategy=GradientStrategy.Adjoint),
                                   [] if inputs is None else inputs, p, int(qubits), hamiltonian, dtype=dtype,
                                   checkpoint_every=int(checkpoint_every), backend=backend)
        ctx.save_for_backward(torch.as_tensor(np.asarray(est.gradient), dtype=params.dtype, device=params.device))
        return torch.as_tensor(est.expectation, dtype=params.dtype, device=params.device)

    @staticmethod
    def backward(ctx, grad_output):
        (g,) = ctx.saved_tensors
        return grad_output * g, None, None, None, None, None, None, None


def expectation(params, circuit, qubits, hamiltonian, dtype="c64", backend=None, checkpoint_every=0, inputs=None):
    """Differentiable <H> of the circuit at `params` (a 1-D tensor)."""
    return QFExpectation.apply(params, circuit, qubits, hamiltonian, dtype, backend, checkpoint_every, inputs)
