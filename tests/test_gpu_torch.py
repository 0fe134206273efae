"""torch.autograd binding of the adjoint gradient against the oracle's
parameter shift and central finite differences (step 1e-4)."""
import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import ParameterizedCircuit
from quantumforge_gb300 import workloads as W

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pc(ops, n_params):
    pc = ParameterizedCircuit(n_params)
    for r in ops:
        pc.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), int(r["param"]), float(r["theta"])))
    return pc


@pytest.mark.parametrize("dtype,tol", [("c128", 1e-9), ("c64", 2e-5)])
def test_autograd_matches_shift_and_finite_differences(backend, dtype, tol):
    from quantumforge_gb300.torch_ops import expectation

    n = 10
    ops, params, H = W.vqe_tfim(n, 2, seed=21)
    pc = _pc(ops, params.size)
    theta = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    e = expectation(theta, pc, n, H, dtype=dtype, backend=backend)
    (g,) = torch.autograd.grad(2.5 * e, theta)
    shift = O.parameter_shift(ops, n, params, H.array())
    fd = O.finite_difference(ops, n, params, H.array(), 1e-4)
    assert abs(e.item() - O.energy(ops, n, params, H.array())) < tol
    assert np.abs(g.numpy() / 2.5 - shift).max() < tol
    assert np.abs(g.numpy() / 2.5 - fd).max() < 1e-6 + tol  # central differences are O(h^2) = 1e-8 accurate


def test_autograd_in_an_optimisation_step(backend):
    from quantumforge_gb300.torch_ops import expectation

    n = 8
    ops, params, H = W.vqe_tfim(n, 2, seed=5)
    pc = _pc(ops, params.size)
    theta = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    opt = torch.optim.SGD([theta], lr=0.05)
    e0 = expectation(theta, pc, n, H, dtype="c128", backend=backend)
    opt.zero_grad()
    e0.backward()
    opt.step()
    e1 = expectation(theta, pc, n, H, dtype="c128", backend=backend)
    assert e1.item() < e0.item()
