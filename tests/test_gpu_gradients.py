"""GPU gradients: the reference's gradient tests (tests/gradients.rs,
tests/quantum_core.rs:79-124) through the engine, and the Pauli-sum adjoint
against the oracle. complex128 gradients within the reference's tolerances;
complex64 (f32 gate arithmetic, f64 accumulation) within the bound stated per
test."""
import math

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import (NoiseChannel, ParameterizedCircuit, PauliSum, QuantumError, RotationAxis,
                                SingleQubitObservable)
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import workloads as W
from quantumforge_gb300.gradients import (
    GradientOptions,
    GradientStrategy,
    backprop_gradient_with_inputs,
    finite_difference_gradient_with_inputs,
    gradient_with_inputs,
)

pytestmark = pytest.mark.gpu
Z = SingleQubitObservable.Z


def pc_from_ops(ops, n_params, n_inputs=0):
    pc = ParameterizedCircuit(n_params, n_inputs)
    for r in ops:
        pc.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), int(r["param"]),
                              float(r["theta"])))
    return pc


def test_ry_gradient_matches_the_analytic_derivative(backend):  # tests/gradients.rs:18-48
    c = ParameterizedCircuit.new(1)
    c.rotation(RotationAxis.Y, 0, 0)
    for s in (GradientStrategy.ParameterShift, GradientStrategy.Adjoint, GradientStrategy.Backprop):
        est = c.gradient(GradientOptions(strategy=s), [0.7], 1, Z, 0, backend=backend)
        assert abs(est.gradient[0] + math.sin(0.7)) < 1e-10, s


def test_all_exact_strategies_agree(backend):  # tests/gradients.rs:50-107
    c = ParameterizedCircuit.new(42)
    params = []
    for layer in range(3):
        for q in range(7):
            c.rotation(RotationAxis.Y, q, len(params))
            params.append(0.3 + 0.1 * layer)
        for q in range(7):
            c.rotation(RotationAxis.X, q, len(params))
            params.append(-0.2 + 0.05 * q)
        for q in range(6):
            c.cnot(q, q + 1)
    ref = c.gradient(GradientOptions(strategy=GradientStrategy.ParameterShift), params, 7, Z, 0, backend=backend)
    assert ref.gradient.size == 42
    oracle_ref = O.parameter_shift(c.ops(), 7, params, A.terms_array([(0, 1, 1.0)]))
    assert np.abs(ref.gradient - oracle_ref).max() < 1e-10
    for s in (GradientStrategy.Adjoint, GradientStrategy.Backprop):
        est = c.gradient(GradientOptions(strategy=s), params, 7, Z, 0, backend=backend)
        assert np.abs(est.gradient - ref.gradient).max() < 1e-9


def test_backprop_free_function_matches_the_method(backend):  # tests/gradients.rs:109-130
    c = ParameterizedCircuit.new(2)
    c.rotation(RotationAxis.Y, 0, 0)
    c.rotation(RotationAxis.Z, 1, 1)
    c.cnot(0, 1)
    c.rotation(RotationAxis.X, 0, 0)
    free = backprop_gradient_with_inputs(c, [], [0.4, -1.1], 2, Z, 0, backend=backend)
    method = c.gradient(GradientOptions(strategy=GradientStrategy.Backprop), [0.4, -1.1], 2, Z, 0, backend=backend)
    assert np.array_equal(free, method.gradient)


def test_shared_parameter_sums_occurrence_wise_derivatives(backend):  # tests/gradients.rs:132-172
    c = ParameterizedCircuit.new(1)
    c.rotation(RotationAxis.Y, 0, 0)
    c.rotation(RotationAxis.Y, 1, 0)
    c.cnot(0, 1)
    shift = c.parameter_shift_gradient([0.9], 2, 1, backend=backend)
    adj = c.adjoint_gradient([0.9], 2, Z, 1, backend=backend)
    assert abs(shift[0] - adj[0]) < 1e-10
    single = ParameterizedCircuit.new(1)
    single.rotation(RotationAxis.Y, 0, 0)
    single.cnot(0, 1)
    assert abs(shift[0] - single.parameter_shift_gradient([0.9], 2, 1, backend=backend)[0]) > 1e-3


def test_finite_difference_converges_at_second_order(backend):  # tests/gradients.rs:174-203
    c = ParameterizedCircuit.new(2)
    c.rotation(RotationAxis.Y, 0, 0)
    c.rotation(RotationAxis.X, 1, 1)
    c.cnot(0, 1)
    c.rotation(RotationAxis.Y, 2, 0)
    exact = c.parameter_shift_gradient([0.5, -0.4], 3, 0, backend=backend)
    prev = math.inf
    for step in (1e-2, 1e-3, 1e-4):
        err = np.abs(finite_difference_gradient_with_inputs(c, [], [0.5, -0.4], 3, Z, 0, step, backend=backend)
                     - exact).max()
        assert err * 50 < prev
        prev = err
    assert prev < 1e-8


@pytest.mark.parametrize("step", [0.0, -1.0, float("nan"), float("inf")])
def test_finite_difference_step_must_be_positive_and_finite(backend, step):  # tests/gradients.rs:205-221
    c = ParameterizedCircuit.new(1)
    c.rotation(RotationAxis.Y, 0, 0)
    with pytest.raises(QuantumError) as e:
        finite_difference_gradient_with_inputs(c, [], [0.3], 1, Z, 0, step, backend=backend)
    assert e.value.kind == "InvalidFiniteDifferenceStep"


def test_auto_selects_and_reports_cost(backend):  # tests/gradients.rs:223-361
    c = ParameterizedCircuit.new(3)
    c.rotation(RotationAxis.Y, 0, 0)
    c.rotation(RotationAxis.X, 1, 1)
    c.rotation(RotationAxis.Y, 2, 2)
    c.cnot(0, 1)
    prof = c.circuit_profile()
    assert (prof.operations, prof.parameters, prof.parameterized_operations, prof.has_channel) == (4, 3, 3, False)
    assert GradientStrategy.select(prof) == GradientStrategy.Adjoint
    est = c.gradient_auto([0.1, 0.2, 0.3], 4, Z, 0, backend=backend)
    assert est.strategy == GradientStrategy.Adjoint and est.evaluations == 2
    shift = c.gradient(GradientOptions(strategy=GradientStrategy.ParameterShift), [0.1, 0.2, 0.3], 4, Z, 0,
                       backend=backend)
    assert shift.evaluations == 6
    assert np.abs(shift.gradient - est.gradient).max() < 1e-12
    sampled = c.gradient(GradientOptions(shots=100), [0.1, 0.2, 0.3], 4, Z, 0, backend=backend)
    assert sampled.strategy == GradientStrategy.ParameterShift
    noisy = ParameterizedCircuit.new(1)
    noisy.rotation(RotationAxis.Y, 0, 0)
    noisy.channel(0, NoiseChannel.Depolarizing(0.1))
    with pytest.raises(QuantumError) as e:
        noisy.gradient_auto([0.3], 1, Z, 0, backend=backend)
    assert e.value.kind == "OperationRequiresDensityMatrix"


def test_adjoint_matches_parameter_shift_with_inputs(backend):  # tests/quantum_core.rs:91-124
    c = ParameterizedCircuit.with_inputs(2, 1)
    c.encode_rotation(RotationAxis.Y, 0, 0)
    c.rotation(RotationAxis.X, 1, 0)
    c.cnot(0, 1)
    c.rotation(RotationAxis.Z, 0, 1)
    c.rotation(RotationAxis.Y, 1, 0)
    for obs in (SingleQubitObservable.X, SingleQubitObservable.Y, SingleQubitObservable.Z):
        adj = c.adjoint_gradient_with_inputs([0.43], [0.31, -0.82], 2, obs, 1, backend=backend)
        sh = c.parameter_shift_gradient_with_inputs([0.43], [0.31, -0.82], 2, obs, 1, backend=backend)
        assert np.abs(adj - sh).max() < 1e-12


def test_parameter_validation(backend):
    c = ParameterizedCircuit.new(2)
    c.rotation(RotationAxis.Y, 0, 0)
    with pytest.raises(QuantumError) as e:
        c.adjoint_gradient([0.1], 1, Z, 0, backend=backend)
    assert e.value.kind == "InvalidParameterCount"
    with pytest.raises(QuantumError) as e:
        c.adjoint_gradient([0.1, float("nan")], 1, Z, 0, backend=backend)
    assert e.value.kind == "NonFiniteParameter"
    with pytest.raises(QuantumError) as e:
        c.adjoint_gradient([0.1, 0.2], 1, Z, 3, backend=backend)
    assert e.value.kind == "QubitOutOfRange"


# ---- Pauli-sum adjoint (VQE) ----------------------------------------------------
@pytest.mark.parametrize("n,layers,tile", [(6, 2, 0), (12, 3, 0), (12, 3, 8), (16, 2, 10)])
def test_vqe_adjoint_c128_matches_oracle(backend, n, layers, tile):
    ops, params, H = W.vqe_tfim(n, layers, seed=n)
    pc = pc_from_ops(ops, params.size)
    e_ref, g_ref = O.adjoint_uncompute(ops, n, params, H.array(), threads=8)
    for every in (0, 2 * n + n, n):
        est = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H,
                                   dtype="c128", checkpoint_every=every, exec_opts={"tile_qubits": tile},
                                   backend=backend)
        assert abs(est.expectation - e_ref) < 1e-10
        assert np.abs(est.gradient - g_ref).max() < 1e-10, every


@pytest.mark.parametrize("compiled", [False, True])
@pytest.mark.parametrize("n,layers", [(12, 4), (18, 3)])
def test_vqe_adjoint_c64_error_bound(backend, n, layers, compiled):
    """compiled: forward and backward passes as generated register-tiled
    kernels (the default from 24 qubits), else the shared-memory kernels."""
    ops, params, H = W.vqe_xxz(n, layers, seed=n)
    pc = pc_from_ops(ops, params.size)
    e_ref, g_ref = O.adjoint_uncompute(ops, n, params, H.array(), threads=8)
    eo = {"jit": True} if compiled else {"smem_tiles": True}
    for every in (0, 3 * n):
        est = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H,
                                   dtype="c64", checkpoint_every=every, exec_opts=eo, backend=backend)
        assert abs(est.expectation - e_ref) < 1e-5
        assert np.abs(est.gradient - g_ref).max() < 1e-5


@pytest.mark.parametrize("n,layers,every", [(13, 3, 0), (14, 8, 42), (16, 2, 0)])
def test_vqe_adjoint_compiled_passes_match_shared_memory_passes(backend, n, layers, every):
    """TFIM (RY.RZ + CZ ring) and XXZ (RX.RY + CNOT ring) circuits: the
    compiled dual passes give the shared-memory kernels' gradient (c64)."""
    for wl in (W.vqe_tfim(n, layers, seed=n), W.vqe_xxz(n, layers, seed=n + 1)):
        ops, params, H = wl
        pc = pc_from_ops(ops, params.size)
        res = []
        for eo in ({"jit": True}, {"smem_tiles": True}):
            res.append(gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H,
                                            dtype="c64", checkpoint_every=every, exec_opts=eo, backend=backend))
        assert abs(res[0].expectation - res[1].expectation) < 2e-6
        assert np.abs(res[0].gradient - res[1].gradient).max() < 2e-6


def test_vqe_adjoint_equals_gpu_parameter_shift_c64(backend):
    n = 14
    ops, params, H = W.vqe_tfim(n, 2, seed=1)
    pc = pc_from_ops(ops, params.size)
    adj = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, dtype="c64",
                               backend=backend)
    sh = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.ParameterShift), [], params, n, H,
                              dtype="c64", backend=backend)
    assert abs(adj.expectation - sh.expectation) < 1e-5
    assert np.abs(adj.gradient - sh.gradient).max() < 1e-5


def test_expectation_entry_point(backend):
    n = 9
    ops, params, H = W.vqe_xxz(n, 2, seed=2)
    pc = pc_from_ops(ops, params.size)
    e = pc.expectation_pauli_sum(params, n, H, backend=backend)
    assert abs(e - O.energy(ops, n, params, H.array())) < 1e-10
