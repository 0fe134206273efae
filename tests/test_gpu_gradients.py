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


def _shots_circuit(n):
    r = np.random.default_rng(40 + n)
    c = ParameterizedCircuit.with_inputs(4, 2)
    for q in range(n):
        c.encode_rotation(RotationAxis.Y, q, q % 2)
    for layer in range(2):
        for q in range(n):
            c.rotation(int(r.integers(0, 3)), q, int(r.integers(0, 4)))
        for q in range(n - 1):
            c.cnot(q, q + 1)
    return c, r.uniform(-np.pi, np.pi, 4), r.uniform(-1, 1, 2)


@pytest.mark.parametrize("n", [1, 5, 9])
def test_shot_estimates_match_the_oracle_draw_for_draw(backend, n):  # src/lib.rs:3361-3479, 4806-4838
    """complex128: every shot's outcome is the oracle's literal
    clone-and-measure outcome, so estimates and gradients are equal."""
    from quantumforge_gb300 import ShotConfig

    c, params, inputs = _shots_circuit(n)
    ops = c.ops()
    shots, seed = 3000, 1234 + n
    for obs in (A.PAULI_X, A.PAULI_Y, A.PAULI_Z):
        q = n - 1
        est, (lo, hi) = c.expectation_with_inputs_shots_with_ci(inputs, params, n, obs, q, ShotConfig(shots, seed),
                                                                backend=backend)
        ok = O.estimate_observable_shots(O.run(ops, n, params, inputs), obs, q, shots, seed)
        assert est == 2.0 * ok / shots - 1.0
        assert lo <= est <= hi and hi - lo < 0.1
        assert c.expectation_with_inputs_shots(inputs, params, n, obs, q, ShotConfig(shots, seed), backend=backend) == est
        g = c.parameter_shift_gradient_with_inputs_shots(inputs, params, n, obs, q, ShotConfig(shots, seed),
                                                         backend=backend)
        want = np.zeros(4)
        for k in range(len(ops)):
            if int(ops[k]["kind"]) != A.OP_ROTATION:
                continue
            e = []
            for sh, sd in ((np.pi / 2, seed + 2 * k), (-np.pi / 2, seed + 2 * k + 1)):
                okk = O.estimate_observable_shots(O.run(ops, n, params, inputs, shift_op=k, shift=sh), obs, q, shots, sd)
                e.append(2.0 * okk / shots - 1.0)
            want[int(ops[k]["param"])] += 0.5 * (e[0] - e[1])
        assert np.array_equal(g, want)
        exact = c.parameter_shift_gradient_with_inputs(inputs, params, n, obs, q, backend=backend)
        assert np.abs(g - exact).max() < 0.2


def test_shot_estimates_validate_like_the_reference(backend):
    from quantumforge_gb300 import ShotConfig

    c, params, inputs = _shots_circuit(3)
    for call in (lambda: c.expectation_with_inputs_shots(inputs, params, 3, Z, 0, ShotConfig(0, 1), backend=backend),
                 lambda: c.parameter_shift_gradient_with_inputs_shots(inputs, params, 3, Z, 0, ShotConfig(0, 1),
                                                                      backend=backend),
                 lambda: c.expectation_density_with_inputs_shots(inputs, params, 3, Z, 0, ShotConfig(0, 1),
                                                                 backend=backend),
                 lambda: c.parameter_shift_gradient_density_with_inputs_shots(inputs, params, 3, Z, 0,
                                                                              ShotConfig(0, 1), backend=backend)):
        with pytest.raises(QuantumError) as e:
            call()
        assert e.value.kind == "InvalidShotCount"
    with pytest.raises(QuantumError) as e:
        c.expectation_with_inputs_shots(inputs, params, 3, Z, 3, ShotConfig(10, 1), backend=backend)
    assert e.value.kind == "QubitOutOfRange"
    # complex64 state: the same draws, outcomes equal except within float32 distance of P(1)
    est64 = c.expectation_with_inputs_shots(inputs, params, 3, Z, 1, ShotConfig(4000, 9), dtype="c64", backend=backend)
    est128 = c.expectation_with_inputs_shots(inputs, params, 3, Z, 1, ShotConfig(4000, 9), backend=backend)
    assert abs(est64 - est128) <= 2 * 3 / 4000


def test_density_shot_estimates_sample_the_exact_expectation(backend):  # src/lib.rs:3188-3320, 4840-4850
    from quantumforge_gb300 import ShotConfig, sample_expectation

    c, params, inputs = _shots_circuit(4)
    c.channel(2, NoiseChannel.AmplitudeDamping(0.2))
    c.rotation(RotationAxis.X, 2, 3)
    c.channel(1, NoiseChannel.Depolarizing(0.05))
    sc = ShotConfig(5000, 77)
    exact = c.expectation_density_with_inputs(inputs, params, 4, A.PAULI_Z, 2, backend=backend)
    est, (lo, hi) = c.expectation_density_with_inputs_shots_with_ci(inputs, params, 4, A.PAULI_Z, 2, sc,
                                                                   backend=backend)
    assert est == sample_expectation(exact, sc)
    assert c.expectation_density_with_inputs_shots(inputs, params, 4, A.PAULI_Z, 2, sc, backend=backend) == est
    assert lo <= exact <= hi
    g = c.parameter_shift_gradient_density_with_inputs_shots(inputs, params, 4, A.PAULI_Z, 2, sc, backend=backend)
    ops = c.ops()
    want = np.zeros(4)
    for k in range(len(ops)):
        if int(ops[k]["kind"]) != A.OP_ROTATION:
            continue
        e = []
        for sh, sd in ((np.pi / 2, 77 + 2 * k), (-np.pi / 2, 77 + 2 * k + 1)):
            ex = _density_shifted(c, params, inputs, k, sh)
            e.append(sample_expectation(ex, ShotConfig(5000, sd)))
        want[int(ops[k]["param"])] += 0.5 * (e[0] - e[1])
    assert np.abs(g - want).max() < 1e-12
    exact_g = c.parameter_shift_gradient_density_with_inputs(inputs, params, 4, A.PAULI_Z, 2, backend=backend)
    assert np.abs(g - exact_g).max() < 0.15


def _density_shifted(c, params, inputs, k, shift):
    """Exact density expectation <Z_2> with rotation occurrence k shifted, from the oracle."""
    ops = c.ops().copy()
    rot = {A.PAULI_X: A.GATE_RX, A.PAULI_Y: A.GATE_RY, A.PAULI_Z: A.GATE_RZ}
    for j in range(len(ops)):
        kind = int(ops[j]["kind"])
        if kind in (A.OP_ROTATION, A.OP_ENCODING):
            src = params if kind == A.OP_ROTATION else inputs
            ops[j]["theta"] = src[int(ops[j]["param"])] + (shift if j == k else 0.0)
            ops[j]["gate"] = rot[int(ops[j]["gate"])]
            ops[j]["kind"] = A.OP_GATE
            ops[j]["param"] = 0
    return O.dm_expectation(O.run_density(ops, 4), A.PAULI_Z, 2)


def test_shot_mse_composes_the_per_sample_estimates(backend):  # src/lib.rs:3802-3927
    from quantumforge_gb300 import ShotConfig

    c, params, _ = _shots_circuit(3)
    data = [([0.1, -0.4], 0.3), ([0.7, 0.2], -0.5), ([-0.9, 0.5], 0.05)]
    sc = ShotConfig(2000, 31)
    for dens in (False, True):
        f = c.mse_loss_and_gradient_density_shots if dens else c.mse_loss_and_gradient_shots
        pred = c.expectation_density_with_inputs_shots if dens else c.expectation_with_inputs_shots
        grad = c.parameter_shift_gradient_density_with_inputs_shots if dens else c.parameter_shift_gradient_with_inputs_shots
        loss, g = f(data, params, 3, Z, 0, sc, backend=backend)
        want_l, want_g = 0.0, np.zeros(4)
        for k, (x, y) in enumerate(data):
            s = 31 + k * 0x9E3779B9
            r = pred(x, params, 3, Z, 0, ShotConfig(2000, s), backend=backend) - y
            want_l += r * r
            want_g += 2 * r * grad(x, params, 3, Z, 0, ShotConfig(2000, s + 1), backend=backend)
        assert loss == want_l / 3 and np.array_equal(g, want_g / 3)
