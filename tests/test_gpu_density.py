"""GPU density matrices (qf_dm_*) against the oracle's restatement of
DensityMatrix (src/lib.rs:1551-2235): the reference's own CUDA density tests
(tests/quantum_core.rs:622-647, 702-731) at their 1e-12 tolerance, the
thermal-channel known answers (tests/noise_thermo.rs:44-124) and random noisy
circuits. complex128 entries within 1e-11 after tens of fused gates;
complex64 within 2e-6."""
import math

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import Circuit, DensityMatrix, Gate, NoiseChannel, QuantumError, SmallRng, StateVector
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def close(a, b, tol):
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= tol


def test_cuda_density_circuit_matches_cpu_gates_and_noise_channels(backend):  # tests/quantum_core.rs:702-731
    c = Circuit()
    for gate, q in ((Gate.H, 0), (Gate.Rx(0.37), 1), (Gate.Ry(-0.81), 2), (Gate.Y, 1), (Gate.Z, 2), (Gate.Rz(-0.44), 0)):
        c.push(gate, q)
    c.cnot(0, 2)
    c.cz(1, 2)
    c.swap(0, 1)
    c.channel(0, NoiseChannel.AmplitudeDamping(0.17))
    c.channel(1, NoiseChannel.PhaseDamping(0.29))
    c.channel(2, NoiseChannel.Depolarizing(0.13))
    initial = O.dm_from_state(O.zero(3))
    expected = O.run_density(c.ops(), 3, initial)
    actual = backend.run_density_circuit(initial, c)
    assert close(actual, expected, 1e-12)
    assert abs(np.trace(actual).real - 1.0) < 1e-12
    rho = backend.upload_density(initial)
    c.run_density(rho)
    assert close(rho.entries(), expected, 1e-12)
    assert abs(rho.trace().real - 1.0) < 1e-12
    assert abs(rho.purity() - O.dm_purity(expected)) < 1e-12


def test_cuda_resident_density_measurement_matches_cpu_collapse(backend):  # tests/quantum_core.rs:622-647
    psi = O.cnot(O.apply(O.apply(O.zero(3), A.GATE_H, 0.0, 0), A.GATE_RY, 0.71, 1), 1, 2)
    initial = O.dm_from_state(psi)
    cpu = initial.copy()
    expected = O.dm_measure(cpu, 1, O.Rng(8831))
    dev = backend.upload_density(initial)
    rng = SmallRng.seeded(8831)
    assert dev.measure(1, rng) == expected
    got = dev.entries()
    assert close(got, cpu, 1e-12)
    assert abs(np.trace(got).real - 1.0) < 1e-12
    r2 = O.Rng(8831)
    r2.next_f64()
    assert rng.state == r2.state.value


def test_thermal_damping_prepares_the_gibbs_state_on_the_device(backend):  # tests/noise_thermo.rs:44-79
    gd, beta = 0.10, 1.0
    gu = gd * math.exp(-beta)
    target = math.exp(-beta) / (1.0 + math.exp(-beta))
    rate = 1.0 - gu - gd
    sv = StateVector.zero(1, backend=backend)
    sv.apply(Gate.X, 0)
    rho = DensityMatrix.from_state(sv)
    ch = NoiseChannel.ThermalDamping(gd, beta)
    for step in range(21):
        assert abs(rho.probability_one(0) - (target + (1.0 - target) * rate ** step)) < 1e-12
        assert abs(rho.trace().real - 1.0) < 1e-12
        assert rho.purity() <= 1.0 + 1e-12
        rho.apply_channel(ch, 0)
    hot = DensityMatrix.from_state(sv)
    for _ in range(50):
        hot.apply_channel(NoiseChannel.ThermalDamping(0.3, 0.0), 0)
    assert abs(hot.probability_one(0) - 0.5) < 1e-12


def _noisy_density_circuit(n, seed):
    r = np.random.default_rng(seed)
    c = Circuit.from_ops(W.random_circuit(n, 2, seed, two_qubit="mixed"))
    kinds = [NoiseChannel.Depolarizing, NoiseChannel.AmplitudeDamping, NoiseChannel.PhaseDamping,
             lambda g: NoiseChannel.ThermalDamping(g, float(r.uniform(0.0, 2.0)))]
    for k in range(3):
        for q in range(n):
            if r.uniform() < 0.6:
                c.channel(q, kinds[int(r.integers(0, 4))](float(r.uniform(0.02, 0.4))))
        for op in W.random_circuit(n, 1, seed + 11 * k, two_qubit="mixed"):
            c.operations.append((int(op["kind"]), int(op["gate"]), int(op["q0"]), int(op["q1"]), 0, float(op["theta"]), 0))
    return c


@pytest.mark.parametrize("n,seed,dtype,tol", [(2, 1, "c128", 1e-12), (5, 2, "c128", 1e-11), (8, 3, "c128", 1e-11),
                                              (10, 4, "c128", 1e-11), (3, 7, "c64", 2e-6), (4, 8, "c64", 2e-6),
                                              (6, 5, "c64", 2e-6), (9, 6, "c64", 2e-6)])
@pytest.mark.parametrize("start", ["pure", "mixed"])
def test_random_noisy_density_circuits_match_the_oracle(backend, n, seed, dtype, tol, start):
    c = _noisy_density_circuit(n, seed)
    if start == "pure":
        psi = O.run(W.random_circuit(n, 2, seed + 100), n)
        init = O.dm_from_state(psi)
        sv = StateVector.from_amplitudes(psi, dtype=dtype, backend=backend)
        rho = DensityMatrix.from_state(sv)
    else:
        init = O.dm_maximally_mixed(n)
        rho = DensityMatrix.maximally_mixed(n, dtype=dtype, backend=backend)
    want = O.run_density(c.ops(), n, init)
    c.run_density(rho)
    assert close(rho.entries(), want, tol)
    assert abs(rho.trace() - O.dm_trace(want)) < tol * 4
    assert abs(rho.purity() - O.dm_purity(want)) < tol * 4
    assert close(rho.probabilities(), np.real(np.diag(want)), tol)
    for q in (0, n - 1):
        for obs in (A.PAULI_X, A.PAULI_Y, A.PAULI_Z):
            assert abs(rho.expectation(obs, q) - O.dm_expectation(want, obs, q)) < tol * 4
        assert abs(rho.probability_one(q) - O.dm_probability_one(want, q)) < tol * 4
    r_gpu, r_cpu = SmallRng.seeded(77), O.Rng(77)
    q = n // 2
    o = rho.measure(q, r_gpu)
    assert o == O.dm_measure(want, q, r_cpu)
    assert close(rho.entries(), want, tol * 4)


def test_density_errors(backend):
    rho = DensityMatrix.zero(3, backend=backend)
    m = Circuit()
    m.push(Gate.H, 0)
    m.measure(0, 0)
    with pytest.raises(QuantumError) as e:
        m.run_density(rho)
    assert e.value.kind == "OperationRequiresShotExecution"
    assert close(rho.entries(), O.dm_from_state(O.zero(3)), 0.0)  # rejected before anything ran
    for ch in (NoiseChannel.Depolarizing(1.5), NoiseChannel.ThermalDamping(0.1, -1.0)):
        with pytest.raises(QuantumError) as e:
            rho.apply_channel(ch, 0)
        assert e.value.kind == "InvalidProbability"
    with pytest.raises(QuantumError) as e:
        rho.apply_channel(NoiseChannel.AmplitudeDamping(0.1), 3)
    assert e.value.kind == "QubitOutOfRange"
    with pytest.raises(QuantumError) as e:
        rho.measure(5, SmallRng.seeded(1))
    assert e.value.kind == "QubitOutOfRange"
    with pytest.raises(QuantumError) as e:
        DensityMatrix.zero(18, backend=backend)
    assert e.value.kind == "StateTooLarge"
    with pytest.raises(QuantumError) as e:
        DensityMatrix.from_state(StateVector.zero(4, backend=backend)).apply_cnot(0, 0)
    assert e.value.kind == "InvalidQubitPair"


def _resolve(ops, params, inputs):
    """Rotation and encoding records bound to fixed gates (the oracle's run_density takes Circuit ops)."""
    out = ops.copy()
    rot = {A.PAULI_X: A.GATE_RX, A.PAULI_Y: A.GATE_RY, A.PAULI_Z: A.GATE_RZ}
    for k in range(len(out)):
        kind = int(out[k]["kind"])
        if kind in (A.OP_ROTATION, A.OP_ENCODING):
            src = params if kind == A.OP_ROTATION else inputs
            out[k]["theta"] = src[int(out[k]["param"])]
            out[k]["gate"] = rot[int(out[k]["gate"])]
            out[k]["kind"] = A.OP_GATE
            out[k]["param"] = 0
    return out


def test_noisy_parameterized_circuit_uses_density_matrix_parameter_shift(backend):  # tests/quantum_core.rs:125-182
    from quantumforge_gb300 import ParameterizedCircuit, RotationAxis

    c = ParameterizedCircuit.with_inputs(1, 1)
    c.encode_rotation(RotationAxis.Y, 0, 0)
    c.rotation(RotationAxis.X, 0, 0)
    c.channel(0, NoiseChannel.AmplitudeDamping(0.23))
    c.channel(0, NoiseChannel.Depolarizing(0.08))
    inputs, params = [0.39], np.array([0.71])
    with pytest.raises(QuantumError) as e:
        c.run_with_inputs(inputs, params, 1, backend=backend)
    assert e.value.kind == "OperationRequiresDensityMatrix"
    eps = 1e-6
    for obs in (A.PAULI_X, A.PAULI_Y, A.PAULI_Z):
        g = c.parameter_shift_gradient_density_with_inputs(inputs, params, 1, obs, 0, backend=backend)[0]
        vp = c.expectation_density_with_inputs(inputs, params + eps, 1, obs, 0, backend=backend)
        vm = c.expectation_density_with_inputs(inputs, params - eps, 1, obs, 0, backend=backend)
        assert abs(g - (vp - vm) / (2 * eps)) < 1e-8
        rho = O.run_density(_resolve(c.ops(), params, inputs), 1)
        assert abs(c.expectation_density_with_inputs(inputs, params, 1, obs, 0, backend=backend)
                   - O.dm_expectation(rho, obs, 0)) < 1e-13
    data = [([0.15], 0.62), ([0.71], -0.08), ([-0.32], 0.91)]
    _, grad = c.mse_loss_and_gradient_density(data, params, 1, A.PAULI_Z, 0, backend=backend)
    lp = c.mse_loss_and_gradient_density(data, params + eps, 1, A.PAULI_Z, 0, backend=backend)[0]
    lm = c.mse_loss_and_gradient_density(data, params - eps, 1, A.PAULI_Z, 0, backend=backend)[0]
    assert abs(grad[0] - (lp - lm) / (2 * eps)) < 1e-8


@pytest.mark.parametrize("n,dtype,tol", [(4, "c128", 1e-12), (7, "c128", 1e-11), (6, "c64", 2e-6)])
def test_density_parameter_shift_matches_the_oracle(backend, n, dtype, tol):
    from quantumforge_gb300 import ParameterizedCircuit, RotationAxis

    r = np.random.default_rng(n)
    c = ParameterizedCircuit.with_inputs(5, 2)
    for q in range(n):
        c.encode_rotation(RotationAxis.Y, q, q % 2)
    for layer in range(2):
        for q in range(n):
            c.rotation(int(r.integers(0, 3)), q, int(r.integers(0, 5)))
            c.channel(q, NoiseChannel.AmplitudeDamping(float(r.uniform(0.01, 0.2))))
        for q in range(n - 1):
            c.cnot(q, q + 1)
        c.channel(n // 2, NoiseChannel.ThermalDamping(0.1, 0.5))
    params, inputs = r.uniform(-np.pi, np.pi, 5), r.uniform(-1, 1, 2)
    g = c.parameter_shift_gradient_density_with_inputs(inputs, params, n, A.PAULI_Z, 1, dtype=dtype, backend=backend)
    ops = c.ops()
    want = np.zeros(5)
    for k in range(len(ops)):
        if int(ops[k]["kind"]) != A.OP_ROTATION:
            continue
        res = []
        for d in (np.pi / 2, -np.pi / 2):
            shifted = _resolve(ops, params, inputs)
            shifted[k]["theta"] += d
            res.append(O.dm_expectation(O.run_density(shifted, n), A.PAULI_Z, 1))
        want[int(ops[k]["param"])] += 0.5 * (res[0] - res[1])
    assert np.abs(g - want).max() < tol * 10


def test_fifteen_qubit_complex64_channel_groups_match_complex128(backend):
    """Channel groups of a 15-qubit complex64 matrix (4^15 entries, 8 GiB: more
    than 16 tile-index bits, all three bytes of the paired kernel's deposit
    tables) against the complex128 matrix, whose channels run one kernel each:
    trace, purity, P(1) and <X>, <Y>, <Z> of every qubit."""
    n = 15
    c = Circuit()
    for q in range(n):
        c.push(Gate.Ry(0.3 + 0.1 * q), q)
    for q in range(0, n - 1, 2):
        c.cnot(q, q + 1)
    kinds = (NoiseChannel.AmplitudeDamping, NoiseChannel.Depolarizing, NoiseChannel.PhaseDamping)
    for q in range(n):
        c.channel(q, kinds[q % 3](0.05 + 0.02 * q))
    for q in range(n):
        c.push(Gate.Rx(0.2 * q - 1.0), q)
    for q in range(n - 1, 0, -3):
        c.channel(q, NoiseChannel.AmplitudeDamping(0.11))
    got, want = {}, {}
    for dtype, out in (("c64", got), ("c128", want)):
        rho = DensityMatrix.zero(n, dtype=dtype, backend=backend)
        c.run_density(rho)
        out["trace"] = rho.trace().real
        out["purity"] = rho.purity()
        out["p1"] = np.array([rho.probability_one(q) for q in range(n)])
        out["xyz"] = np.array([[rho.expectation(o, q) for o in (A.PAULI_X, A.PAULI_Y, A.PAULI_Z)] for q in range(n)])
        del rho
    assert abs(want["trace"] - 1.0) < 1e-9 and abs(got["trace"] - 1.0) < 1e-5
    assert abs(got["purity"] - want["purity"]) < 1e-5 * max(1.0, want["purity"])
    assert np.abs(got["p1"] - want["p1"]).max() < 1e-5
    assert np.abs(got["xyz"] - want["xyz"]).max() < 1e-5
