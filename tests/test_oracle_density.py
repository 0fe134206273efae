"""The oracle's density-matrix restatement (DensityMatrix, src/lib.rs:1551-2235;
Circuit::run_density, src/lib.rs:2804-2818), pinned by the reference's own
tests (tests/noise_thermo.rs:44-147, tests/proptest_quantum_core.rs:143-158,
tests/quantum_core.rs:768-808) and by an independent numpy statement of
M rho M^dagger and of the Kraus sums."""
import math

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import workloads as W

DEP, AD, PD, TH = A.CHANNEL_DEPOLARIZING, A.CHANNEL_AMPLITUDE_DAMPING, A.CHANNEL_PHASE_DAMPING, A.CHANNEL_THERMAL_DAMPING


def _one():
    return O.dm_from_state(O.apply(O.zero(1), A.GATE_X, 0.0, 0))


def _plus():
    return O.dm_from_state(O.apply(O.zero(1), A.GATE_H, 0.0, 0))


def _entropy(rho):
    w = np.linalg.eigvalsh(rho)
    w = w[w > 0]
    return float(-(w * np.log(w)).sum())


def test_thermal_damping_prepares_the_gibbs_state_at_the_predicted_rate():  # tests/noise_thermo.rs:44-79
    gd, beta = 0.10, 1.0
    gu = gd * math.exp(-beta)
    target = math.exp(-beta) / (1.0 + math.exp(-beta))
    rate = 1.0 - gu - gd
    rho = _one()
    for step in range(21):
        predicted = target + (1.0 - target) * rate ** step
        assert abs(O.dm_probability_one(rho, 0) - predicted) < 1e-12
        assert abs(O.dm_trace(rho).real - 1.0) < 1e-12
        assert O.dm_purity(rho) <= 1.0 + 1e-12
        O.dm_channel(rho, TH, gd, 0, beta)
    for _ in range(200):
        O.dm_channel(rho, TH, gd, 0, beta)
    assert abs(O.dm_probability_one(rho, 0) - target) < 1e-12
    expected_entropy = -(target * math.log(target) + (1 - target) * math.log(1 - target))
    assert abs(_entropy(rho) - expected_entropy) < 1e-12


def test_thermal_damping_fixed_point_is_independent_of_the_starting_state():  # tests/noise_thermo.rs:81-96
    target = math.exp(-0.8) / (1.0 + math.exp(-0.8))
    for rho in (_one(), _plus()):
        for _ in range(400):
            O.dm_channel(rho, TH, 0.15, 0, 0.8)
        assert abs(O.dm_probability_one(rho, 0) - target) < 1e-12
        assert abs(rho[0, 1]) < 1e-12


def test_thermal_damping_interpolates_between_amplitude_damping_and_infinite_temperature():  # :98-124
    rho = _one()
    for _ in range(50):
        O.dm_channel(rho, TH, 0.3, 0, 0.0)
    assert abs(O.dm_probability_one(rho, 0) - 0.5) < 1e-12
    rho = _one()
    for _ in range(150):
        O.dm_channel(rho, TH, 0.3, 0, 40.0)
    assert O.dm_probability_one(rho, 0) < 1e-12


@pytest.mark.parametrize("kind,p,beta", [(TH, 1.5, 1.0), (TH, 0.1, -1.0), (AD, 1.2, 0.0), (PD, -0.2, 0.0),
                                         (DEP, float("nan"), 0.0)])
def test_channels_reject_invalid_parameters(kind, p, beta):  # tests/noise_thermo.rs:126-147
    with pytest.raises(O.OracleError) as e:
        O.dm_channel(_one(), kind, p, 0, beta)
    assert e.value.kind == "InvalidProbability"


def test_density_matrix_stays_normalized():  # tests/proptest_quantum_core.rs:143-158
    ops = A.ops_array([(A.OP_GATE, A.GATE_H, 0, 0, 0, 0.0), (A.OP_CNOT, 0, 0, 1, 0, 0.0)])
    rho = O.run_density(ops, 2, O.dm_maximally_mixed(2))
    assert abs(O.dm_trace(rho).real - 1.0) < 1e-9


@pytest.mark.parametrize("gate,kind,p,exact", [(A.GATE_X, AD, 0.31, 0.69), (A.GATE_H, PD, 0.73, 0.5),
                                               (A.GATE_I, DEP, 0.6, 0.4)])
def test_channel_populations_of_the_shot_reference(gate, kind, p, exact):  # tests/quantum_core.rs:768-808
    rho = O.dm_from_state(O.apply(O.zero(2), gate, 0.0, 0))
    ops = A.ops_array([A.channel_record(kind, 0, p)])
    assert abs(O.dm_probability_one(O.run_density(ops, 2, rho), 0) - exact) < 1e-12


def test_unitary_circuits_match_the_outer_product_of_the_state_vector():
    n = 4
    ops = W.random_circuit(n, 6, 3, two_qubit="mixed")
    psi = O.run(ops, n)
    rho = O.run_density(ops, n)
    assert np.abs(rho - np.outer(psi, psi.conj())).max() < 1e-12
    assert abs(O.dm_purity(rho) - 1.0) < 1e-12
    for q in range(n):
        for obs in (A.PAULI_X, A.PAULI_Y, A.PAULI_Z):
            assert abs(O.dm_expectation(rho, obs, q) - O.expectation(psi, obs, q)) < 1e-12


def _kraus(kind, p, beta):
    s = math.sqrt
    if kind == DEP:
        X = np.array([[0, 1], [1, 0]], complex)
        Y = np.array([[0, -1j], [1j, 0]])
        Z = np.diag([1.0, -1.0]).astype(complex)
        return [s(1 - p) * np.eye(2)] + [s(p / 3) * P for P in (X, Y, Z)]
    if kind == AD:
        return [np.diag([1.0, s(1 - p)]).astype(complex), np.array([[0, s(p)], [0, 0]], complex)]
    if kind == PD:
        return [np.diag([1.0, s(1 - p)]).astype(complex), np.diag([0.0, s(p)]).astype(complex)]
    gu = p * math.exp(-beta)
    return [np.diag([s(1 - gu), s(1 - p)]).astype(complex), np.array([[0, s(p)], [0, 0]], complex),
            np.array([[0, 0], [s(gu), 0]], complex)]


def _lift(M, q, n):
    out = np.array([[1.0]], complex)
    for k in reversed(range(n)):
        out = np.kron(out, M if k == q else np.eye(2))
    return out


@pytest.mark.parametrize("seed", range(4))
def test_channels_and_gates_match_an_independent_kraus_statement(seed):
    r = np.random.default_rng(seed)
    n = 3
    v = r.normal(size=(1 << n, 4)) + 1j * r.normal(size=(1 << n, 4))
    rho = v @ v.conj().T
    rho /= np.trace(rho)
    for kind in (DEP, AD, PD, TH):
        p, beta, q = float(r.uniform(0.05, 0.9)), float(r.uniform(0, 2)), int(r.integers(0, n))
        want = sum(_lift(K, q, n) @ rho @ _lift(K, q, n).conj().T for K in _kraus(kind, p, beta))
        got = O.dm_channel(rho.copy(), kind, p, q, beta)
        assert np.abs(got - want).max() < 1e-13, kind
    U = O.gate_matrix(A.GATE_RY, 0.37)
    got = O.dm_apply(rho.copy(), A.GATE_RY, 0.37, 1)
    assert np.abs(got - _lift(U, 1, n) @ rho @ _lift(U, 1, n).conj().T).max() < 1e-13


def test_measurement_collapses_both_sides_and_renormalises():
    psi = O.apply(O.apply(O.zero(3), A.GATE_H, 0.0, 0), A.GATE_RY, 0.71, 1)
    psi = O.cnot(psi, 1, 2)
    rho = O.dm_from_state(psi)
    o = O.dm_measure(rho, 1, O.Rng(8831))
    assert abs(O.dm_trace(rho).real - 1.0) < 1e-12
    idx = np.arange(8)
    wrong = ((idx >> 1) & 1) != o
    assert np.all(rho[wrong, :] == 0) and np.all(rho[:, wrong] == 0)
