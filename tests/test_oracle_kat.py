"""The oracle pinned against the reference's own known-answer tests.

Each test restates one reference test (file:line in the reference crate) on
the CPU oracle with the same constants and tolerances. These run without a
GPU.
"""
import math

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import workloads as W
from quantumforge_gb300.core import PauliSum, SmallRng

Z1 = lambda q: _abi_terms([(0, 1 << q, 1.0)])  # noqa: E731
X1 = lambda q: _abi_terms([(1 << q, 0, 1.0)])  # noqa: E731
Y1 = lambda q: _abi_terms([(1 << q, 1 << q, 1.0)])  # noqa: E731


def _abi_terms(t):
    return A.terms_array(t)


def ops(*recs):
    return A.ops_array(list(recs))


def g(gate, q, theta=0.0):
    return (A.OP_GATE, gate, q, 0, 0, theta)


def rot(axis, q, p):
    return (A.OP_ROTATION, axis, q, 0, p, 0.0)


def enc(axis, q, i):
    return (A.OP_ENCODING, axis, q, 0, i, 0.0)


def cnot(c, t):
    return (A.OP_CNOT, 0, c, t, 0, 0.0)


# ---- SmallRng (src/lib.rs:4881-4911) ----------------------------------------
def test_smallrng_seed_finaliser_matches_published_splitmix64():
    # splitmix64 with state 0 returns 0xE220A8397B1DCDAF first; SmallRng::seeded
    # runs exactly that finaliser on seed + golden-ratio increment.
    assert O.lib().qfo_rng_seeded(0) == 0xE220A8397B1DCDAF
    assert SmallRng.seeded(0).state == 0xE220A8397B1DCDAF


def test_smallrng_python_and_oracle_streams_agree():
    for seed in (0, 1, 2, 42, 721, 991, 1234, 7721, 2**64 - 1):
        a, b = SmallRng.seeded(seed), O.Rng(seed)
        for _ in range(200):
            assert a.next_u64() == b.next_u64()
        assert a.next_f64() == b.next_f64()


def test_smallrng_f64_is_53_bit():
    r = O.Rng(5)
    for _ in range(1000):
        u = r.next_f64()
        assert 0.0 <= u < 1.0
        assert u * 2**53 == int(u * 2**53)


# ---- tests/quantum_core.rs ----------------------------------------------------
def test_phase_gates_s_t_and_adjoints():  # tests/quantum_core.rs:14-46
    s2 = 1 / math.sqrt(2)
    t = O.apply(O.apply(O.zero(1), A.GATE_X, 0, 0), A.GATE_T, 0, 0)
    assert abs(t[1].real - s2) <= 1e-12 and abs(t[1].imag - s2) <= 1e-12
    inv = O.apply(O.apply(O.zero(1), A.GATE_T, 0, 0), A.GATE_TDG, 0, 0)
    assert abs(inv[0] - 1) <= 1e-12
    z = O.apply(O.zero(1), A.GATE_X, 0, 0)
    for _ in range(4):
        O.apply(z, A.GATE_T, 0, 0)
    assert abs(z[1] + 1) <= 1e-12
    s = O.apply(O.apply(O.zero(1), A.GATE_X, 0, 0), A.GATE_S, 0, 0)
    assert abs(s[1] - 1j) <= 1e-12


def test_bell_state_probabilities():  # tests/quantum_core.rs:49-64
    a = O.cnot(O.apply(O.zero(2), A.GATE_H, 0, 0), 0, 1)
    p = O.probabilities(a)
    assert np.allclose(p, [0.5, 0, 0, 0.5], atol=1e-14, rtol=0)


def test_shared_rotation_parameter_shift_accumulates_occurrences():  # tests/quantum_core.rs:79-88
    theta = 0.37
    gr = O.parameter_shift(ops(rot(A.PAULI_Y, 0, 0), rot(A.PAULI_Y, 0, 0)), 1, [theta], Z1(0))
    assert abs(gr[0] - (-2.0 * math.sin(2.0 * theta))) <= 1e-12


def test_adjoint_matches_parameter_shift_with_inputs_and_shared_parameters():  # tests/quantum_core.rs:91-124
    c = ops(enc(A.PAULI_Y, 0, 0), rot(A.PAULI_X, 1, 0), cnot(0, 1), rot(A.PAULI_Z, 0, 1), rot(A.PAULI_Y, 1, 0))
    inputs, params = [0.43], [0.31, -0.82]
    for obs in (X1(1), Y1(1), Z1(1)):
        adj = O.adjoint_stored(c, 2, params, obs, inputs=inputs)
        sh = O.parameter_shift(c, 2, params, obs, inputs=inputs)
        assert np.allclose(adj, sh, atol=1e-12, rtol=0)
    noisy = np.concatenate([c, ops((A.OP_CHANNEL, 0, 0, 0, 0, 0.0))])
    with pytest.raises(O.OracleError) as e:
        O.adjoint_stored(noisy, 2, params, Z1(0), inputs=inputs)
    assert e.value.kind == "OperationRequiresDensityMatrix"


def test_seeded_measurement_is_reproducible():  # tests/quantum_core.rs:734-745
    a = O.apply(O.zero(1), A.GATE_H, 0, 0)
    b = a.copy()
    assert O.measure(a, 0, O.Rng(1234)) == O.measure(b, 0, O.Rng(1234))


def test_circuit_shots_record_bits_and_execute_classical_conditions():  # tests/quantum_core.rs:747-766
    c = ops(g(A.GATE_H, 0), (A.OP_MEASURE, 0, 0, 0, 0, 0.0), (A.OP_COND, A.GATE_X, 1, 0, 0, 0.0, 1),
            (A.OP_MEASURE, 0, 1, 0, 1, 0.0))
    out, w = O.run_shots(c, 2, 512, 991, literal=True)
    out2, _ = O.run_shots(c, 2, 512, 991, literal=True)
    assert (out == out2).all()
    cnt = O.counts(out, w)
    assert sum(cnt.values()) == 512 and set(cnt) == {(0, 0), (1, 1)}
    with pytest.raises(O.OracleError) as e:
        O.run(c, 2)
    assert e.value.kind == "OperationRequiresShotExecution"


def test_feedforward_circuit_outcomes():  # the circuit of tests/quantum_core.rs:649-676, seed 721
    c = ops(g(A.GATE_H, 0), g(A.GATE_H, 1), (A.OP_MEASURE, 0, 0, 0, 0, 0.0), (A.OP_COND, A.GATE_X, 2, 0, 0, 0.0, 1),
            (A.OP_MEASURE, 0, 1, 0, 1, 0.0), (A.OP_MEASURE, 0, 2, 0, 2, 0.0))
    out, w = O.run_shots(c, 3, 64, 721, literal=True)
    cnt = O.counts(out, w)
    assert sum(cnt.values()) == 64
    assert set(cnt) == {(0, 0, 0), (1, 1, 1), (0, 1, 0), (1, 0, 1)}


# ---- tests/differential_anchors.rs ------------------------------------------------
@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_self_inverse_gates(n):  # tests/differential_anchors.rs:12-61
    base = O.zero(n)
    for gate in (A.GATE_X, A.GATE_H, A.GATE_Z):
        a = O.run(ops(g(gate, 0), g(gate, 0)), n)
        assert np.abs(a - base).max() < 1e-12
    if n >= 2:
        a = O.run(ops(cnot(0, 1), cnot(0, 1)), n)
        assert np.abs(a - base).max() < 1e-12


@pytest.mark.parametrize("n", range(1, 7))
def test_probabilities_sum_to_one(n):  # tests/differential_anchors.rs:63-72
    a = O.run(ops(*[g(A.GATE_H, q) for q in range(n)]), n)
    assert abs(O.probabilities(a).sum() - 1) < 1e-10


def test_bell_ghz_dj_anchors():  # tests/differential_anchors.rs:76-123
    s2 = 1 / math.sqrt(2)
    bell = O.run(ops(g(A.GATE_H, 0), cnot(0, 1)), 2)
    assert abs(bell[0].real - s2) < 1e-12 and abs(bell[3].real - s2) < 1e-12
    assert abs(bell[1]) ** 2 < 1e-24 and abs(bell[2]) ** 2 < 1e-24
    ghz = O.run(ops(g(A.GATE_H, 0), *[cnot(0, i) for i in range(1, 4)]), 4)
    assert abs(ghz[0].real - s2) < 1e-12 and abs(ghz[15].real - s2) < 1e-12
    assert all(abs(x) ** 2 < 1e-24 for x in ghz[1:15])
    dj = O.run(ops(*[g(A.GATE_H, q) for q in range(3)], *[g(A.GATE_H, q) for q in range(3)]), 3)
    assert O.probabilities(dj)[0] > 1 - 1e-10


# ---- tests/proptest_quantum_core.rs (seeded instances) -------------------------
def _random_small_circuit(seed, n, length, gates_only=False):
    r = np.random.default_rng(seed)
    recs = []
    gset = [A.GATE_H, A.GATE_X, A.GATE_Y, A.GATE_Z, A.GATE_S, A.GATE_T, A.GATE_RX, A.GATE_RY, A.GATE_RZ]
    for _ in range(length):
        a, b = int(r.integers(0, n)), int(r.integers(0, n))
        if not gates_only and r.random() < 0.5 and a != b:
            recs.append(cnot(a, b))
        else:
            gate = gset[int(r.integers(0, len(gset)))]
            recs.append(g(gate, a, float(r.uniform(-10, 10)) if gate >= A.GATE_RX else 0.0))
    return recs


@pytest.mark.parametrize("seed", range(20))
def test_unitary_circuits_preserve_norm(seed):  # tests/proptest_quantum_core.rs:22-50
    n = 1 + seed % 5
    a = O.run(ops(*_random_small_circuit(seed, n, 24)) if n > 0 else ops(), n)
    assert abs(O.norm_sqr(a) - 1) < 1e-9


@pytest.mark.parametrize("seed", range(12))
def test_shots_are_normalised_reproducible_and_tree_equals_literal(seed):  # :52-83
    n = 1 + seed % 4
    recs = _random_small_circuit(seed + 100, n, 12)
    c = ops(*recs, *[(A.OP_MEASURE, 0, q, 0, q, 0.0) for q in range(n)])
    shots = 1 + (seed * 37) % 199
    lit, w = O.run_shots(c, n, shots, seed * 7919 + 3, literal=True)
    lit2, _ = O.run_shots(c, n, shots, seed * 7919 + 3, literal=True)
    tree, w2 = O.run_shots(c, n, shots, seed * 7919 + 3)
    assert w == w2 == n
    assert (lit == lit2).all()
    assert (lit == tree).all(), "the memoised tree must reproduce the literal per-shot stream bit for bit"


# ---- tests/gradients.rs ---------------------------------------------------------
def test_ry_gradient_matches_analytic_derivative():  # tests/gradients.rs:18-48
    c, theta = ops(rot(A.PAULI_Y, 0, 0)), 0.7
    for fn in (O.parameter_shift, lambda *a: O.adjoint_stored(*a), lambda *a: O.adjoint_uncompute(*a)[1]):
        assert abs(fn(c, 1, [theta], Z1(0))[0] - (-math.sin(theta))) < 1e-10


def _seven_qubit_circuit():  # tests/gradients.rs:50-66
    recs, params = [], []
    for layer in range(3):
        for q in range(7):
            recs.append(rot(A.PAULI_Y, q, len(params)))
            params.append(0.3 + 0.1 * layer)
        for q in range(7):
            recs.append(rot(A.PAULI_X, q, len(params)))
            params.append(-0.2 + 0.05 * q)
        for q in range(6):
            recs.append(cnot(q, q + 1))
    return ops(*recs), params


def test_all_exact_strategies_agree():  # tests/gradients.rs:50-107
    c, params = _seven_qubit_circuit()
    ref = O.parameter_shift(c, 7, params, Z1(0))
    assert ref.size == 42
    assert np.abs(O.adjoint_stored(c, 7, params, Z1(0)) - ref).max() < 1e-9
    assert np.abs(O.adjoint_uncompute(c, 7, params, Z1(0))[1] - ref).max() < 1e-9


def test_shared_parameter_sums_occurrence_wise_derivatives():  # tests/gradients.rs:132-172
    c = ops(rot(A.PAULI_Y, 0, 0), rot(A.PAULI_Y, 1, 0), cnot(0, 1))
    sh = O.parameter_shift(c, 2, [0.9], Z1(1))
    adj = O.adjoint_stored(c, 2, [0.9], Z1(1))
    assert abs(sh[0] - adj[0]) < 1e-10
    single = O.parameter_shift(ops(rot(A.PAULI_Y, 0, 0), cnot(0, 1)), 2, [0.9], Z1(1))
    assert abs(sh[0] - single[0]) > 1e-3


def test_finite_difference_converges_at_second_order():  # tests/gradients.rs:174-203
    c = ops(rot(A.PAULI_Y, 0, 0), rot(A.PAULI_X, 1, 1), cnot(0, 1), rot(A.PAULI_Y, 2, 0))
    params = [0.5, -0.4]
    exact = O.parameter_shift(c, 3, params, Z1(0))
    prev = math.inf
    for step in (1e-2, 1e-3, 1e-4):
        err = np.abs(O.finite_difference(c, 3, params, Z1(0), step) - exact).max()
        assert err * 50 < prev
        prev = err
    assert prev < 1e-8


@pytest.mark.parametrize("step", [0.0, -1.0, float("nan"), float("inf")])
def test_finite_difference_step_must_be_positive_and_finite(step):  # tests/gradients.rs:205-221
    with pytest.raises(O.OracleError) as e:
        O.finite_difference(ops(rot(A.PAULI_Y, 0, 0)), 1, [0.3], Z1(0), step)
    assert e.value.kind == "InvalidFiniteDifferenceStep"


def test_shift_equals_adjoint_auto_cost_circuit():  # tests/gradients.rs:324-361
    c = ops(rot(A.PAULI_Y, 0, 0), rot(A.PAULI_X, 1, 1), rot(A.PAULI_Y, 2, 2), cnot(0, 1))
    p = [0.1, 0.2, 0.3]
    assert np.abs(O.parameter_shift(c, 4, p, Z1(0)) - O.adjoint_stored(c, 4, p, Z1(0))).max() < 1e-12


# ---- Pauli sums, QAOA and MaxCut ---------------------------------------------------
def test_pauli_sum_single_terms_match_expectation_xyz():
    c = W.random_circuit(5, 4, 11)
    a = O.run(c, 5)
    for q in range(5):
        for obs, t in ((A.PAULI_X, X1(q)), (A.PAULI_Y, Y1(q)), (A.PAULI_Z, Z1(q))):
            assert abs(O.pauli_expectation(a, t).real - O.expectation(a, obs, q)) < 1e-13


def test_pauli_sum_adjoint_matches_shift_tfim():
    c, p = W.hea_vqe(6, 2, 9)
    H = PauliSum.tfim_ring(6, 0.7).array()
    e, adj = O.adjoint_uncompute(c, 6, p, H)
    assert np.abs(adj - O.parameter_shift(c, 6, p, H)).max() < 1e-10
    assert np.abs(adj - O.adjoint_stored(c, 6, p, H)).max() < 1e-12
    assert abs(e - O.energy(c, 6, p, H)) < 1e-12


def test_maxcut_expectation_matches_brute_force():  # tests/qaoa_transfer.rs:54-70
    edges = O.random_3_regular(10, 11)
    assert abs(O.maxcut_expectation(O.zero(10), edges)) < 1e-12
    uniform = O.run(ops(*[g(A.GATE_H, q) for q in range(10)]), 10)
    assert abs(O.maxcut_expectation(uniform, edges) - 0.5 * len(edges)) < 1e-9


def test_maxcut_hamiltonian_equals_maxcut_expectation():
    edges = O.random_3_regular(8, 7)
    c = W.qaoa_maxcut(8, edges, 2, [0.3, 0.5], [0.8, 0.2])
    a = O.run(c, 8)
    assert abs(O.pauli_expectation(a, PauliSum.maxcut(edges).array()).real - O.maxcut_expectation(a, edges)) < 1e-12


@pytest.mark.parametrize("n,seed", [(8, 7), (10, 11), (12, 4), (20, 99)])
def test_random_3_regular_is_deterministic_and_valid(n, seed):  # tests/maxcut_families.rs
    e1 = O.random_3_regular(n, seed)
    assert e1 == O.random_3_regular(n, seed) == W.random_3_regular(n, seed)
    assert e1 == sorted(e1) and len(e1) == 3 * n // 2
    deg = np.zeros(n, int)
    for u, v, w in e1:
        assert u < v and w == 1.0
        deg[u] += 1
        deg[v] += 1
    assert (deg == 3).all()


def test_parallel_apply_matches_sequential_apply():
    # the OpenMP clone/map/collect restatement (rayon branch) is value-identical
    c = W.random_circuit(12, 3, 5)
    seq = O.run(c, 12, threads=0)
    par = O.run(c, 12, threads=4)
    assert np.array_equal(seq.view(np.float64), par.view(np.float64))
