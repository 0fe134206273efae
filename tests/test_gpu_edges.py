"""Edge cases through the C ABI on the GPU: empty op lists, one-qubit states,
one shot, and the largest states this GPU holds (a 34-qubit complex64 and a
33-qubit complex128 GHZ state, 128 GiB each), checked against values the
circuit fixes exactly."""
import gc

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import (Circuit, DensityMatrix, Gate, NoiseChannel, PauliSum, SmallRng, StateVector,
                                StateVectorBatch)
from quantumforge_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def test_empty_op_lists_leave_every_kind_of_state_unchanged(backend):
    init = O.run(A.ops_array([(A.OP_GATE, A.GATE_H, 0, 0, 0, 0.0), (A.OP_GATE, A.GATE_RY, 1, 0, 0, 0.3)]), 3)
    empty = Circuit()
    assert np.array_equal(backend.run_circuit(init, empty), init)
    sv = StateVector.from_amplitudes(init, backend=backend)
    sv.apply_ops(empty.ops())
    assert np.array_equal(sv.amplitudes(), init)
    b = StateVectorBatch.from_states([init, init], backend=backend)
    b.apply_ops(empty.ops())
    assert all(np.array_equal(x, init) for x in b.download())
    rho = DensityMatrix.from_state(sv)
    empty.run_density(rho)
    assert np.abs(rho.entries() - np.outer(init, init.conj())).max() < 1e-15
    # no measurement: every shot reads the empty register
    got, width, ties = empty.run_shots_packed(3, 17, 5, backend=backend)
    assert width == 0 and not got.any() and ties == 0
    got, width, ties = empty.run_shots_packed(3, 17, 5, backend=backend, noise=True)
    assert width == 0 and not got.any()


def test_one_qubit_states_through_every_path(backend):
    c = Circuit()
    c.push(Gate.Ry(1.1), 0)
    c.channel(0, NoiseChannel.AmplitudeDamping(0.3))
    c.measure(0, 0)
    c.push(Gate.H, 0)
    c.measure(0, 1)
    want, _ = O.run_shots(c.ops(), 1, 500, 3, noise=True)
    for engine in ("tree", "trajectories"):
        got, width, ties = c.run_shots_packed(1, 500, 3, backend=backend, noise=True, tie_eps=1e-12,
                                              exec_opts={"shots_engine": engine})
        assert width == 2 and int((got != want).sum()) <= ties
    u = Circuit()
    u.push(Gate.Ry(1.1), 0)
    assert np.abs(backend.run_circuit(O.zero(1), u) - O.run(u.ops(), 1)).max() < 1e-15
    rho = DensityMatrix.zero(1, backend=backend)
    u.run_density(rho)
    assert abs(rho.probability_one(0) - np.sin(0.55) ** 2) < 1e-15
    b = StateVectorBatch.zero(1, 3, backend=backend)
    b.run_circuit(u)
    outs = b.measure(0, SmallRng.seeded(9))
    r = O.Rng(9)
    assert outs == [int(r.next_f64() < np.sin(0.55) ** 2) for _ in range(3)]


def test_a_single_shot(backend):
    c = Circuit()
    c.push(Gate.H, 0)
    c.measure(0, 0)
    c.if_classical_bit(0, 1, Gate.X, 1)
    c.measure(1, 1)
    got, width, _ = c.run_shots_packed(2, 1, 77, backend=backend)
    want, _ = O.run_shots(c.ops(), 2, 1, 77, literal=True)
    assert got.size == 1 and np.array_equal(got, want)


def _ghz(n):
    recs = [(A.OP_GATE, A.GATE_H, 0, 0, 0, 0.0)] + [(A.OP_CNOT, 0, q, q + 1, 0, 0.0) for q in range(n - 1)]
    return A.ops_array(recs)


@pytest.mark.parametrize("n,dtype", [(34, "c64"), (33, "c128")])
def test_largest_ghz_state(backend, n, dtype):
    """128 GiB of amplitudes: <Z_q> = 0, <Z_0 Z_q> = 1, norm 1, and every
    sampled register all zeros or all ones."""
    gc.collect()
    sv = StateVector.zero(n, dtype=dtype, backend=backend)
    try:
        sv.apply_ops(_ghz(n))
        tol = 1e-5 if dtype == "c64" else 1e-12
        assert abs(sv.norm_sqr() - 1.0) < tol
        z = sv.expectation_z_all()
        assert np.abs(z).max() < tol
        H = PauliSum()
        for q in (1, n // 2, n - 1):
            H.add_term(0, 1 | (1 << q), 1.0)
        assert abs(sv.expectation_pauli_sum(H).real - 3.0) < 3 * tol
        order = list(range(0, n, 2))[:16]
        packed, ties = sv.sample(order, list(range(len(order))), 4000, 11, tie_eps=1e-6)
        full = (1 << len(order)) - 1
        assert set(np.unique(packed).tolist()) <= {0, full}
        assert 1500 < int((packed == full).sum()) < 2500
    finally:
        del sv
        gc.collect()


def _inverse(ops):
    from quantumforge_gb300 import workloads as W

    return W.inverse_circuit(ops)


@pytest.mark.parametrize("plan", ["lookahead", "first_come"])
def test_headline_circuit_round_trip_at_full_size(backend, plan):
    """The 30-qubit depth-40 mixed circuit (1798 gates) and its inverse through
    the compiled complex64 passes return |0...0>: a size-independent check of
    the headline workload's planner and kernels (f32 error over 3596 gates)."""
    from quantumforge_gb300 import workloads as W

    gc.collect()
    ops = W.random_circuit(30, 40, 1, two_qubit="mixed")
    sv = StateVector.zero(30, dtype="c64", backend=backend)
    try:
        sv.apply_ops(ops, exec_opts={"plan": plan})
        z = sv.expectation_z_all()
        assert np.abs(z).max() < 0.01  # a scrambled state
        sv.apply_ops(_inverse(ops), exec_opts={"plan": plan})
        assert abs(sv.norm_sqr() - 1.0) < 1e-4
        assert np.abs(sv.expectation_z_all() - 1.0).max() < 1e-4
    finally:
        del sv
        gc.collect()
