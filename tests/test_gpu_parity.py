"""GPU parity: the engine's kernels against the CPU oracle on the same seeded
inputs, through the C ABI. complex128 results must match within 1e-10 (the
reference's own CUDA tests use 1e-12 for short circuits, kept where they
apply); complex64 within the f32 bound stated per test; integer outcomes
bit-exact unless a decision is reported as a tie."""
import math

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import (Circuit, Gate, NoiseChannel, PauliSum, QuantumError, RotationAxis, SmallRng, StateVector,
                                StateVectorBatch)
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import workloads as W

pytestmark = pytest.mark.gpu

C128_TOL = 1e-10
C64_TOL = 2e-6  # max |amplitude error| of f32 sweeps over a few hundred gates


def close(a, b, tol):
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= tol


# ---- the reference's CUDA tests (tests/quantum_core.rs:401-731) ---------------
def test_cuda_ry_matches_cpu_reference(backend):  # :401-421
    sv = StateVector.zero(5, backend=backend)
    sv.apply(Gate.H, 0).apply(Gate.Ry(-0.2), 3)
    cpu = O.apply(O.apply(O.zero(5), A.GATE_H, 0, 0), A.GATE_RY, -0.2, 3)
    for ax, q, th in ((A.GATE_RX, 2, 0.73), (A.GATE_RY, 4, -0.2), (A.GATE_RZ, 1, 1.1)):
        sv.apply(Gate(ax, th), q)
        O.apply(cpu, ax, th, q)
    assert close(sv.amplitudes(), cpu, 1e-12)


def test_cuda_rotation_chain_matches_cpu_reference(backend):  # tests/quantum_core.rs:401-422
    gpu = O.apply(O.apply(O.zero(5), A.GATE_H, 0, 0), A.GATE_RY, -0.2, 3)
    cpu = gpu.copy()
    got = backend.apply_rotation_chain(gpu, [(RotationAxis.X, 2, 0.73), (RotationAxis.Y, 4, -0.2), (RotationAxis.Z, 1, 1.1)])
    for g, q, t in ((A.GATE_RX, 2, 0.73), (A.GATE_RY, 4, -0.2), (A.GATE_RZ, 1, 1.1)):
        O.apply(cpu, g, t, q)
    assert close(got, cpu, 1e-12)
    assert close(backend.apply_ry(gpu, 3, 0.4), O.apply(gpu.copy(), A.GATE_RY, 0.4, 3), 1e-12)
    assert close(backend.apply_ry_chain(gpu, [(0, 0.1), (1, 0.2)]),
                 O.apply(O.apply(gpu.copy(), A.GATE_RY, 0.1, 0), A.GATE_RY, 0.2, 1), 1e-12)


def test_cuda_device_state_stays_resident_between_dispatches():  # tests/quantum_core.rs:424-446
    from quantumforge_gb300 import CudaBackend

    initial = O.apply(O.zero(4), A.GATE_H, 0, 0)
    b = CudaBackend(0)
    dev = b.upload(initial)
    dev.apply_rotation(RotationAxis.X, 2, 0.31)
    dev.apply_rotation_chain([(RotationAxis.Y, 1, -0.83), (RotationAxis.Z, 3, 1.27)])
    del b  # the state keeps its backend alive, like the reference's Arc
    want = initial.copy()
    for g, q, t in ((A.GATE_RX, 2, 0.31), (A.GATE_RY, 1, -0.83), (A.GATE_RZ, 3, 1.27)):
        O.apply(want, g, t, q)
    assert close(dev.amplitudes(), want, 1e-12)


def test_cuda_entangling_gates_match_cpu_reference(backend):  # :446-486
    cpu = O.zero(5)
    for q in range(5):
        O.apply(cpu, A.GATE_H, 0, q)
    O.apply(cpu, A.GATE_RZ, 0.37, 2)
    sv = StateVector.from_amplitudes(cpu, backend=backend)
    sv.apply_cnot(0, 4)
    O.cnot(cpu, 0, 4)
    assert close(sv.amplitudes(), cpu, 1e-12)
    sv.apply_cz(1, 3)
    O.cz(cpu, 1, 3)
    assert close(sv.amplitudes(), cpu, 1e-12)
    sv.apply_swap(0, 2)
    O.swap(cpu, 0, 2)
    assert close(sv.amplitudes(), cpu, 1e-12)


def test_cuda_executes_the_unitary_circuit_api(backend):  # :488-511
    c = Circuit()
    for gate, q in ((Gate.H, 0), (Gate.X, 1), (Gate.Y, 2), (Gate.Z, 3), (Gate.Rx(0.19), 0), (Gate.Ry(-0.57), 1),
                    (Gate.Rz(1.03), 2)):
        c.push(gate, q)
    c.cnot(0, 3)
    c.cz(1, 2)
    c.swap(0, 1)
    expected = O.run(c.ops(), 4)
    for mode in ("unfused", "fused"):
        got = backend.run_circuit(O.zero(4), c, exec_opts={"mode": mode})
        assert close(got, expected, 1e-12)


def _batch_inputs():
    inputs = [O.zero(3)]
    inputs.append(O.apply(O.apply(O.zero(3), A.GATE_X, 0, 0), A.GATE_RY, 0.31, 2))
    inputs.append(O.apply(O.apply(O.zero(3), A.GATE_H, 0, 1), A.GATE_RZ, math.pi / 2, 2))
    inputs.append(O.apply(O.apply(O.zero(3), A.GATE_X, 0, 1), A.GATE_H, 0, 2))
    return inputs


def test_cuda_batched_circuit_matches_independent_cpu_runs(backend):  # tests/quantum_core.rs:519-600
    c = Circuit()
    c.push(Gate.H, 0)
    c.push(Gate.Rx(0.19), 2)
    c.push(Gate.Ry(-0.53), 1)
    c.cnot(0, 2)
    c.cz(1, 2)
    c.swap(0, 1)
    c.push(Gate.Rz(math.pi / 2), 2)
    inputs = _batch_inputs()
    with pytest.raises(QuantumError) as e:
        backend.upload_batch([])
    assert e.value.kind == "EmptyBatch"
    with pytest.raises(QuantumError) as e:
        backend.upload_batch([O.zero(2), O.zero(3)])
    assert e.value.kind == "IncompatibleBatch"
    got = backend.run_circuit_batch(inputs, c)
    assert len(got) == len(inputs)
    for g_, st in zip(got, inputs):
        assert close(g_, O.run(c.ops(), 3, init=st), 1e-12)
    # one uniform per state in batch order from the shared SmallRng (seed 7721)
    pre = [O.apply(st.copy(), A.GATE_H, 0, 0) for st in inputs]
    cpu = [p.copy() for p in pre]
    rng_cpu = O.Rng(7721)
    want = [O.measure(a, 0, rng_cpu) for a in cpu]
    batch = backend.upload_batch(pre)
    rng_gpu = SmallRng.seeded(7721)
    assert batch.measure(0, rng_gpu) == want
    assert rng_gpu.state == rng_cpu.state.value
    for g_, a in zip(batch.download(), cpu):
        assert close(g_, a, 1e-12)


@pytest.mark.parametrize("n,size,dtype,tol", [(14, 5, "c128", C128_TOL), (10, 1000, "c128", C128_TOL),
                                              (13, 3, "c64", C64_TOL), (2, 7, "c128", 1e-12)])
def test_batch_sweeps_every_state_like_independent_runs(backend, n, size, dtype, tol):
    ops = W.random_circuit(n, 16, 5 + n, two_qubit="mixed")
    r = np.random.default_rng(n)
    states = [(lambda v: v / np.linalg.norm(v))(r.normal(size=1 << n) + 1j * r.normal(size=1 << n)) for _ in range(size)]
    batch = StateVectorBatch.from_states(states, dtype=dtype, backend=backend)
    batch.apply_ops(ops)
    got = batch.download()
    for b in sorted({0, size // 2, size - 1}):
        assert close(got[b], O.run(ops, n, init=states[b]), tol), b
    rng_gpu, rng_cpu = SmallRng.seeded(99), O.Rng(99)
    q = n - 1
    outs = batch.measure(q, rng_gpu)
    after = batch.download()
    for b in sorted({0, size // 2, size - 1}):
        a = O.run(ops, n, init=states[b])
        st = O.Rng(0)
        st.state.value = rng_cpu.state.value
        for _ in range(b):  # the uniforms of the states before b
            st.next_f64()
        assert O.measure(a, q, st) == outs[b]
        assert close(after[b], a, tol), b


def test_batch_copy_errors_and_rejected_ops(backend):
    src = StateVectorBatch.from_states(_batch_inputs(), backend=backend)
    dst = StateVectorBatch.zero(3, 4, backend=backend)
    dst.copy_from_device(src)
    for a, b in zip(dst.download(), _batch_inputs()):
        assert np.array_equal(a, b)
    with pytest.raises(QuantumError) as e:
        StateVectorBatch.zero(3, 5, backend=backend).copy_from_device(src)
    assert e.value.kind == "IncompatibleDeviceState"
    with pytest.raises(QuantumError) as e:
        StateVectorBatch.zero(3, 0, backend=backend)
    assert e.value.kind == "EmptyBatch"
    c = Circuit()
    c.channel(0, NoiseChannel.Depolarizing(0.1))
    with pytest.raises(QuantumError) as e:
        dst.run_circuit(c)
    assert e.value.kind == "OperationRequiresDensityMatrix"
    m = Circuit()
    m.measure(0, 0)
    with pytest.raises(QuantumError) as e:
        dst.run_circuit(m)
    assert e.value.kind == "OperationRequiresShotExecution"
    with pytest.raises(QuantumError) as e:
        dst.measure(3, SmallRng.seeded(1))
    assert e.value.kind == "QubitOutOfRange"
    with pytest.raises(QuantumError) as e:
        dst.apply_gate(Gate.H, 5)
    assert e.value.kind == "QubitOutOfRange"
    zero = StateVectorBatch.zero(2, 3, backend=backend)
    assert all(np.array_equal(a, O.zero(2)) for a in zero.download())


def test_cuda_resident_measurement_matches_the_cpu_reference(backend):  # :602-622
    init = O.apply(O.zero(2), A.GATE_H, 0, 1)
    cpu = init.copy()
    expected = O.measure(cpu, 1, O.Rng(342))
    sv = StateVector.from_amplitudes(init, backend=backend)
    assert sv.measure(1, SmallRng.seeded(342)) == expected
    assert close(sv.amplitudes(), cpu, 1e-12)


def _shots_vs_oracle(backend, c, n, shots, seed, dtype="c128", tie_eps=1e-12):
    """Per-shot outcomes of both shot engines against the oracle's literal
    per-shot re-simulation (run_shots_impl); a shot may differ only where a
    decision fell within tie_eps of P(1) (counted by the engine)."""
    want, w2 = O.run_shots(c.ops(), n, shots, seed, literal=True)
    for engine in ("tree", "trajectories"):
        got, width, ties = c.run_shots_packed(n, shots, seed, dtype=dtype, backend=backend, tie_eps=tie_eps,
                                              exec_opts={"shots_engine": engine})
        assert width == w2
        assert int((got != want).sum()) <= ties, (engine, int((got != want).sum()), ties)
    return got, width, ties


def test_feedforward_circuit_matches_the_reference_engine(backend):  # tests/quantum_core.rs:649-676, seed 721
    c = Circuit()
    c.push(Gate.H, 0)
    c.push(Gate.H, 1)
    c.measure(0, 0)
    c.if_classical_bit(0, 1, Gate.X, 2)
    c.measure(1, 1)
    c.measure(2, 2)
    got, width, ties = _shots_vs_oracle(backend, c, 3, 64, 721)
    assert ties == 0
    res = c.run_shots(3, 64, 721, backend=backend)
    assert sum(res.counts.values()) == 64
    assert set(res.counts) == {(0, 0, 0), (1, 1, 1), (0, 1, 0), (1, 0, 1)}


def test_classical_condition_circuit_matches_the_reference_engine(backend):  # tests/quantum_core.rs:747-766
    c = Circuit()
    c.push(Gate.H, 0)
    c.measure(0, 0)
    c.if_classical_bit(0, 1, Gate.X, 1)
    c.measure(1, 1)
    got, width, ties = _shots_vs_oracle(backend, c, 2, 512, 991)
    assert ties == 0 and set(c.run_shots(2, 512, 991, backend=backend).counts) == {(0, 0), (1, 1)}


def _mid_circuit(n, seed):
    r = np.random.default_rng(seed)
    c = Circuit.from_ops(W.random_circuit(n, 3, seed, two_qubit="mixed"))
    for k in range(4):  # a measurement, conditionals on it, more gates
        q = int(r.integers(0, n))
        c.measure(q, k)
        for _ in range(2):
            c.if_classical_bit(k, int(r.integers(0, 2)), Gate(int(r.integers(1, 12)), float(r.uniform(-3, 3))),
                               int(r.integers(0, n)))
        for op in W.random_circuit(n, 1, seed + 10 * k, two_qubit="ladder"):
            c.operations.append((int(op["kind"]), int(op["gate"]), int(op["q0"]), int(op["q1"]), 0, float(op["theta"]), 0))
    c.measure(0, 4)  # qubit 0 may already have been measured: a repeated measurement
    for q in range(1, min(n, 6)):  # a terminal block of distinct qubits
        c.measure(q, 4 + q)
    return c


# complex128 decisions equal the reference's except within 1e-12 of P(1);
# complex64 states carry f32 rounding through the collapses: window 2e-5
@pytest.mark.parametrize("n,seed,dtype,tie", [(6, 1, "c128", 1e-12), (9, 2, "c128", 1e-12), (10, 3, "c64", 2e-5),
                                              (8, 4, "c64", 2e-5)])
def test_mid_circuit_measurement_and_feed_forward_match_the_reference_engine(backend, n, seed, dtype, tie):
    c = _mid_circuit(n, seed)
    got, width, ties = _shots_vs_oracle(backend, c, n, 1500, 100 + seed, dtype=dtype, tie_eps=tie)
    assert len(set(got.tolist())) > 1


def test_repeated_measurement_repeats_the_outcome(backend):
    c = Circuit()
    c.push(Gate.H, 0)
    c.measure(0, 0)
    c.measure(0, 1)
    got, width, ties = _shots_vs_oracle(backend, c, 1, 256, 5)
    assert set(got.tolist()) <= {0, 3}


# ---- noise trajectories: run_shots_with_noise (src/lib.rs:2829-2916, 1356-1506) ----
def _noisy_vs_oracle(backend, c, n, shots, seed, dtype="c128", tie_eps=1e-12, init=None, engines=("tree", "trajectories")):
    """Per-shot outcomes of both shot engines (the branch tree of device states
    and the per-shot shared-memory trajectories) against the oracle's literal
    per-shot trajectories; a shot may differ only where a decision fell
    within tie_eps of a branch threshold (counted by the engine)."""
    want, w2 = O.run_shots(c.ops(), n, shots, seed, init=init, noise=True)
    for engine in engines:
        got, width, ties = c.run_shots_packed(n if init is None else init, shots, seed, dtype=dtype, backend=backend,
                                              tie_eps=tie_eps, noise=True, exec_opts={"shots_engine": engine})
        assert width == w2
        assert int((got != want).sum()) <= ties, (engine, int((got != want).sum()), ties)
    return got, width, ties


def test_noisy_shots_match_the_reference_engine(backend):  # tests/quantum_core.rs:678-700
    c = Circuit()
    c.push(Gate.H, 0)
    c.push(Gate.Ry(0.54), 1)
    c.cnot(0, 1)
    c.channel(0, NoiseChannel.AmplitudeDamping(0.23))
    c.channel(1, NoiseChannel.PhaseDamping(0.13))
    c.channel(0, NoiseChannel.Depolarizing(0.17))
    c.measure(0, 0)
    c.if_classical_bit(0, 1, Gate.X, 2)
    c.measure(2, 1)
    c.measure(1, 2)
    got, width, ties = _noisy_vs_oracle(backend, c, 3, 256, 9981)
    assert ties == 0
    want = O.counts(O.run_shots(c.ops(), 3, 256, 9981, noise=True)[0], 3)
    assert backend.run_circuit_shots_batched(3, c, 256, 9981).counts == want
    with pytest.raises(QuantumError) as e:
        c.run_shots(3, 1, 5, backend=backend)
    assert e.value.kind == "OperationRequiresDensityMatrix"


@pytest.mark.parametrize("gate,channel,exact", [
    (Gate.X, NoiseChannel.AmplitudeDamping(0.31), 0.69), (Gate.H, NoiseChannel.PhaseDamping(0.73), 0.5),
    (Gate.I, NoiseChannel.Depolarizing(0.6), 0.4)])
def test_noisy_shots_sample_kraus_trajectories(backend, gate, channel, exact):  # tests/quantum_core.rs:768-808
    init = O.apply(O.zero(2), gate.code, 0.0, 0)
    c = Circuit()
    c.channel(0, channel)
    c.measure(0, 0)
    c.if_classical_bit(0, 1, Gate.X, 1)
    c.measure(1, 1)
    got, width, ties = _noisy_vs_oracle(backend, c, 2, 12_000, 5, init=init)
    assert abs((got & 1).mean() - exact) < 0.025
    assert np.array_equal(got & 1, (got >> 1) & 1)


def test_thermal_damping_circuit_shots_run(backend):  # tests/noise_thermo.rs:185-203
    c = Circuit()
    c.push(Gate.H, 0)
    c.channel(0, NoiseChannel.ThermalDamping(0.2, 1.0))
    c.measure(0, 0)
    got, width, ties = _noisy_vs_oracle(backend, c, 1, 256, 7)
    res = c.run_shots_with_noise(1, 256, 7, backend=backend)
    assert sum(res.counts.values()) == 256


def _noisy_circuit(n, seed):
    r = np.random.default_rng(seed)
    c = Circuit.from_ops(W.random_circuit(n, 2, seed, two_qubit="mixed"))
    kinds = [NoiseChannel.Depolarizing, NoiseChannel.AmplitudeDamping, NoiseChannel.PhaseDamping,
             lambda g: NoiseChannel.ThermalDamping(g, float(r.uniform(0.0, 2.0)))]
    for k in range(3):
        for q in range(n):  # a noise layer
            c.channel(q, kinds[int(r.integers(0, 4))](float(r.uniform(0.02, 0.3))))
        if k == 1:  # a mid-circuit measurement and feed-forward
            c.measure(int(r.integers(0, n)), 0)
            c.if_classical_bit(0, 1, Gate.Ry(float(r.uniform(-3, 3))), int(r.integers(0, n)))
        for op in W.random_circuit(n, 1, seed + 7 * k, two_qubit="ladder"):
            c.operations.append((int(op["kind"]), int(op["gate"]), int(op["q0"]), int(op["q1"]), 0, float(op["theta"]), 0))
    for q in range(min(n, 5)):  # a terminal block
        c.measure(q, 1 + q)
    return c


@pytest.mark.parametrize("n,seed,dtype,tie", [(5, 1, "c128", 1e-12), (8, 2, "c128", 1e-12), (11, 3, "c128", 1e-12),
                                              (7, 4, "c64", 2e-5), (10, 5, "c64", 2e-5)])
def test_random_noisy_circuits_match_the_reference_engine(backend, n, seed, dtype, tie):
    c = _noisy_circuit(n, seed)
    got, width, ties = _noisy_vs_oracle(backend, c, n, 600, 300 + seed, dtype=dtype, tie_eps=tie)
    assert len(set(got.tolist())) > 1


def test_noisy_shots_normalise_the_initial_state(backend):
    r = np.random.default_rng(3)
    init = 3.0 * (r.normal(size=64) + 1j * r.normal(size=64))  # far from unit norm
    c = Circuit()
    c.channel(2, NoiseChannel.AmplitudeDamping(0.4))
    c.push(Gate.H, 1)
    for q in range(6):
        c.measure(q, q)
    _noisy_vs_oracle(backend, c, 6, 2000, 11, init=init)
    d = Circuit()  # no channel: the sampler path, normalised the same way
    d.push(Gate.H, 1)
    for q in range(6):
        d.measure(q, q)
    _noisy_vs_oracle(backend, d, 6, 2000, 12, init=init)
    with pytest.raises(QuantumError) as e:
        c.run_shots_with_noise(np.zeros(64, complex), 4, 1, backend=backend)
    assert e.value.kind == "InvalidProbability"


@pytest.mark.parametrize("channel", [NoiseChannel.Depolarizing(1.5), NoiseChannel.AmplitudeDamping(-0.1),
                                     NoiseChannel.ThermalDamping(0.1, -1.0), NoiseChannel.PhaseDamping(float("nan"))])
def test_invalid_channel_parameters_are_rejected(backend, channel):
    c = Circuit()
    c.push(Gate.H, 0)
    c.channel(0, channel)
    c.measure(0, 0)
    with pytest.raises(QuantumError) as e:
        c.run_shots_with_noise(2, 8, 1, backend=backend)
    assert e.value.kind == "InvalidProbability"


@pytest.mark.parametrize("n,dtype,tie", [(13, "c128", 1e-12), (14, "c64", 2e-5)])
def test_trajectory_engine_at_the_largest_shared_memory_state(backend, n, dtype, tie):
    c = _noisy_circuit(n, 40 + n)
    _noisy_vs_oracle(backend, c, n, 120, 17, dtype=dtype, tie_eps=tie, engines=("trajectories",))


def test_noisy_shots_over_many_branches_stay_within_memory(backend):
    """Depth-first walk: 16 qubits, 8 noise layers, 4000 shots spread over
    thousands of trajectories while at most one state per level is alive."""
    n = 16
    c = Circuit()
    for q in range(n):
        c.push(Gate.H, q)
    for layer in range(8):
        for q in range(0, n, 3):
            c.channel(q, NoiseChannel.Depolarizing(0.3))
        c.cnot(layer % n, (layer + 1) % n)
    for q in range(4):
        c.measure(q, q)
    got, width, ties = c.run_shots_packed(n, 4000, 21, backend=backend, noise=True)
    want, _ = O.run_shots(c.ops(), n, 4000, 21, noise=True)
    assert int((got != want).sum()) <= ties


# ---- random circuits -------------------------------------------------------------
@pytest.mark.parametrize("n,depth,seed", [(3, 6, 1), (8, 12, 2), (12, 20, 3), (16, 20, 4), (20, 20, 5)])
@pytest.mark.parametrize("mode", ["unfused", "fused"])
def test_random_ladder_circuit_c128(backend, n, depth, seed, mode):
    ops = W.random_circuit(n, depth, seed)
    expected = O.run(ops, n)
    sv = StateVector.zero(n, backend=backend)
    sv.apply_ops(ops, exec_opts={"mode": mode})
    assert close(sv.amplitudes(), expected, C128_TOL)


@pytest.mark.parametrize("n,seed", [(10, 11), (14, 12), (18, 13)])
@pytest.mark.parametrize("tile", [6, 8, 10, 11, 13])
def test_mixed_circuit_fused_tiles_c128(backend, n, seed, tile):
    ops = W.random_circuit(n, 12, seed, two_qubit="mixed")
    expected = O.run(ops, n)
    sv = StateVector.zero(n, backend=backend)
    sv.apply_ops(ops, exec_opts={"mode": "fused", "tile_qubits": tile})
    assert close(sv.amplitudes(), expected, C128_TOL)


@pytest.mark.parametrize("n,seed", [(12, 21), (18, 22), (20, 23)])
@pytest.mark.parametrize("mode", ["unfused", "fused"])
def test_mixed_circuit_c64(backend, n, seed, mode):
    ops = W.random_circuit(n, 20, seed, two_qubit="mixed")
    expected = O.run(ops, n)
    sv = StateVector.zero(n, dtype="c64", backend=backend)
    sv.apply_ops(ops, exec_opts={"mode": mode})
    got = sv.amplitudes()
    assert close(got, expected, C64_TOL)
    assert abs(sv.norm_sqr() - 1.0) < 1e-5


def test_every_gate_kind_on_every_qubit_position(backend):
    n = 7
    recs = []
    for gate in range(12):
        for q in range(n):
            recs.append((A.OP_GATE, gate, q, 0, 0, 0.3 + 0.1 * q if gate >= A.GATE_RX else 0.0))
    for a in range(n):
        for b in range(n):
            if a != b:
                recs.append((A.OP_CNOT, 0, a, b, 0, 0.0))
                recs.append((A.OP_GATE, A.GATE_H, a, 0, 0, 0.0))
                recs.append((A.OP_CZ, 0, a, b, 0, 0.0))
                recs.append((A.OP_SWAP, 0, a, b, 0, 0.0))
                recs.append((A.OP_GATE, A.GATE_RY, b, 0, 0, 0.2 * a))
    ops = A.ops_array(recs)
    expected = O.run(ops, n)
    for mode, tile in (("unfused", 0), ("fused", 3), ("fused", 5), ("fused", 7)):
        for dtype, tol in (("c128", C128_TOL), ("c64", C64_TOL)):
            sv = StateVector.zero(n, dtype=dtype, backend=backend)
            sv.apply_ops(ops, exec_opts={"mode": mode, "tile_qubits": tile})
            assert close(sv.amplitudes(), expected, tol), (mode, tile, dtype)


# ---- reductions ----------------------------------------------------------------
@pytest.mark.parametrize("dtype,tol", [("c128", 1e-12), ("c64", 1e-6)])
@pytest.mark.parametrize("n", [1, 2, 5, 9, 16, 21])
def test_probabilities_and_expectations(backend, dtype, tol, n):
    ops = W.random_circuit(n, 6, 40 + n, two_qubit="mixed" if n > 3 else "ladder")
    a = O.run(ops, n)
    sv = StateVector.from_amplitudes(a, dtype=dtype, backend=backend)
    assert close(sv.probabilities(), O.probabilities(a), tol)
    zs = sv.expectation_z_all()
    for q in range(n):
        assert abs(zs[q] - O.expectation(a, A.PAULI_Z, q)) < 10 * tol
        for obs in (A.PAULI_X, A.PAULI_Y, A.PAULI_Z):
            assert abs(sv.expectation(obs, q) - O.expectation(a, obs, q)) < 10 * tol
    assert abs(sv.norm_sqr() - O.norm_sqr(a)) < 10 * tol


@pytest.mark.parametrize("n", [4, 10, 17])
def test_pauli_sum_expectations(backend, n):
    ops = W.random_circuit(n, 5, 60 + n, two_qubit="mixed")
    a = O.run(ops, n)
    sv = StateVector.from_amplitudes(a, backend=backend)
    r = np.random.default_rng(n)
    rand = PauliSum()
    for _ in range(12):
        x = int(r.integers(0, 1 << n))
        z = int(r.integers(0, 1 << n))
        rand.add_term(x, z, complex(r.normal(), r.normal()))
    for H in (PauliSum.tfim_ring(n, 0.8), PauliSum.xxz_ring(n, 0.5), rand):
        got = sv.expectation_pauli_sum(H)
        want = O.pauli_expectation(a, H.array())
        assert abs(got - want) < 1e-10 * max(1.0, len(H))


# ---- sampling ---------------------------------------------------------------------
@pytest.mark.parametrize("n,seed", [(2, 991), (5, 721), (10, 42), (12, 43), (14, 44)])
def test_terminal_shots_bit_exact(backend, n, seed):
    ops = W.with_terminal_measurements(W.random_circuit(n, 10, seed), n)
    shots = 4000
    exp_packed, width = O.run_shots(ops, n, shots, seed)
    c = Circuit.from_ops(ops)
    assert np.array_equal(c.ops(), ops)
    res = c.run_shots(n, shots, seed, backend=backend, tie_eps=1e-12)
    assert res.ties == 0
    assert res.counts == O.counts(exp_packed, width)
    assert res.shots == shots


def test_sample_on_resident_state_matches_literal_reference(backend):
    n = 6
    ops = W.random_circuit(n, 8, 17)
    a = O.run(ops, n)
    meas = A.ops_array([(A.OP_MEASURE, 0, q, 0, q, 0.0) for q in (3, 0, 5, 1, 4, 2)])
    exp_packed, width = O.run_shots(meas, n, 2000, 5, init=a, literal=True)
    sv = StateVector.from_amplitudes(a, backend=backend)
    packed, ties = sv.sample([3, 0, 5, 1, 4, 2], [3, 0, 5, 1, 4, 2], 2000, 5, tie_eps=1e-12)
    assert ties == 0
    assert (packed == exp_packed).all()


def test_shot_validation(backend):
    c = Circuit()
    c.push(Gate.H, 0)
    c.measure(0, 0)
    with pytest.raises(QuantumError) as e:
        c.run_shots(1, 0, 1, backend=backend)
    assert e.value.kind == "InvalidShotCount"
    c.measure(0, 5000)
    with pytest.raises(QuantumError) as e:
        c.run_shots(1, 10, 1, backend=backend)
    assert e.value.kind == "ClassicalBitOutOfRange"


# ---- errors leave the state untouched ---------------------------------------------
def test_errors_are_typed_and_state_is_untouched(backend):
    sv = StateVector.zero(3, backend=backend)
    sv.apply(Gate.H, 0)
    before = sv.amplitudes().copy()
    with pytest.raises(QuantumError) as e:
        sv.apply(Gate.X, 3)
    assert e.value.kind == "QubitOutOfRange"
    with pytest.raises(QuantumError) as e:
        sv.apply_cnot(1, 1)
    assert e.value.kind == "InvalidQubitPair"
    bad = A.ops_array([(A.OP_GATE, A.GATE_X, 1, 0, 0, 0.0), (A.OP_CHANNEL, 0, 0, 0, 0, 0.0)])
    with pytest.raises(QuantumError) as e:
        sv.apply_ops(bad)
    assert e.value.kind == "OperationRequiresDensityMatrix"
    assert np.array_equal(sv.amplitudes(), before)
    with pytest.raises(QuantumError) as e:
        StateVector.zero(0, backend=backend)
    assert e.value.kind == "ZeroQubits"
    with pytest.raises(QuantumError) as e:
        StateVector.zero(20, memory_budget=1000, backend=backend)
    assert e.value.kind == "MemoryBudgetExceeded"


def _all_kinds_circuit(n, seed):
    """Every gate kind on every qubit and every ordered pair of a spread of
    qubits (lane, register and warp positions of the register-tiled pass)."""
    r = np.random.default_rng(seed)
    recs = []
    for gate in range(12):
        for q in range(n):
            recs.append((A.OP_GATE, gate, q, 0, 0, float(r.uniform(-3, 3)) if gate >= A.GATE_RX else 0.0))
    picks = sorted(set([0, 1, 3, 4, 5, 7, n // 2, n - 2, n - 1]))
    for a in picks:
        for b in picks:
            if a != b:
                for kind in (A.OP_CNOT, A.OP_CZ, A.OP_SWAP):
                    recs.append((kind, 0, a, b, 0, 0.0))
                    recs.append((A.OP_GATE, int(r.integers(4, 12)), int(r.integers(0, n)), 0, 0, float(r.uniform(-3, 3))))
    return A.ops_array(recs)


@pytest.mark.parametrize("n,tile", [(12, 12), (14, 12), (15, 13), (17, 12), (17, 13)])
def test_register_tiled_passes_match_oracle_and_smem_kernel(backend, n, tile):
    ops = _all_kinds_circuit(n, n * 31 + tile)
    expected = O.run(ops, n)
    sv = StateVector.zero(n, dtype="c64", backend=backend)
    sv.apply_ops(ops, exec_opts={"tile_qubits": tile})
    rs = sv.amplitudes()
    sv2 = StateVector.zero(n, dtype="c64", backend=backend)
    sv2.apply_ops(ops, exec_opts={"tile_qubits": tile, "smem_tiles": True})
    sm = sv2.amplitudes()
    assert close(rs, expected, C64_TOL)
    assert close(sm, expected, C64_TOL)


@pytest.mark.parametrize("n,seed,tile", [(12, 5, 12), (16, 6, 12), (21, 7, 12), (22, 8, 12), (22, 8, 13)])
def test_register_tiled_mixed_circuits(backend, n, seed, tile):
    """Both pass planners. The SWAPs of these circuits relabel register and
    warp positions, so some passes store through other warp qubits than they
    load: a warp that stored before another had loaded once corrupted 3 % of
    a 22-qubit state (22, 8, 12); repeated runs catch such races."""
    ops = W.random_circuit(n, 24, seed, two_qubit="mixed")
    expected = O.run(ops, n, threads=8)
    for plan in ("lookahead", "first_come"):
        for _ in range(3):
            sv = StateVector.zero(n, dtype="c64", backend=backend)
            sv.apply_ops(ops, exec_opts={"tile_qubits": tile, "plan": plan})
            assert close(sv.amplitudes(), expected, C64_TOL), plan


@pytest.mark.parametrize("n,seed,kinds", [(14, 3, True), (17, 4, False), (20, 9, False), (13, 21, True), (15, 22, True),
                                          (16, 23, True), (18, 24, True), (19, 25, False)])
def test_compiled_passes_match_oracle(backend, n, seed, kinds):
    """Passes compiled by the pass compiler (NVRTC) against the oracle, and
    a second run of the same structure with new angles (cached kernels)."""
    ops = _all_kinds_circuit(n, seed) if kinds else W.random_circuit(n, 16, seed, two_qubit="mixed")
    for trial in range(2):
        if trial == 1:  # same structure, new angles: reuses the compiled kernels
            ops = ops.copy()
            ops["theta"] = ops["theta"] * 0.7 + 0.1
        expected = O.run(ops, n, threads=8)
        sv = StateVector.zero(n, dtype="c64", backend=backend)
        sv.apply_ops(ops, exec_opts={"jit": True})
        assert close(sv.amplitudes(), expected, C64_TOL), trial


@pytest.mark.parametrize("n,seed,kinds", [(14, 41, True), (16, 42, True), (17, 43, False), (20, 44, False)])
def test_compiled_13_qubit_tiles_match_oracle(backend, n, seed, kinds):
    """Compiled forward passes on 13-qubit tiles (512 threads, 4 warp bits; the
    default for large complex64 states), with new angles on a second run."""
    ops = _all_kinds_circuit(n, seed) if kinds else W.random_circuit(n, 16, seed, two_qubit="mixed")
    for trial in range(2):
        if trial == 1:
            ops = ops.copy()
            ops["theta"] = ops["theta"] * 0.7 + 0.1
        expected = O.run(ops, n, threads=8)
        sv = StateVector.zero(n, dtype="c64", backend=backend)
        sv.apply_ops(ops, exec_opts={"jit": True, "tile_qubits": 13})
        assert close(sv.amplitudes(), expected, C64_TOL), trial


@pytest.mark.parametrize("dual", [False, True])
def test_compiled_pass_with_hundreds_of_factored_gates(backend, dual):
    """A pass of 768 gates on 12 qubits (60 layers of RY/RX and a CNOT chain):
    the scale pulled out of ~400 unitary gates is applied every 96 of them, so
    float32 neither overflows nor underflows. Forward against the oracle; the
    adjoint's dual passes (overlaps scaled by |G|^2) against the oracle's
    parameter shift."""
    r = np.random.default_rng(77)
    n, layers = 14, 60
    if not dual:
        recs = []
        for layer in range(layers):
            g = A.GATE_RY if layer % 2 == 0 else A.GATE_RX
            recs += [(A.OP_GATE, g, q, 0, 0, float(r.uniform(1.2, 1.9))) for q in range(12)]
            recs += [(A.OP_CNOT, 0, q, q + 1, 0, 0.0) for q in range(11)]
        ops = A.ops_array(recs)
        want = O.run(ops, n)
        # compiled passes; shared-memory passes (factored T_MAT1F ops with T_SCALE
        # rescaling) in complex64 and complex128
        for dtype, opts, tol in (("c64", {"jit": True}, 2e-5), ("c64", {"smem_tiles": True}, 2e-5),
                                 ("c128", {}, 1e-10)):
            sv = StateVector.zero(n, dtype=dtype, backend=backend)
            sv.apply_ops(ops, exec_opts=opts)
            got = sv.amplitudes()
            assert np.isfinite(got).all(), (dtype, opts)
            assert close(got, want, tol), (dtype, opts)
        return
    from quantumforge_gb300 import ParameterizedCircuit, RotationAxis
    from quantumforge_gb300.gradients import GradientOptions, GradientStrategy, gradient_with_inputs

    # fixed-angle RY/RX gates (factored; parameterised rotations keep the plain
    # form) between CNOT chains and the trainable rotations: 10 layers of 58
    # items (120 factored gates, 120 overlap slots) make one backward pass
    pc = ParameterizedCircuit(24)
    for layer in range(10):
        fixed = A.GATE_RY if layer % 2 == 0 else A.GATE_RX
        for q in range(12):
            pc.operations.append((A.OP_GATE, fixed, q, 0, 0, float(r.uniform(1.2, 1.9))))
        for q in range(11):
            pc.cnot(q, q + 1)
        for q in range(12):
            pc.rotation(RotationAxis.Y if layer % 2 == 0 else RotationAxis.X, q, (layer * 12 + q) % 24)
        for q in range(11):
            pc.cnot(q, q + 1)
    params = r.uniform(1.2, 1.9, 24)
    n = 12  # one 4096-amplitude tile keeps the oracle's 240 shifted runs short
    H = PauliSum()
    H.add_term(0, 1 | (1 << 11), 1.0)
    H.add_term(1 << 3, 0, 0.5)
    est = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, dtype="c64",
                               backend=backend, exec_opts={"jit": True})
    want = O.parameter_shift(pc.ops(), n, params, A.terms_array([(0, 1 | (1 << 11), 1.0), (1 << 3, 0, 0.5)]), threads=8)
    smem = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, dtype="c64",
                                backend=backend, exec_opts={"jit": False})
    assert np.isfinite(est.gradient).all()
    assert np.abs(est.gradient - want).max() < 2e-4
    assert np.abs(est.gradient - smem.gradient).max() < 2e-4


def test_state_outliving_its_context_is_released_safely(engine_lib):
    from quantumforge_gb300 import CudaBackend

    b = CudaBackend(0)
    sv = StateVector.zero(4, backend=b)
    sv.apply(Gate.H, 0)
    b.close()  # frees the state's memory and orphans the handle
    with pytest.raises(QuantumError) as e:
        sv.apply(Gate.X, 0)
    assert e.value.kind == "InvalidArgument"
    del sv  # qf_sv_destroy on an orphan must not touch the released context


@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_run_circuit_with_pinned_host_buffers(backend, dtype):
    """qf_run_circuit with page-locked f64 host amplitudes (read and written in
    place by the conversion kernels) against the oracle, and the pageable path."""
    import ctypes as C

    torch = pytest.importorskip("torch")
    from quantumforge_gb300 import _native

    n = 14
    ops = W.random_circuit(n, 8, 31, two_qubit="mixed")
    rng = np.random.default_rng(3)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    expected = O.run(ops, n, init=init)
    lib = _native.load()
    code = A.C64 if dtype == "c64" else A.C128
    tol = C64_TOL if dtype == "c64" else C128_TOL
    h_in = torch.from_numpy(init.view(np.float64).copy()).pin_memory()
    h_out = torch.empty(2 << n, dtype=torch.float64).pin_memory()
    eo = A.exec_opts(None)
    _native.check(lib.qf_run_circuit(backend.handle, n, code, _native.ptr(ops), len(ops), C.c_void_p(h_in.data_ptr()),
                                     C.c_void_p(h_out.data_ptr()), 2 << n, C.byref(eo)))
    got = h_out.numpy().view(np.complex128)
    assert close(got, expected, tol)
    out2 = np.empty(2 << n, dtype=np.float64)  # pageable buffers: staged copies
    src = np.ascontiguousarray(init).view(np.float64)
    _native.check(lib.qf_run_circuit(backend.handle, n, code, _native.ptr(ops), len(ops), _native.ptr(src),
                                     _native.ptr(out2), 2 << n, C.byref(eo)))
    assert np.array_equal(out2, h_out.numpy())


# ---- single-state trajectory steps and normalisation on a resident state -----------
@pytest.mark.parametrize("dtype,tol", [("c128", 1e-12), ("c64", 2e-6)])
def test_apply_channel_trajectory_matches_the_oracle(backend, dtype, tol):  # src/lib.rs:1356-1506
    r = np.random.default_rng(5)
    n = 9
    for trial in range(24):
        v = r.normal(size=1 << n) + 1j * r.normal(size=1 << n)
        v /= np.linalg.norm(v)
        kind = trial % 4
        p, beta, q, seed = float(r.uniform(0.05, 0.9)), float(r.uniform(0, 2)), int(r.integers(0, n)), int(r.integers(1, 1 << 40))
        ch = NoiseChannel(kind, p, beta)
        sv = StateVector.from_amplitudes(v, dtype=dtype, backend=backend)
        rng = SmallRng.seeded(seed)
        sv.apply_channel_trajectory(ch, q, rng)
        a = v.copy()
        orng = O.Rng(seed)
        O.channel_trajectory(a, kind, p, q, orng, beta)
        assert rng.state == orng.state.value
        assert close(sv.amplitudes(), a, tol), (trial, kind)
    with pytest.raises(QuantumError) as e:
        sv.apply_channel_trajectory(NoiseChannel.Depolarizing(1.5), 0, SmallRng.seeded(1))
    assert e.value.kind == "InvalidProbability"
    with pytest.raises(QuantumError) as e:
        sv.apply_channel_trajectory(NoiseChannel.Depolarizing(0.1), n, SmallRng.seeded(1))
    assert e.value.kind == "QubitOutOfRange"


def test_normalize_divides_by_the_norm(backend):  # src/lib.rs:1005-1014
    v = 3.0 * (np.arange(16) + 1j)
    sv = StateVector.from_amplitudes(v, backend=backend)
    sv.normalize()
    assert close(sv.amplitudes(), v / np.sqrt(np.vdot(v, v).real), 1e-15)
    with pytest.raises(QuantumError) as e:
        StateVector.from_amplitudes(np.zeros(4, complex), backend=backend).normalize()
    assert e.value.kind == "InvalidProbability"
