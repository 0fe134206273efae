"""Host-side pieces of the Python mirror that need no GPU: the counts map of
ShotResult, NoiseChannel records and the package's exported names."""
import math

import numpy as np
import pytest

import oracle as O
import quantumforge_gb300 as qf
from quantumforge_gb300 import _abi as A
from quantumforge_gb300.core import NoiseChannel, ShotResult


def test_shot_result_counts_are_lsb_first_and_sorted_like_the_btreemap():
    r = ShotResult.from_packed(np.array([1, 2, 3, 1, 0], dtype=np.uint64), 2, ties=1)
    assert r.shots == 5 and r.ties == 1
    assert list(r.counts.items()) == [((0, 0), 1), ((0, 1), 1), ((1, 0), 2), ((1, 1), 1)]
    empty = ShotResult.from_packed(np.zeros(3, dtype=np.uint64), 0)
    assert empty.counts == {(): 3}


def test_noise_channel_records():
    rec = NoiseChannel.ThermalDamping(0.2, 0.7).record(3)
    assert rec[:3] == (A.OP_CHANNEL, A.CHANNEL_THERMAL_DAMPING, 3) and rec[5] == 0.2
    bits = (rec[4] << 32) | rec[3]
    assert np.uint64(bits).view(np.float64) == 0.7
    assert NoiseChannel.Depolarizing(0.1).record(0) == (A.OP_CHANNEL, A.CHANNEL_DEPOLARIZING, 0, 0, 0, 0.1)
    up, down = NoiseChannel.ThermalDamping(0.2, 0.7).thermal_rates()
    assert down == 0.2 and up == 0.2 * math.exp(-0.7)
    assert NoiseChannel.AmplitudeDamping(0.3).thermal_rates() is None
    c = qf.Circuit()
    c.channel(1, NoiseChannel.PhaseDamping(0.25))
    assert qf.Circuit.from_ops(c.ops()).ops().tobytes() == c.ops().tobytes()


def test_package_exports():
    for name in ("Circuit", "NoiseChannel", "StateVector", "StateVectorBatch", "ShotResult", "CudaBackend"):
        assert hasattr(qf, name), name


def test_wilson_interval_matches_the_reference_formula():  # src/lib.rs:2493-2513
    from quantumforge_gb300 import wilson_ci

    assert wilson_ci(0, 0, 0.95) == (0.0, 1.0)
    lo, hi = wilson_ci(5, 10, 0.95)
    assert abs(lo - 0.2365895936154873) < 1e-15 and abs(hi - 0.7634104063845127) < 1e-15
    lo, hi = wilson_ci(10, 10, 0.95)
    assert hi == 1.0 and 0.7 < lo < 0.73
    # the z of each confidence band: 2.576, 1.96, 1.645, and 1.96 below 0.90
    widths = [wilson_ci(50, 100, c)[1] - wilson_ci(50, 100, c)[0] for c in (0.99, 0.95, 0.90, 0.5)]
    assert widths[0] > widths[1] > widths[2] and widths[3] == widths[1]


def test_sample_expectation_draws_the_seeded_stream():  # src/lib.rs:4840-4850
    from quantumforge_gb300 import QuantumError, ShotConfig, sample_expectation

    for e, shots, seed in [(0.3, 1000, 5), (-1.0, 7, 0), (1.0, 10, 3), (0.0, 4321, 2**64 - 1), (1.7, 9, 1)]:
        r = O.Rng(seed)
        p = min(max((1 + e) / 2, 0.0), 1.0)
        k = sum(r.next_f64() < p for _ in range(shots))
        assert sample_expectation(e, ShotConfig(shots, seed)) == 2 * k / shots - 1
    with pytest.raises(QuantumError) as err:
        sample_expectation(0.2, ShotConfig(0, 1))
    assert err.value.kind == "InvalidShotCount"


def test_op_arrays_are_cached_read_only_and_follow_edits():
    """Circuit.ops() / ParameterizedCircuit.ops() return one read-only record
    array while the operation list is unchanged, rebuilt after any edit, equal
    byte for byte to a record-by-record construction."""
    def by_record(records):
        arr = np.zeros(len(records), dtype=A.OP_DTYPE)
        for i, r in enumerate(records):
            arr[i] = (r[0], r[1], r[6] if len(r) > 6 else 0, r[2], r[3], r[4], r[5])
        return arr

    c = qf.Circuit()
    assert c.ops().shape == (0,)
    c.operations.append((A.OP_GATE, A.GATE_H, 0, 0, 0, 0.0))
    c.operations.append((A.OP_CNOT, 0, 0, 1, 0, 0.0))
    c.channel(1, NoiseChannel.Depolarizing(0.1))
    a = c.ops()
    assert c.ops() is a and not a.flags.writeable
    assert a.tobytes() == by_record(c.operations).tobytes()
    with pytest.raises(ValueError):
        a[0]["q0"] = 3
    c.operations.append((A.OP_GATE, A.GATE_X, 1, 0, 0, 0.0))
    b = c.ops()
    assert b is not a and len(b) == 4 and b.tobytes() == by_record(c.operations).tobytes()
    c.operations[0] = (A.OP_GATE, A.GATE_Z, 1, 0, 0, 0.0)
    assert int(c.ops()[0]["gate"]) == A.GATE_Z and int(c.ops()[0]["q0"]) == 1
    del c.operations[1]
    assert c.ops().tobytes() == by_record(c.operations).tobytes()

    pc = qf.ParameterizedCircuit(2)
    pc.operations.append((A.OP_ROTATION, A.PAULI_Y, 0, 0, 0, 0.0))
    pc.operations.append((A.OP_ROTATION, A.PAULI_Z, 0, 0, 1, 0.0))
    p = pc.ops()
    assert pc.ops() is p and p.tobytes() == by_record(pc.operations).tobytes()
    pc.operations.pop()
    assert len(pc.ops()) == 1
