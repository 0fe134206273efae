"""Host-side pieces of the Python mirror that need no GPU: the counts map of
ShotResult, NoiseChannel records and the package's exported names."""
import math

import numpy as np

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
