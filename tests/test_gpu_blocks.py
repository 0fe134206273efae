"""k-qubit dense-block fusion (qf_exec_opts.block_qubits = 2..5) against the
oracle: the gates of each tile pass are multiplied into dense blocks on the
host in f64 and applied as one 2^m x 2^m matrix per block. Every engine that
runs blocks is checked: the compiled register passes (complex64, k <= 4), the
tensor-core pass (complex64, k = 5), the shared-memory interpreter (complex64
with `blocks_engine="simt"` or small states, and complex128). Tolerances:
complex128 1e-10 (the reference's precision), complex64 5e-6 absolute
(3xTF32 tensor-core products and f32 sums over up to 32 terms)."""
import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import StateVector
from quantumforge_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = {"c64": 5e-6, "c128": 1e-10}


@pytest.mark.parametrize("dtype", ["c64", "c128"])
@pytest.mark.parametrize("k", [2, 3, 4, 5])
@pytest.mark.parametrize("n", [3, 7, 13])
def test_blocks_match_oracle(backend, dtype, k, n):
    ops = W.random_circuit(n, 8, 40 + n + k, two_qubit="mixed")
    want = O.run(ops, n)
    sv = StateVector.zero(n, dtype=dtype, backend=backend)
    sv.apply_ops(ops, exec_opts={"block_qubits": k})
    err = float(np.abs(sv.amplitudes() - want).max())
    assert err < TOL[dtype], (dtype, k, n, err)


@pytest.mark.parametrize("k", [2, 3, 4])
def test_compiled_block_passes_match_oracle(backend, k):
    """complex64 blocks of up to 4 qubits in the compiled register passes
    (several 4096-amplitude tiles per pass)."""
    n = 15
    ops = W.random_circuit(n, 10, 70 + k, two_qubit="mixed")
    want = O.run(ops, n)
    sv = StateVector.zero(n, dtype="c64", backend=backend)
    sv.apply_ops(ops, exec_opts={"block_qubits": k, "jit": True})
    err = float(np.abs(sv.amplitudes() - want).max())
    assert err < TOL["c64"], (k, err)
    # new angles, same structure: the compiled kernels are reused with new constants
    ops2 = ops.copy()
    ops2["theta"] = ops2["theta"] * 0.5 + 0.1
    sv2 = StateVector.zero(n, dtype="c64", backend=backend)
    sv2.apply_ops(ops2, exec_opts={"block_qubits": k, "jit": True})
    assert float(np.abs(sv2.amplitudes() - O.run(ops2, n)).max()) < TOL["c64"]


@pytest.mark.parametrize("engine", ["auto", "simt"])
def test_five_qubit_blocks_match_oracle(backend, engine):
    """complex64 blocks of 5 qubits: tensor cores (auto) and the FP32
    interpreter (simt), on states of several tiles."""
    for n, seed in ((12, 5), (15, 6), (17, 7)):
        ops = W.random_circuit(n, 10, seed, two_qubit="mixed")
        want = O.run(ops, n)
        sv = StateVector.zero(n, dtype="c64", backend=backend)
        sv.apply_ops(ops, exec_opts={"block_qubits": 5, "blocks_engine": engine})
        err = float(np.abs(sv.amplitudes() - want).max())
        assert err < TOL["c64"], (engine, n, err)


def test_blocks_keep_the_state_normalised_at_scale(backend):
    """A 26-qubit circuit, forward then inverse with 5- and 4-qubit blocks:
    back to |0...0> (the oracle cannot run this size)."""
    n = 26
    ops = W.random_circuit(n, 12, 9, two_qubit="mixed")
    inv = W.inverse_circuit(ops)
    for k in (4, 5):
        sv = StateVector.zero(n, dtype="c64", backend=backend)
        sv.apply_ops(ops, exec_opts={"block_qubits": k})
        sv.apply_ops(inv, exec_opts={"block_qubits": k})
        a = sv.amplitudes()
        assert abs(a[0] - 1.0) < 1e-4 and float(np.abs(a[1:]).max()) < 1e-4, k


def test_autotuner_picks_a_runnable_fastest_option(backend):
    """The execution autotuner times every candidate (per-gate passes, 13-qubit
    tiles, fusion widths 2..5) and returns the fastest; the choice reproduces
    the oracle's state."""
    from quantumforge_gb300.autotune import autotune_exec

    n = 16
    ops = W.random_circuit(n, 6, 12, two_qubit="mixed")
    best, times = autotune_exec(ops, n, backend=backend, reps=1)
    assert len(times) >= 4 and min(times.values()) > 0
    sv = StateVector.zero(n, dtype="c64", backend=backend)
    sv.apply_ops(ops, exec_opts=best)
    assert float(np.abs(sv.amplitudes() - O.run(ops, n)).max()) < TOL["c64"]
