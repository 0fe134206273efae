"""The oracle's noise trajectories (apply_channel_trajectory, src/lib.rs:1356-1506)
and run_shots_with_noise (src/lib.rs:2829-2916), pinned by the reference's
own statistical tests (tests/quantum_core.rs:768-808,
tests/noise_thermo.rs:149-203) and by a second, pure-Python restatement of
the trajectory arithmetic that must agree with the C oracle bit for bit."""
import math

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import _abi as A
from quantumforge_gb300.core import SmallRng

DEP, AD, PD, TH = A.CHANNEL_DEPOLARIZING, A.CHANNEL_AMPLITUDE_DAMPING, A.CHANNEL_PHASE_DAMPING, A.CHANNEL_THERMAL_DAMPING
EPS = 2.220446049250313e-16


def ops(*recs):
    return A.ops_array(list(recs))


def g(gate, q, theta=0.0):
    return (A.OP_GATE, gate, q, 0, 0, theta)


def meas(q, c):
    return (A.OP_MEASURE, 0, q, 0, c, 0.0)


def cond(c, v, gate, q):
    return (A.OP_COND, gate, q, 0, c, 0.0, v)


def _density_p1(rho0, kind, p, beta=0.0):
    """P(1) on qubit 0 after the channel, from its Kraus operators (one qubit)."""
    if kind == DEP:
        X = np.array([[0, 1], [1, 0]], complex)
        Y = np.array([[0, -1j], [1j, 0]])
        Z = np.diag([1.0, -1.0]).astype(complex)
        rho = (1 - p) * rho0 + p / 3 * sum(P @ rho0 @ P.conj().T for P in (X, Y, Z))
    elif kind in (AD, PD):
        K0 = np.diag([1.0, math.sqrt(1 - p)]).astype(complex)
        K1 = (np.array([[0, math.sqrt(p)], [0, 0]], complex) if kind == AD
              else np.diag([0.0, math.sqrt(p)]).astype(complex))
        rho = K0 @ rho0 @ K0.conj().T + K1 @ rho0 @ K1.conj().T
    else:
        gu = p * math.exp(-beta)
        rho = np.zeros((2, 2), complex)
        rho[1, 1] = rho0[1, 1] * (1 - p) + rho0[0, 0] * gu
        rho[0, 0] = 1 - rho[1, 1]
    return rho[1, 1].real


@pytest.mark.parametrize("gate,kind,p,exact", [
    (A.GATE_X, AD, 0.31, 0.69), (A.GATE_H, PD, 0.73, 0.5), (A.GATE_I, DEP, 0.6, 0.4)])
def test_noisy_shots_sample_kraus_trajectories(gate, kind, p, exact):  # tests/quantum_core.rs:768-808
    init = O.apply(O.zero(2), gate, 0, 0)
    a1 = init[:2]
    rho0 = np.outer(a1, a1.conj())
    assert _density_p1(rho0, kind, p) == pytest.approx(exact, abs=1e-12)
    c = ops(A.channel_record(kind, 0, p), meas(0, 0), cond(0, 1, A.GATE_X, 1), meas(1, 1))
    with pytest.raises(O.OracleError) as e:
        O.run_shots(c, 2, 1, 5, init=init, literal=True)
    assert e.value.kind == "OperationRequiresDensityMatrix"
    out, w = O.run_shots(c, 2, 12_000, 5, init=init, noise=True)
    out2, _ = O.run_shots(c, 2, 12_000, 5, init=init, noise=True)
    assert np.array_equal(out, out2) and w == 2
    bits0 = (out & 1).astype(int)
    assert abs(bits0.mean() - exact) < 0.025
    assert np.array_equal(bits0, ((out >> 1) & 1).astype(int))


def test_thermal_damping_trajectories_reproduce_the_channel():  # tests/noise_thermo.rs:149-183
    gd, beta = 0.20, 0.70
    gu = gd * math.exp(-beta)
    expected = 0.5 * (1.0 - gd) + 0.5 * gu
    plus = np.array([1.0, 1.0], complex) / math.sqrt(2.0)
    total = 0.0
    for seed in range(1, 20_001):
        a = plus.copy()
        O.channel_trajectory(a, TH, gd, 0, O.Rng(seed), beta)
        assert abs(np.vdot(a, a).real - 1.0) < 1e-12
        total += abs(a[1]) ** 2
    assert abs(total / 20_000 - expected) < 0.02


def test_thermal_damping_circuit_shots_run():  # tests/noise_thermo.rs:185-203
    c = ops(g(A.GATE_H, 0), A.channel_record(TH, 0, 0.2, 1.0), meas(0, 0))
    out, w = O.run_shots(c, 1, 256, 7, noise=True)
    assert out.size == 256 and w == 1


@pytest.mark.parametrize("kind,p,beta", [(DEP, 1.5, 0.0), (DEP, float("nan"), 0.0), (AD, -0.1, 0.0), (PD, 2.0, 0.0),
                                         (TH, 1.1, 0.5), (TH, 0.1, -1.0), (TH, 0.1, float("inf"))])
def test_invalid_channel_parameters_are_rejected(kind, p, beta):  # validate_probability, thermal_rates
    a = O.zero(2)
    with pytest.raises(O.OracleError) as e:
        O.channel_trajectory(a, kind, p, 0, O.Rng(1), beta)
    assert e.value.kind == "InvalidProbability"


def test_channel_on_a_missing_qubit_is_rejected():
    with pytest.raises(O.OracleError) as e:
        O.channel_trajectory(O.zero(2), AD, 0.1, 2, O.Rng(1))
    assert e.value.kind == "QubitOutOfRange"


def test_noisy_shots_normalise_the_initial_state():  # run_shots_impl: state.normalize() when allow_noise
    init = np.array([3.0, 4.0], complex)  # |3|^2 + |4|^2 = 25
    c = ops(A.channel_record(AD, 0, 0.0), meas(0, 0))
    out, _ = O.run_shots(c, 1, 4000, 3, init=init, noise=True)
    assert abs((out & 1).mean() - 16 / 25) < 0.03
    with pytest.raises(O.OracleError) as e:
        O.run_shots(c, 1, 1, 3, init=np.zeros(2, complex), noise=True)
    assert e.value.kind == "InvalidProbability"


def test_damping_extremes_take_the_only_branch_with_weight():
    # from |1>, AD with gamma = 1 always jumps; the no-jump branch (norm 1 - 1 = 0) is never taken
    a = O.apply(O.zero(1), A.GATE_X, 0, 0)
    O.channel_trajectory(a, AD, 1.0, 0, O.Rng(4))
    assert np.array_equal(a, np.array([1.0, 0.0], complex))
    # from |0>, PD with gamma = 1 never jumps; norm of the kept branch is 1
    b = O.zero(1)
    O.channel_trajectory(b, PD, 1.0, 0, O.Rng(4))
    assert np.array_equal(b, np.array([1.0, 0.0], complex))


# ---- a second restatement in Python, sequential sums, no fused operations ----
def _seq_sum(vals):
    s = -0.0
    for v in vals:
        s += v
    return s


def _ns(z):
    return z.real * z.real + z.imag * z.imag


def _mulf(z, s):
    return complex(z.real * s, z.imag * s)


def _py_trajectory(a, kind, p, beta, q, rng):
    dim = len(a)
    mask = 1 << q
    if kind == DEP:
        u = rng.next_f64()
        if u >= 1.0 - p and p > 0.0:
            b = min(int(math.floor((u - (1.0 - p)) * (3.0 / p))), 2)
            gate = (A.GATE_X, A.GATE_Y, A.GATE_Z)[b]
            arr = np.array(a, complex)
            arr = O.apply(arr, gate, 0.0, q)
            a[:] = list(arr)
        return
    norm = _seq_sum(_ns(z) for z in a)
    p_one = _seq_sum(_ns(a[i]) for i in range(dim) if i & mask)
    if kind in (AD, PD):
        jp = min(1.0, max(0.0, p * p_one / norm))
        jump = rng.next_f64() < jp
        bn = p * p_one if jump else norm - p * p_one
        inv = 1.0 / math.sqrt(bn)
        if jump:
            sc = math.sqrt(p) * inv
            for base in range(dim):
                if base & mask:
                    continue
                v = _mulf(a[base | mask], sc)
                a[base], a[base | mask] = (v, 0j) if kind == AD else (0j, v)
        else:
            es = math.sqrt(1.0 - p) * inv
            for i in range(dim):
                a[i] = _mulf(a[i], es if i & mask else inv)
        return
    gu = p * math.exp(-beta)
    p1 = min(1.0, max(0.0, p_one / norm))
    p0 = 1.0 - p1
    down, up = p1 * p, p0 * gu
    stay = p0 * (1.0 - gu) + p1 * (1.0 - p)
    u = rng.next_f64()
    br, bn = (1, down) if u < down else ((2, up) if u < down + up else (0, stay))
    inv = 1.0 / math.sqrt(bn)
    if br == 1:
        sc = math.sqrt(p) * inv
        for base in range(dim):
            if not base & mask:
                a[base], a[base | mask] = _mulf(a[base | mask], sc), 0j
    elif br == 2:
        sc = math.sqrt(gu) * inv
        for base in range(dim):
            if not base & mask:
                a[base | mask], a[base] = _mulf(a[base], sc), 0j
    else:
        gs, es = math.sqrt(1.0 - gu) * inv, math.sqrt(1.0 - p) * inv
        for i in range(dim):
            a[i] = _mulf(a[i], es if i & mask else gs)


@pytest.mark.parametrize("seed", range(6))
def test_c_and_python_restatements_agree_bit_for_bit(seed):
    rng = np.random.default_rng(seed)
    n = 4
    for trial in range(40):
        v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        v /= np.linalg.norm(v)
        kind = int(rng.integers(0, 4))
        p = float(rng.uniform(0.05, 0.95))
        beta = float(rng.uniform(0.0, 2.0))
        q = int(rng.integers(0, n))
        s = int(rng.integers(0, 2**63))
        a = v.copy()
        O.channel_trajectory(a, kind, p, q, O.Rng(s), beta)
        b = list(v)
        _py_trajectory(b, kind, p, beta, q, SmallRng.seeded(s))
        assert np.array_equal(a.view(np.float64), np.array(b, complex).view(np.float64)), (trial, kind)
