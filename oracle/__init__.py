"""CPU oracle — TEST INFRASTRUCTURE ONLY.

ctypes wrapper over ``oracle/_build/libqf_oracle.so``, the plain-C restatement
of the reference's complex128 CPU simulator (see qf_oracle.h). Only the
test-suite, the smoke check and the benchmark's CPU legs use it, and only as
the reference the engine's results are compared with and as the timed CPU
baseline; the engine never links or calls it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libqf_oracle.so"
_lib = None

P = C.c_void_p
U32, U64, I64, F64 = C.c_uint32, C.c_uint64, C.c_int64, C.c_double


def build() -> Path:
    subprocess.run(["make", "-C", str(HERE), "-s"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        sig = {
            "qfo_rng_seeded": ([U64], U64),
            "qfo_rng_next_u64": ([C.POINTER(U64)], U64),
            "qfo_rng_next_f64": ([C.POINTER(U64)], F64),
            "qfo_gate_matrix": ([C.c_int, F64, P], C.c_int),
            "qfo_sv_zero": ([P, U32], C.c_int),
            "qfo_sv_apply": ([P, U32, C.c_int, F64, U32, C.c_int], C.c_int),
            "qfo_sv_apply_cnot": ([P, U32, U32, U32], C.c_int),
            "qfo_sv_apply_cz": ([P, U32, U32, U32], C.c_int),
            "qfo_sv_apply_swap": ([P, U32, U32, U32], C.c_int),
            "qfo_sv_norm_sqr": ([P, U32], F64),
            "qfo_sv_probabilities": ([P, U32, P], None),
            "qfo_sv_expectation": ([P, U32, C.c_int, U32, C.POINTER(F64)], C.c_int),
            "qfo_sv_measure": ([P, U32, U32, C.POINTER(U64), C.POINTER(C.c_uint8)], C.c_int),
            "qfo_sv_expectation_pauli_sum": ([P, U32, P, U64, P], C.c_int),
            "qfo_run_ops": ([P, U32, P, U64, P, U64, P, U64, I64, F64, C.c_int], C.c_int),
            "qfo_run_shots_literal": ([P, U32, P, U64, U64, U64, P, C.POINTER(U32)], C.c_int),
            "qfo_run_shots_noisy_literal": ([P, U32, P, U64, U64, U64, P, C.POINTER(U32)], C.c_int),
            "qfo_sv_normalize": ([P, U32], C.c_int),
            "qfo_sv_channel_trajectory": ([P, U32, C.c_int, F64, F64, U32, C.POINTER(U64)], C.c_int),
            "qfo_run_shots_tree": ([P, U32, P, U64, U64, U64, P, C.POINTER(U32), C.c_int], C.c_int),
            "qfo_dm_from_state": ([P, U32, P], None),
            "qfo_dm_maximally_mixed": ([U32, P], None),
            "qfo_dm_apply": ([P, U32, C.c_int, F64, U32], C.c_int),
            "qfo_dm_apply_2q": ([P, U32, C.c_int, U32, U32], C.c_int),
            "qfo_dm_apply_channel": ([P, U32, C.c_int, F64, F64, U32], C.c_int),
            "qfo_dm_trace": ([P, U32, P], None),
            "qfo_dm_purity": ([P, U32], F64),
            "qfo_dm_expectation": ([P, U32, C.c_int, U32, C.POINTER(F64)], C.c_int),
            "qfo_dm_probability_one": ([P, U32, U32, C.POINTER(F64)], C.c_int),
            "qfo_dm_measure": ([P, U32, U32, C.POINTER(U64), C.POINTER(C.c_uint8)], C.c_int),
            "qfo_run_density": ([P, U32, P, U64], C.c_int),
            "qfo_estimate_observable_shots": ([P, U32, C.c_int, U32, U64, U64, C.POINTER(U64)], C.c_int),
            "qfo_parameter_shift_gradient": ([U32, P, U64, P, U64, P, U64, P, U64, P, C.c_int], C.c_int),
            "qfo_finite_difference_gradient": ([U32, P, U64, P, U64, P, U64, P, U64, F64, P, C.c_int], C.c_int),
            "qfo_adjoint_gradient_stored": ([U32, P, U64, P, U64, P, U64, P, U64, P], C.c_int),
            "qfo_adjoint_gradient_uncompute": ([U32, P, U64, P, U64, P, U64, P, U64, C.POINTER(F64), P, C.c_int], C.c_int),
            "qfo_expectation": ([U32, P, U64, P, U64, P, U64, P, U64, C.POINTER(F64), C.c_int], C.c_int),
            "qfo_maxcut_expectation": ([P, U32, P, P, U64], F64),
            "qfo_random_3_regular": ([U32, U64, P], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


class OracleError(Exception):
    def __init__(self, status: int):
        from quantumforge_gb300._abi import STATUS_NAMES

        self.status = status
        self.kind = STATUS_NAMES.get(status, str(status))
        super().__init__(self.kind)


def _chk(st: int) -> None:
    if st:
        raise OracleError(st)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a if a is not None else [], dtype=np.float64)


# ---- SmallRng ---------------------------------------------------------------
class Rng:
    def __init__(self, seed: int):
        self.state = U64(lib().qfo_rng_seeded(seed))

    def next_u64(self) -> int:
        return lib().qfo_rng_next_u64(C.byref(self.state))

    def next_f64(self) -> float:
        return lib().qfo_rng_next_f64(C.byref(self.state))


def gate_matrix(gate: int, theta: float = 0.0) -> np.ndarray:
    out = np.zeros(8)
    _chk(lib().qfo_gate_matrix(gate, theta, _p(out)))
    return out.view(np.complex128).reshape(2, 2)


# ---- state vectors (complex128 numpy arrays) ---------------------------------
def zero(n: int) -> np.ndarray:
    a = np.zeros(1 << n, dtype=np.complex128)
    a[0] = 1
    return a


def apply(a: np.ndarray, gate: int, theta: float, q: int, threads: int = 0) -> np.ndarray:
    n = a.size.bit_length() - 1
    _chk(lib().qfo_sv_apply(_p(a), n, gate, theta, q, threads))
    return a


def cnot(a, c, t):
    _chk(lib().qfo_sv_apply_cnot(_p(a), a.size.bit_length() - 1, c, t))
    return a


def cz(a, x, y):
    _chk(lib().qfo_sv_apply_cz(_p(a), a.size.bit_length() - 1, x, y))
    return a


def swap(a, x, y):
    _chk(lib().qfo_sv_apply_swap(_p(a), a.size.bit_length() - 1, x, y))
    return a


def run(ops: np.ndarray, n: int, params=None, inputs=None, init=None, threads: int = 0, shift_op: int = -1,
        shift: float = 0.0) -> np.ndarray:
    a = zero(n) if init is None else np.array(init, dtype=np.complex128)
    p, i = _f64(params), _f64(inputs)
    _chk(lib().qfo_run_ops(_p(a), n, _p(ops), len(ops), _p(p), p.size, _p(i), i.size, shift_op, shift, threads))
    return a


def probabilities(a) -> np.ndarray:
    out = np.empty(a.size)
    lib().qfo_sv_probabilities(_p(a), a.size.bit_length() - 1, _p(out))
    return out


def norm_sqr(a) -> float:
    return lib().qfo_sv_norm_sqr(_p(a), a.size.bit_length() - 1)


def expectation(a, obs: int, q: int) -> float:
    v = F64()
    _chk(lib().qfo_sv_expectation(_p(a), a.size.bit_length() - 1, obs, q, C.byref(v)))
    return v.value


def measure(a, q: int, rng: Rng) -> int:
    o = C.c_uint8()
    _chk(lib().qfo_sv_measure(_p(a), a.size.bit_length() - 1, q, C.byref(rng.state), C.byref(o)))
    return o.value


def channel_trajectory(a, kind: int, p: float, q: int, rng: Rng, beta_delta: float = 0.0) -> None:
    """apply_channel_trajectory in place on `a` (one draw from `rng`)."""
    _chk(lib().qfo_sv_channel_trajectory(_p(a), a.size.bit_length() - 1, kind, p, beta_delta, q, C.byref(rng.state)))


def normalize(a) -> None:
    _chk(lib().qfo_sv_normalize(_p(a), a.size.bit_length() - 1))


def pauli_expectation(a, terms: np.ndarray) -> complex:
    out = np.zeros(2)
    _chk(lib().qfo_sv_expectation_pauli_sum(_p(a), a.size.bit_length() - 1, _p(terms), len(terms), _p(out)))
    return complex(out[0], out[1])


def run_shots(ops, n, shots, seed, init=None, literal=False, threads=0, noise=False):
    """Circuit::run_shots (noise=False) or run_shots_with_noise (noise=True,
    always the literal per-shot form): (packed outcomes, register width)."""
    a = zero(n) if init is None else np.ascontiguousarray(init, dtype=np.complex128)
    out = np.zeros(shots, dtype=np.uint64)
    w = U32()
    if noise:
        _chk(lib().qfo_run_shots_noisy_literal(_p(a), n, _p(ops), len(ops), shots, seed, _p(out), C.byref(w)))
    elif literal:
        _chk(lib().qfo_run_shots_literal(_p(a), n, _p(ops), len(ops), shots, seed, _p(out), C.byref(w)))
    else:
        _chk(lib().qfo_run_shots_tree(_p(a), n, _p(ops), len(ops), shots, seed, _p(out), C.byref(w), threads))
    return out, w.value


def counts(packed: np.ndarray, width: int) -> dict:
    vals, cnts = np.unique(packed, return_counts=True)
    return dict(sorted({tuple(int((int(v) >> b) & 1) for b in range(width)): int(c) for v, c in zip(vals, cnts)}.items()))


# ---- density matrices (row-major D x D complex128) ---------------------------
def _dm_n(rho) -> int:
    return int(rho.shape[0]).bit_length() - 1


def dm_from_state(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128)
    rho = np.empty((a.size, a.size), dtype=np.complex128)
    lib().qfo_dm_from_state(_p(a), a.size.bit_length() - 1, _p(rho))
    return rho


def dm_maximally_mixed(n: int) -> np.ndarray:
    rho = np.empty((1 << n, 1 << n), dtype=np.complex128)
    lib().qfo_dm_maximally_mixed(n, _p(rho))
    return rho


def dm_apply(rho, gate: int, theta: float, q: int) -> np.ndarray:
    _chk(lib().qfo_dm_apply(_p(rho), _dm_n(rho), gate, theta, q))
    return rho


def dm_apply_2q(rho, kind: int, a: int, b: int) -> np.ndarray:
    _chk(lib().qfo_dm_apply_2q(_p(rho), _dm_n(rho), kind, a, b))
    return rho


def dm_channel(rho, kind: int, p: float, q: int, beta_delta: float = 0.0) -> np.ndarray:
    _chk(lib().qfo_dm_apply_channel(_p(rho), _dm_n(rho), kind, p, beta_delta, q))
    return rho


def dm_trace(rho) -> complex:
    out = np.zeros(2)
    lib().qfo_dm_trace(_p(rho), _dm_n(rho), _p(out))
    return complex(out[0], out[1])


def dm_purity(rho) -> float:
    return lib().qfo_dm_purity(_p(rho), _dm_n(rho))


def dm_expectation(rho, observable: int, q: int) -> float:
    v = F64()
    _chk(lib().qfo_dm_expectation(_p(rho), _dm_n(rho), observable, q, C.byref(v)))
    return v.value


def dm_probability_one(rho, q: int) -> float:
    v = F64()
    _chk(lib().qfo_dm_probability_one(_p(rho), _dm_n(rho), q, C.byref(v)))
    return v.value


def dm_measure(rho, q: int, rng: Rng) -> int:
    o = C.c_uint8()
    _chk(lib().qfo_dm_measure(_p(rho), _dm_n(rho), q, C.byref(rng.state), C.byref(o)))
    return o.value


def run_density(ops, n: int, rho=None) -> np.ndarray:
    """Circuit::run_density from `rho` (default |0...0><0...0|)."""
    if rho is None:
        rho = dm_from_state(zero(n))
    rho = np.ascontiguousarray(rho, dtype=np.complex128).copy()
    _chk(lib().qfo_run_density(_p(rho), n, _p(ops), len(ops)))
    return rho


def estimate_observable_shots(a, observable: int, q: int, shots: int, seed: int) -> int:
    """Outcome-0 count of `shots` literal measurements (src/lib.rs:4806-4838)."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    ok = U64()
    _chk(lib().qfo_estimate_observable_shots(_p(a), a.size.bit_length() - 1, observable, q, shots, seed, C.byref(ok)))
    return ok.value


# ---- gradients --------------------------------------------------------------
def parameter_shift(ops, n, params, terms, inputs=None, threads=0):
    p, i = _f64(params), _f64(inputs)
    g = np.zeros(p.size)
    _chk(lib().qfo_parameter_shift_gradient(n, _p(ops), len(ops), _p(p), p.size, _p(i), i.size, _p(terms), len(terms),
                                            _p(g), threads))
    return g


def finite_difference(ops, n, params, terms, step, inputs=None, threads=0):
    p, i = _f64(params), _f64(inputs)
    g = np.zeros(p.size)
    _chk(lib().qfo_finite_difference_gradient(n, _p(ops), len(ops), _p(p), p.size, _p(i), i.size, _p(terms), len(terms),
                                              step, _p(g), threads))
    return g


def adjoint_stored(ops, n, params, terms, inputs=None):
    p, i = _f64(params), _f64(inputs)
    g = np.zeros(p.size)
    _chk(lib().qfo_adjoint_gradient_stored(n, _p(ops), len(ops), _p(p), p.size, _p(i), i.size, _p(terms), len(terms), _p(g)))
    return g


def adjoint_uncompute(ops, n, params, terms, inputs=None, threads=0):
    p, i = _f64(params), _f64(inputs)
    g = np.zeros(p.size)
    e = F64()
    _chk(lib().qfo_adjoint_gradient_uncompute(n, _p(ops), len(ops), _p(p), p.size, _p(i), i.size, _p(terms), len(terms),
                                              C.byref(e), _p(g), threads))
    return e.value, g


def energy(ops, n, params, terms, inputs=None, threads=0) -> float:
    p, i = _f64(params), _f64(inputs)
    e = F64()
    _chk(lib().qfo_expectation(n, _p(ops), len(ops), _p(p), p.size, _p(i), i.size, _p(terms), len(terms), C.byref(e),
                               threads))
    return e.value


def maxcut_expectation(a, edges) -> float:
    uv = np.ascontiguousarray([[u, v] for u, v, _ in edges], dtype=np.uint32).reshape(-1)
    w = np.ascontiguousarray([w for _, _, w in edges], dtype=np.float64)
    return lib().qfo_maxcut_expectation(_p(a), a.size.bit_length() - 1, _p(uv), _p(w), len(edges))


def random_3_regular(n: int, seed: int):
    uv = np.zeros(3 * n, dtype=np.uint32)
    _chk(lib().qfo_random_3_regular(n, seed, _p(uv)))
    return [(int(uv[2 * e]), int(uv[2 * e + 1]), 1.0) for e in range(3 * n // 2)]
