"""Reference-shaped API over the GB300 engine.

Names, argument meaning and errors follow the reference crate's
``StateVector`` (src/lib.rs:928-1351), ``Gate`` (src/lib.rs:2239-2382),
``Circuit`` (src/lib.rs:2384-2916), ``ParameterizedCircuit``
(src/lib.rs:2919-3704, 4651-4740) and ``cuda::CudaBackend``
(src/cuda.rs:515-1484). Every state lives in device memory; every operation
is a call through the C ABI of include/qf.h.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._native import QuantumError, check, load, ptr

_DTYPES = {"c64": _abi.C64, "complex64": _abi.C64, "c128": _abi.C128, "complex128": _abi.C128,
           _abi.C64: _abi.C64, _abi.C128: _abi.C128}


def _dtype_code(dtype) -> int:
    try:
        return _DTYPES[dtype]
    except KeyError:
        raise QuantumError(_abi.STATUS_CODES["InvalidArgument"], f"unknown dtype {dtype!r}") from None


# ---------------------------------------------------------------------------
# SmallRng (src/lib.rs:4881-4911) — host generator for measure()
# ---------------------------------------------------------------------------
_M64 = (1 << 64) - 1


class SmallRng:
    """xorshift64 with a splitmix64 seed finaliser, bit-identical to the reference."""

    __slots__ = ("state",)

    def __init__(self, state: int):
        self.state = state & _M64

    @classmethod
    def seeded(cls, seed: int) -> "SmallRng":
        z = (seed + 0x9E3779B97F4A7C15) & _M64
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        z ^= z >> 31
        return cls(z if z else 0x9E3779B97F4A7C15)

    def next_u64(self) -> int:
        x = self.state
        x ^= (x << 13) & _M64
        x ^= x >> 7
        x ^= (x << 17) & _M64
        self.state = x
        return x

    def next_f64(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))


# ---------------------------------------------------------------------------
# Gates
# ---------------------------------------------------------------------------
class Gate:
    """`enum Gate` (src/lib.rs:2239-2264): I X Y Z H S Sdg T Tdg, Rx/Ry/Rz(theta)."""

    __slots__ = ("code", "theta")

    def __init__(self, code: int, theta: float = 0.0):
        self.code = int(code)
        self.theta = float(theta)

    @staticmethod
    def Rx(theta: float) -> "Gate":
        return Gate(_abi.GATE_RX, theta)

    @staticmethod
    def Ry(theta: float) -> "Gate":
        return Gate(_abi.GATE_RY, theta)

    @staticmethod
    def Rz(theta: float) -> "Gate":
        return Gate(_abi.GATE_RZ, theta)

    def params(self) -> list[float]:
        return [self.theta] if self.code >= _abi.GATE_RX else []

    def matrix(self) -> np.ndarray:
        """Gate::matrix (src/lib.rs:2267-2333) as a 2x2 complex128 array."""
        s = 0.7071067811865476
        c = self.code
        t = self.theta
        if c == _abi.GATE_RX:
            co, si = math.cos(t * 0.5), math.sin(t * 0.5)
            return np.array([[co, -1j * si], [-1j * si, co]])
        if c == _abi.GATE_RY:
            co, si = math.cos(t * 0.5), math.sin(t * 0.5)
            return np.array([[co, -si], [si, co]], dtype=complex)
        if c == _abi.GATE_RZ:
            h = t * 0.5
            return np.array([[complex(math.cos(h), -math.sin(h)), 0], [0, complex(math.cos(h), math.sin(h))]])
        table = {
            _abi.GATE_I: [[1, 0], [0, 1]], _abi.GATE_X: [[0, 1], [1, 0]], _abi.GATE_Y: [[0, -1j], [1j, 0]],
            _abi.GATE_Z: [[1, 0], [0, -1]], _abi.GATE_H: [[s, s], [s, -s]], _abi.GATE_S: [[1, 0], [0, 1j]],
            _abi.GATE_SDG: [[1, 0], [0, -1j]], _abi.GATE_T: [[1, 0], [0, complex(s, s)]],
            _abi.GATE_TDG: [[1, 0], [0, complex(s, -s)]],
        }
        return np.array(table[c], dtype=complex)

    def __eq__(self, other) -> bool:
        return isinstance(other, Gate) and self.code == other.code and self.theta == other.theta

    def __hash__(self) -> int:
        return hash((self.code, self.theta))

    def __repr__(self) -> str:
        name = _abi.GATE_NAMES[self.code]
        return f"{name}({self.theta})" if self.code >= _abi.GATE_RX else name


for _i, _n in enumerate(_abi.GATE_NAMES[:9]):
    setattr(Gate, _n, Gate(_i))


class RotationAxis:
    """`enum RotationAxis` (src/lib.rs:2919-2928)."""

    X, Y, Z = _abi.PAULI_X, _abi.PAULI_Y, _abi.PAULI_Z


class SingleQubitObservable:
    """`enum SingleQubitObservable` (src/lib.rs:2930-2938)."""

    X, Y, Z = _abi.PAULI_X, _abi.PAULI_Y, _abi.PAULI_Z


# ---------------------------------------------------------------------------
# Pauli sums (PauliWord / PauliSum semantics, src/analytic.rs:2547-2830)
# ---------------------------------------------------------------------------
class PauliSum:
    """sum_t c_t P_t with P_t given by (x-mask, z-mask); Y = both bits set."""

    def __init__(self, terms=None):
        self.terms: list[tuple[int, int, complex]] = []
        for t in terms or []:
            self.add_term(*t)

    def add_term(self, xmask: int, zmask: int, coeff) -> "PauliSum":
        self.terms.append((int(xmask), int(zmask), complex(coeff)))
        return self

    def add_word(self, word: dict, coeff) -> "PauliSum":
        """Add c * prod_q P_q for word = {qubit: 'X'|'Y'|'Z'}."""
        x = z = 0
        for q, p in word.items():
            p = p.upper()
            if p in ("X", "Y"):
                x |= 1 << q
            if p in ("Z", "Y"):
                z |= 1 << q
        return self.add_term(x, z, coeff)

    @classmethod
    def single(cls, observable: int, qubit: int) -> "PauliSum":
        return cls().add_word({qubit: "XYZ"[observable]}, 1.0)

    @classmethod
    def tfim_ring(cls, n: int, h: float = 1.0) -> "PauliSum":
        """-sum Z_i Z_{i+1 mod n} - h sum X_i."""
        s = cls()
        for i in range(n):
            s.add_word({i: "Z", (i + 1) % n: "Z"}, -1.0)
        for i in range(n):
            s.add_word({i: "X"}, -h)
        return s

    @classmethod
    def xxz_ring(cls, n: int, delta: float = 0.5) -> "PauliSum":
        """sum (X_i X_{i+1} + Y_i Y_{i+1} + delta Z_i Z_{i+1}) on a ring."""
        s = cls()
        for i in range(n):
            j = (i + 1) % n
            s.add_word({i: "X", j: "X"}, 1.0)
            s.add_word({i: "Y", j: "Y"}, 1.0)
            s.add_word({i: "Z", j: "Z"}, delta)
        return s

    @classmethod
    def maxcut(cls, edges) -> "PauliSum":
        """sum_(u,v,w) w (1 - Z_u Z_v) / 2 — maxcut_expectation (src/qaoa_transfer.rs:199-218)."""
        s = cls()
        total = 0.0
        for u, v, w in edges:
            total += w
            s.add_word({u: "Z", v: "Z"}, -0.5 * w)
        s.add_term(0, 0, 0.5 * total)
        return s

    def array(self) -> np.ndarray:
        return _abi.terms_array(self.terms)

    def __len__(self) -> int:
        return len(self.terms)


def _as_terms(obs) -> np.ndarray:
    if isinstance(obs, PauliSum):
        return obs.array()
    if isinstance(obs, np.ndarray) and obs.dtype == _abi.TERM_DTYPE:
        return np.ascontiguousarray(obs)
    return _abi.terms_array(list(obs))


# ---------------------------------------------------------------------------
# Backend / context
# ---------------------------------------------------------------------------
class CudaBackend:
    """`cuda::CudaBackend::new(ordinal)` (src/cuda.rs:556-790): one device, one stream."""

    def __init__(self, ordinal: int = 0):
        lib = load()
        h = C.c_void_p()
        check(lib.qf_ctx_create(int(ordinal), C.byref(h)))
        self._h = h
        self.ordinal = ordinal

    @property
    def handle(self):
        return self._h

    def synchronize(self) -> None:
        check(load().qf_ctx_synchronize(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            load().qf_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_ordinal(self) -> int:
        return self.ordinal

    # CudaBackend::upload / run_circuit / run_circuit_shots (src/cuda.rs:844, 1050, 1088)
    def upload(self, amplitudes, dtype="c128") -> "StateVector":
        return StateVector.from_amplitudes(amplitudes, dtype=dtype, backend=self)

    def run_circuit(self, state: "StateVector | np.ndarray", circuit: "Circuit", dtype="c128", exec_opts=None) -> np.ndarray:
        amps = state.amplitudes() if isinstance(state, StateVector) else np.asarray(state, dtype=np.complex128)
        n = int(round(math.log2(amps.size)))
        ops = circuit.ops()
        src = np.ascontiguousarray(amps, dtype=np.complex128).view(np.float64)
        out = np.empty(2 * amps.size, dtype=np.float64)
        check(load().qf_run_circuit(self._h, n, _dtype_code(dtype), ptr(ops), len(ops), ptr(src), ptr(out), out.size,
                                    _exec(exec_opts)))
        return out.view(np.complex128)

    # CudaBackend::apply_ry / apply_rotation / apply_ry_chain /
    # apply_rotation_chain (src/cuda.rs:794-840): host state in, rotations
    # applied on the device in one fused sweep, host state out.
    def apply_rotation_chain(self, state, gates, dtype="c128") -> np.ndarray:
        sv = StateVector.from_amplitudes(state.amplitudes() if isinstance(state, StateVector) else state, dtype=dtype,
                                         backend=self)
        sv.apply_rotation_chain(gates)
        return sv.amplitudes()

    def apply_rotation(self, state, axis: int, qubit: int, theta: float, dtype="c128") -> np.ndarray:
        return self.apply_rotation_chain(state, [(axis, qubit, theta)], dtype=dtype)

    def apply_ry_chain(self, state, gates, dtype="c128") -> np.ndarray:
        return self.apply_rotation_chain(state, [(RotationAxis.Y, q, t) for q, t in gates], dtype=dtype)

    def apply_ry(self, state, qubit: int, theta: float, dtype="c128") -> np.ndarray:
        return self.apply_rotation(state, RotationAxis.Y, qubit, theta, dtype=dtype)

    def upload_batch(self, states, dtype="c128") -> "StateVectorBatch":
        return StateVectorBatch.from_states(states, dtype=dtype, backend=self)

    def run_circuit_batch(self, states, circuit: "Circuit", dtype="c128", exec_opts=None) -> list[np.ndarray]:
        """CudaBackend::run_circuit_batch (src/cuda.rs:958-967): one upload,
        one fused sweep over every state, one download."""
        arrs = [s.amplitudes() if isinstance(s, StateVector) else np.asarray(s, dtype=np.complex128) for s in states]
        if not arrs:
            raise QuantumError(_abi.STATUS_CODES["EmptyBatch"], "CUDA state batches must contain at least one state")
        if any(a.size != arrs[0].size for a in arrs):
            raise QuantumError(_abi.STATUS_CODES["IncompatibleBatch"], "all states in a CUDA batch must have the same width")
        n = arrs[0].size.bit_length() - 1
        src = np.ascontiguousarray(np.concatenate(arrs), dtype=np.complex128).view(np.float64)
        out = np.empty_like(src)
        ops = circuit.ops()
        check(load().qf_run_circuit_batch(self._h, n, _dtype_code(dtype), ptr(ops), len(ops), ptr(src), len(arrs), ptr(out),
                                          out.size, _exec(exec_opts)))
        return list(out.view(np.complex128).reshape(len(arrs), 1 << n).copy())

    def upload_density(self, entries, dtype="c128") -> "DensityMatrix":
        """CudaBackend::upload_density (src/cuda.rs:969-1021)."""
        return DensityMatrix.from_entries(entries, dtype=dtype, backend=self)

    def run_density_circuit(self, initial, circuit: "Circuit", dtype="c128", exec_opts=None) -> np.ndarray:
        """CudaBackend::run_density_circuit (src/cuda.rs:1022-1045): host
        entries in, host entries out."""
        e = initial.entries() if isinstance(initial, DensityMatrix) else np.asarray(initial, dtype=np.complex128)
        e = np.ascontiguousarray(e, dtype=np.complex128)
        d = int(e.shape[0])
        n = d.bit_length() - 1
        src = e.reshape(-1).view(np.float64)
        out = np.empty_like(src)
        ops = circuit.ops()
        check(load().qf_run_density_circuit(self._h, n, _dtype_code(dtype), ptr(ops), len(ops), ptr(src), ptr(out),
                                            out.size, _exec(exec_opts)))
        return out.view(np.complex128).reshape(d, d)

    def run_circuit_shots(self, initial_state, circuit: "Circuit", shots: int, seed: int, dtype="c128",
                          tie_eps: float = 0.0) -> "ShotResult":
        return circuit.run_shots(initial_state, shots, seed, dtype=dtype, backend=self, tie_eps=tie_eps)

    def run_circuit_shots_batched(self, initial_state, circuit: "Circuit", shots: int, seed: int, dtype="c128",
                                  tie_eps: float = 0.0) -> "ShotResult":
        """CudaBackend::run_circuit_shots_batched (src/cuda.rs:1157-1266): the
        noise-trajectory semantics when the circuit holds a channel (initial
        state normalised), plain run_shots otherwise."""
        noisy = any(op[0] == _abi.OP_CHANNEL for op in circuit.operations)
        return ShotResult.from_packed(*circuit.run_shots_packed(initial_state, shots, seed, dtype, self, tie_eps,
                                                                noise=noisy))


_default_backend: CudaBackend | None = None


def default_backend() -> CudaBackend:
    global _default_backend
    if _default_backend is None:
        _default_backend = CudaBackend(0)
    return _default_backend


def _exec(opts):
    if opts is None:
        return None
    return C.byref(_abi.exec_opts(opts))


# ---------------------------------------------------------------------------
# StateVector (device resident)
# ---------------------------------------------------------------------------
class StateVector:
    """A state vector resident in GPU memory (StateVector + CudaDeviceState)."""

    def __init__(self, handle, qubits: int, dtype: int, backend: CudaBackend):
        self._h = handle
        self.qubits = qubits
        self.dtype = dtype
        self.backend = backend

    @classmethod
    def zero(cls, qubits: int, dtype="c128", memory_budget: int | None = None, backend: CudaBackend | None = None):
        """StateVector::zero / zero_with_memory_budget (src/lib.rs:930-966)."""
        backend = backend or default_backend()
        h = C.c_void_p()
        check(load().qf_sv_create(backend.handle, int(qubits), _dtype_code(dtype), int(memory_budget or 0), C.byref(h)))
        return cls(h, int(qubits), _dtype_code(dtype), backend)

    zero_with_memory_budget = zero

    @classmethod
    def from_amplitudes(cls, amplitudes, dtype="c128", backend: CudaBackend | None = None):
        """StateVector::from_amplitudes (src/lib.rs:969-978)."""
        a = np.ascontiguousarray(np.asarray(amplitudes, dtype=np.complex128))
        if a.size < 2:
            raise QuantumError(_abi.STATUS_CODES["ZeroQubits"], "a state vector must contain at least one qubit")
        if a.size & (a.size - 1):
            raise QuantumError(_abi.STATUS_CODES["StateSizeNotPowerOfTwo"], f"state vector length {a.size} is not a power of two")
        sv = cls.zero(a.size.bit_length() - 1, dtype=dtype, backend=backend)
        check(load().qf_sv_upload(sv._h, ptr(a.view(np.float64)), 2 * a.size))
        return sv

    def __del__(self):
        try:
            if self._h and self._h.value:
                load().qf_sv_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    def num_qubits(self) -> int:
        return self.qubits

    def copy(self) -> "StateVector":
        other = StateVector.zero(self.qubits, dtype=self.dtype, backend=self.backend)
        check(load().qf_sv_copy_from(other._h, self._h))
        return other

    def amplitudes(self) -> np.ndarray:
        """Download as complex128 (CudaDeviceState::download, src/cuda.rs:1459-1471)."""
        out = np.empty(2 << self.qubits, dtype=np.float64)
        check(load().qf_sv_download(self._h, ptr(out), out.size))
        return out.view(np.complex128)

    # gates (src/lib.rs:1017-1122)
    def apply(self, gate: Gate, qubit: int) -> "StateVector":
        check(load().qf_sv_apply_gate(self._h, gate.code, gate.theta, int(qubit)))
        return self

    def apply_cnot(self, control: int, target: int) -> "StateVector":
        check(load().qf_sv_apply_cnot(self._h, int(control), int(target)))
        return self

    def apply_cz(self, first: int, second: int) -> "StateVector":
        check(load().qf_sv_apply_cz(self._h, int(first), int(second)))
        return self

    def apply_swap(self, first: int, second: int) -> "StateVector":
        check(load().qf_sv_apply_swap(self._h, int(first), int(second)))
        return self

    def apply_rotation_chain(self, gates) -> "StateVector":
        """CudaDeviceState::apply_rotation_chain (src/cuda.rs:1327-1352):
        (axis, qubit, theta) rotations, validated first, one fused sweep."""
        rot = {RotationAxis.X: _abi.GATE_RX, RotationAxis.Y: _abi.GATE_RY, RotationAxis.Z: _abi.GATE_RZ}
        recs = [(_abi.OP_GATE, rot[int(a)], int(q), 0, 0, float(t)) for a, q, t in gates]
        return self.apply_ops(_abi.ops_array(recs))

    def apply_rotation(self, axis: int, qubit: int, theta: float) -> "StateVector":
        return self.apply_rotation_chain([(axis, qubit, theta)])

    def apply_ops(self, ops: np.ndarray, params=None, inputs=None, exec_opts=None) -> "StateVector":
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
        i = None if inputs is None else np.ascontiguousarray(inputs, dtype=np.float64)
        check(load().qf_sv_apply_ops(self._h, ptr(ops), len(ops), ptr(p), 0 if p is None else p.size, ptr(i),
                                     0 if i is None else i.size, _exec(exec_opts)))
        return self

    # reductions (src/lib.rs:998-1166, 1278-1318)
    def norm_sqr(self) -> float:
        v = C.c_double()
        check(load().qf_sv_norm_sqr(self._h, C.byref(v)))
        return v.value

    def probabilities(self) -> np.ndarray:
        out = np.empty(1 << self.qubits, dtype=np.float64)
        check(load().qf_sv_probabilities(self._h, ptr(out), out.size))
        return out

    def expectation_z_all(self) -> np.ndarray:
        out = np.empty(self.qubits, dtype=np.float64)
        check(load().qf_sv_expectation_z_all(self._h, ptr(out), out.size))
        return out

    def expectation(self, observable: int, qubit: int) -> float:
        v = C.c_double()
        check(load().qf_sv_expectation(self._h, int(observable), int(qubit), C.byref(v)))
        return v.value

    def expectation_x(self, qubit: int) -> float:
        return self.expectation(SingleQubitObservable.X, qubit)

    def expectation_y(self, qubit: int) -> float:
        return self.expectation(SingleQubitObservable.Y, qubit)

    def expectation_z(self, qubit: int) -> float:
        return self.expectation(SingleQubitObservable.Z, qubit)

    def expectation_pauli_sum(self, hamiltonian) -> complex:
        t = _as_terms(hamiltonian)
        out = np.zeros(2, dtype=np.float64)
        check(load().qf_sv_expectation_pauli_sum(self._h, ptr(t), len(t), ptr(out)))
        return complex(out[0], out[1])

    def normalize(self) -> "StateVector":
        """StateVector::normalize (src/lib.rs:1005-1014)."""
        check(load().qf_sv_normalize(self._h))
        return self

    def apply_channel_trajectory(self, channel: "NoiseChannel", qubit: int, rng: SmallRng) -> int:
        """StateVector::apply_channel_trajectory (src/lib.rs:1356-1506): one
        draw from `rng`, the Kraus branch taken (returned) applied and renormalised."""
        rec = _abi.ops_array([channel.record(int(qubit))])
        st = C.c_uint64(rng.state)
        br = C.c_int()
        try:
            check(load().qf_sv_apply_channel_trajectory(self._h, ptr(rec), C.byref(st), C.byref(br)))
        finally:
            rng.state = st.value
        return br.value

    def measure(self, qubit: int, rng: SmallRng) -> int:
        """StateVector::measure (src/lib.rs:1321-1351), advancing `rng`."""
        st = C.c_uint64(rng.state)
        o = C.c_uint8()
        status = load().qf_sv_measure(self._h, int(qubit), C.byref(st), C.byref(o))
        rng.state = st.value
        check(status)
        return int(o.value)

    def sample(self, qubit_order, classical_bits, shots: int, seed: int, tie_eps: float = 0.0):
        """Terminal measurements of a resident state: (packed outcomes, ties)."""
        q = np.ascontiguousarray(qubit_order, dtype=np.uint32)
        cb = np.ascontiguousarray(classical_bits, dtype=np.uint32)
        out = np.empty(int(shots), dtype=np.uint64)
        ties = C.c_uint64()
        check(load().qf_sv_sample(self._h, ptr(q), ptr(cb), len(q), int(shots), int(seed), float(tie_eps), ptr(out),
                                  C.byref(ties)))
        return out, ties.value


# ---------------------------------------------------------------------------
# Circuits
# ---------------------------------------------------------------------------
class StateVectorBatch:
    """`CudaDeviceStateBatch` (src/cuda.rs:529-540, 1486-1992): equal-width
    states resident in one device allocation, swept together."""

    def __init__(self, handle, qubits: int, size: int, dtype: int, backend: CudaBackend):
        self._h, self.qubits, self.size, self.dtype, self.backend = handle, qubits, size, dtype, backend

    @classmethod
    def zero(cls, qubits: int, batch_size: int, dtype="c128", backend: CudaBackend | None = None) -> "StateVectorBatch":
        backend = backend or default_backend()
        h = C.c_void_p()
        code = _dtype_code(dtype)
        check(load().qf_batch_create(backend.handle, int(qubits), code, int(batch_size), C.byref(h)))
        return cls(h, int(qubits), int(batch_size), code, backend)

    @classmethod
    def from_states(cls, states, dtype="c128", backend: CudaBackend | None = None) -> "StateVectorBatch":
        """CudaBackend::upload_batch (src/cuda.rs:871-955)."""
        arrs = [s.amplitudes() if isinstance(s, StateVector) else np.asarray(s, dtype=np.complex128) for s in states]
        if not arrs:
            raise QuantumError(_abi.STATUS_CODES["EmptyBatch"], "CUDA state batches must contain at least one state")
        if any(a.size != arrs[0].size for a in arrs):
            raise QuantumError(_abi.STATUS_CODES["IncompatibleBatch"], "all states in a CUDA batch must have the same width")
        n = arrs[0].size.bit_length() - 1
        b = cls.zero(n, len(arrs), dtype=dtype, backend=backend)
        flat = np.ascontiguousarray(np.concatenate(arrs), dtype=np.complex128).view(np.float64)
        check(load().qf_batch_upload(b._h, ptr(flat), flat.size))
        return b

    def __del__(self):
        try:
            if self._h and self._h.value:
                load().qf_batch_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    def batch_size(self) -> int:
        return self.size

    def num_qubits(self) -> int:
        return self.qubits

    def apply_ops(self, ops: np.ndarray, exec_opts=None) -> "StateVectorBatch":
        check(load().qf_batch_apply_ops(self._h, ptr(ops), len(ops), _exec(exec_opts)))
        return self

    def apply_gate(self, gate: Gate, qubit: int) -> "StateVectorBatch":
        return self.apply_ops(_abi.ops_array([(_abi.OP_GATE, gate.code, int(qubit), 0, 0, gate.theta)]))

    def apply_cnot(self, control: int, target: int) -> "StateVectorBatch":
        return self.apply_ops(_abi.ops_array([(_abi.OP_CNOT, 0, int(control), int(target), 0, 0.0)]))

    def apply_cz(self, first: int, second: int) -> "StateVectorBatch":
        return self.apply_ops(_abi.ops_array([(_abi.OP_CZ, 0, int(first), int(second), 0, 0.0)]))

    def apply_swap(self, first: int, second: int) -> "StateVectorBatch":
        return self.apply_ops(_abi.ops_array([(_abi.OP_SWAP, 0, int(first), int(second), 0, 0.0)]))

    def run_circuit(self, circuit: "Circuit", exec_opts=None) -> "StateVectorBatch":
        return self.apply_ops(circuit.ops(), exec_opts)

    def measure(self, qubit: int, rng: SmallRng) -> list[int]:
        """One uniform per state in batch order; returns the outcomes."""
        st = C.c_uint64(rng.state)
        out = np.zeros(self.size, dtype=np.uint8)
        try:
            check(load().qf_batch_measure(self._h, int(qubit), C.byref(st), ptr(out)))
        finally:
            rng.state = st.value
        return out.tolist()

    def copy_from_device(self, source: "StateVectorBatch") -> None:
        check(load().qf_batch_copy_from(self._h, source._h))

    def synchronize(self) -> None:
        self.backend.synchronize()

    def download(self) -> list[np.ndarray]:
        out = np.empty(2 * (self.size << self.qubits), dtype=np.float64)
        check(load().qf_batch_download(self._h, ptr(out), out.size))
        return list(out.view(np.complex128).reshape(self.size, 1 << self.qubits).copy())


class DensityMatrix:
    """`DensityMatrix` (src/lib.rs:1551-2235) resident on the device, the
    reference's `CudaDeviceDensityMatrix` (src/cuda.rs:2007-2237): row-major
    entries rho[row, col]; gates act as U rho U^dagger, channels as their Kraus
    sums."""

    def __init__(self, handle, qubits: int, dtype: int, backend: CudaBackend):
        self._h, self.n, self.dtype, self.backend = handle, qubits, dtype, backend

    @classmethod
    def zero(cls, qubits: int, dtype="c128", backend: CudaBackend | None = None) -> "DensityMatrix":
        backend = backend or default_backend()
        h = C.c_void_p()
        code = _dtype_code(dtype)
        check(load().qf_dm_create(backend.handle, int(qubits), code, C.byref(h)))
        return cls(h, int(qubits), code, backend)

    @classmethod
    def from_state(cls, state: "StateVector") -> "DensityMatrix":
        rho = cls.zero(state.qubits, dtype=state.dtype, backend=state.backend)
        check(load().qf_dm_from_state(rho._h, state._h))
        return rho

    @classmethod
    def maximally_mixed(cls, qubits: int, dtype="c128", backend: CudaBackend | None = None) -> "DensityMatrix":
        rho = cls.zero(qubits, dtype=dtype, backend=backend)
        check(load().qf_dm_set_maximally_mixed(rho._h))
        return rho

    @classmethod
    def from_entries(cls, entries, dtype="c128", backend: CudaBackend | None = None) -> "DensityMatrix":
        e = np.ascontiguousarray(entries, dtype=np.complex128)
        n = int(e.shape[0]).bit_length() - 1
        rho = cls.zero(n, dtype=dtype, backend=backend)
        flat = e.reshape(-1).view(np.float64)
        check(load().qf_dm_upload(rho._h, ptr(flat), flat.size))
        return rho

    def __del__(self):
        try:
            if self._h and self._h.value:
                load().qf_dm_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    def qubits(self) -> int:
        return self.n

    def dimension(self) -> int:
        return 1 << self.n

    def entries(self) -> np.ndarray:
        d = 1 << self.n
        out = np.empty(2 * d * d, dtype=np.float64)
        check(load().qf_dm_download(self._h, ptr(out), out.size))
        return out.view(np.complex128).reshape(d, d)

    def apply_ops(self, ops: np.ndarray, exec_opts=None) -> "DensityMatrix":
        check(load().qf_dm_apply_ops(self._h, ptr(ops), len(ops), _exec(exec_opts)))
        return self

    def apply(self, gate: Gate, qubit: int) -> "DensityMatrix":
        return self.apply_ops(_abi.ops_array([(_abi.OP_GATE, gate.code, int(qubit), 0, 0, gate.theta)]))

    def apply_cnot(self, control: int, target: int) -> "DensityMatrix":
        return self.apply_ops(_abi.ops_array([(_abi.OP_CNOT, 0, int(control), int(target), 0, 0.0)]))

    def apply_cz(self, first: int, second: int) -> "DensityMatrix":
        return self.apply_ops(_abi.ops_array([(_abi.OP_CZ, 0, int(first), int(second), 0, 0.0)]))

    def apply_swap(self, first: int, second: int) -> "DensityMatrix":
        return self.apply_ops(_abi.ops_array([(_abi.OP_SWAP, 0, int(first), int(second), 0, 0.0)]))

    def apply_channel(self, channel: "NoiseChannel", qubit: int) -> "DensityMatrix":
        return self.apply_ops(_abi.ops_array([channel.record(int(qubit))]))

    def depolarize(self, qubit: int, probability: float) -> "DensityMatrix":
        return self.apply_channel(NoiseChannel.Depolarizing(probability), qubit)

    def trace(self) -> complex:
        out = np.zeros(2)
        check(load().qf_dm_trace(self._h, ptr(out)))
        return complex(out[0], out[1])

    def purity(self) -> float:
        v = C.c_double()
        check(load().qf_dm_purity(self._h, C.byref(v)))
        return v.value

    def expectation(self, observable: int, qubit: int) -> float:
        v = C.c_double()
        check(load().qf_dm_expectation(self._h, int(observable), int(qubit), C.byref(v)))
        return v.value

    def expectation_z(self, qubit: int) -> float:
        return self.expectation(_abi.PAULI_Z, qubit)

    def probability_one(self, qubit: int) -> float:
        v = C.c_double()
        check(load().qf_dm_probability_one(self._h, int(qubit), C.byref(v)))
        return v.value

    def probabilities(self) -> np.ndarray:
        out = np.empty(1 << self.n, dtype=np.float64)
        check(load().qf_dm_probabilities(self._h, ptr(out), out.size))
        return out

    def measure(self, qubit: int, rng: SmallRng) -> int:
        st = C.c_uint64(rng.state)
        o = C.c_uint8()
        try:
            check(load().qf_dm_measure(self._h, int(qubit), C.byref(st), C.byref(o)))
        finally:
            rng.state = st.value
        return o.value


@dataclass
class ShotResult:
    """`ShotResult` (src/lib.rs:2453-2464): counts keyed by LSB-first bit tuples."""

    shots: int
    counts: dict
    ties: int = 0

    @staticmethod
    def from_packed(packed: np.ndarray, width: int, ties: int = 0) -> "ShotResult":
        """Counts keyed by LSB-first bit tuples, in the BTreeMap<Vec<u8>, usize>
        order of the reference (lexicographic from classical bit 0)."""
        vals, cnts = np.unique(np.asarray(packed, dtype=np.uint64), return_counts=True)
        bits = ((vals[:, None] >> np.arange(width, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(np.uint8)
        order = np.lexsort(bits.T[::-1]) if width else np.arange(vals.size)
        counts = dict(zip(map(tuple, bits[order].tolist()), cnts[order].tolist()))
        return ShotResult(int(np.asarray(packed).size), counts, ties)


class NoiseChannel:
    """`enum NoiseChannel` (src/lib.rs:1561-1627): a local channel on one qubit.
    Shots sample one Kraus trajectory per channel (run_shots_with_noise)."""

    __slots__ = ("kind", "p", "beta_delta")

    def __init__(self, kind: int, p: float, beta_delta: float = 0.0):
        self.kind, self.p, self.beta_delta = int(kind), float(p), float(beta_delta)

    @staticmethod
    def Depolarizing(probability: float) -> "NoiseChannel":
        return NoiseChannel(_abi.CHANNEL_DEPOLARIZING, probability)

    @staticmethod
    def AmplitudeDamping(gamma: float) -> "NoiseChannel":
        return NoiseChannel(_abi.CHANNEL_AMPLITUDE_DAMPING, gamma)

    @staticmethod
    def PhaseDamping(gamma: float) -> "NoiseChannel":
        return NoiseChannel(_abi.CHANNEL_PHASE_DAMPING, gamma)

    @staticmethod
    def ThermalDamping(gamma_down: float, beta_delta: float) -> "NoiseChannel":
        return NoiseChannel(_abi.CHANNEL_THERMAL_DAMPING, gamma_down, beta_delta)

    def thermal_rates(self):
        """(gamma_up, gamma_down) of a thermal channel, else None (src/lib.rs:1611-1626)."""
        if self.kind != _abi.CHANNEL_THERMAL_DAMPING:
            return None
        if not (math.isfinite(self.p) and 0.0 <= self.p <= 1.0) or not (math.isfinite(self.beta_delta) and self.beta_delta >= 0):
            raise ValueError("invalid thermal damping parameters")
        return self.p * math.exp(-self.beta_delta), self.p

    def record(self, target: int) -> tuple:
        return _abi.channel_record(self.kind, target, self.p, self.beta_delta)

    def __eq__(self, other) -> bool:
        return isinstance(other, NoiseChannel) and (self.kind, self.p, self.beta_delta) == (other.kind, other.p, other.beta_delta)

    def __repr__(self) -> str:
        names = ["Depolarizing", "AmplitudeDamping", "PhaseDamping", "ThermalDamping"]
        extra = f", beta_delta={self.beta_delta}" if self.kind == _abi.CHANNEL_THERMAL_DAMPING else ""
        return f"NoiseChannel.{names[self.kind]}({self.p}{extra})"


def _cached_ops(owner) -> np.ndarray:
    """The ``qf_op`` array of ``owner.operations``, rebuilt only when the list
    differs from the one it was built from (records are tuples; the array is
    read-only and shared between calls)."""
    src = getattr(owner, "_ops_src", None)
    if src is not None and src == owner.operations:
        return owner._ops_arr
    arr = _abi.ops_array(owner.operations)
    arr.flags.writeable = False
    owner._ops_src = list(owner.operations)
    owner._ops_arr = arr
    return arr


class Circuit:
    """`Circuit` (src/lib.rs:2517-2916): an op list executed on a device state."""

    def __init__(self):
        self.operations: list[tuple] = []

    @classmethod
    def from_ops(cls, ops: np.ndarray) -> "Circuit":
        """A circuit from a ``qf_op`` record array."""
        c = cls()
        for r in ops:
            c.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), int(r["param"]),
                                 float(r["theta"]), int(r["flags"])))
        return c

    def push(self, gate: Gate, target: int) -> None:
        self.operations.append((_abi.OP_GATE, gate.code, int(target), 0, 0, gate.theta))

    def cnot(self, control: int, target: int) -> None:
        self.operations.append((_abi.OP_CNOT, 0, int(control), int(target), 0, 0.0))

    def cz(self, first: int, second: int) -> None:
        self.operations.append((_abi.OP_CZ, 0, int(first), int(second), 0, 0.0))

    def swap(self, first: int, second: int) -> None:
        self.operations.append((_abi.OP_SWAP, 0, int(first), int(second), 0, 0.0))

    def channel(self, target: int, channel: NoiseChannel) -> None:
        self.operations.append(channel.record(int(target)))

    def measure(self, target: int, classical_bit: int) -> None:
        self.operations.append((_abi.OP_MEASURE, 0, int(target), 0, int(classical_bit), 0.0))

    def if_classical_bit(self, classical_bit: int, value: int, gate: Gate, target: int) -> None:
        self.operations.append((_abi.OP_COND, gate.code, int(target), 0, int(classical_bit), gate.theta, int(value) & 1))

    # ---- formats (src/serialize.rs, src/qasm.rs, src/qasm_export.rs) ----
    @classmethod
    def from_qasm(cls, source: str) -> "Circuit":
        """qasm::parse_qasm (src/qasm.rs:73): OpenQASM 2.0 text to a circuit."""
        return cls.from_ops(parse_qasm_ops(source)[0])

    @classmethod
    def from_json(cls, text: str) -> "Circuit":
        """Circuit::from_json (src/serialize.rs:150-154)."""
        return cls.from_json_bytes(text.encode())

    @classmethod
    def from_json_bytes(cls, data: bytes) -> "Circuit":
        lib = load()
        n = C.c_uint64()
        check(lib.qf_circuit_from_json(data, len(data), None, 0, C.byref(n), None, None))
        ops = np.zeros(n.value, dtype=_abi.OP_DTYPE)
        check(lib.qf_circuit_from_json(data, len(data), ptr(ops), n.value, C.byref(n), None, None))
        return cls.from_ops(ops)

    def to_json(self) -> str:
        """Circuit::to_json (src/serialize.rs:91-95): serde_json's pretty form."""
        return self._text(lambda lib, ops, out, cap, ln: lib.qf_circuit_to_json(ptr(ops), len(ops), out, cap, ln))

    def to_json_bytes(self) -> bytes:
        """Circuit::to_json_bytes (src/serialize.rs:97-101): the same document."""
        return self.to_json().encode()

    def to_qasm(self, num_qubits: int | None = None) -> str:
        """qasm_export::export_qasm, or export_qasm_with_qubits when
        `num_qubits` is given."""
        nq = -1 if num_qubits is None else int(num_qubits)
        return self._text(lambda lib, ops, out, cap, ln: lib.qf_circuit_to_qasm(ptr(ops), len(ops), nq, out, cap, ln))

    def _text(self, call) -> str:
        lib = load()
        ops = self.ops()
        n = C.c_uint64()
        check(call(lib, ops, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        check(call(lib, ops, C.cast(buf, C.c_void_p), n.value + 1, C.byref(n)))
        return buf.value.decode()

    def has_measurements(self) -> bool:
        return any(op[0] == _abi.OP_MEASURE for op in self.operations)

    def num_qubits(self) -> int:
        m = -1
        for op in self.operations:
            m = max(m, op[2])
            if op[0] in (_abi.OP_CNOT, _abi.OP_CZ, _abi.OP_SWAP):
                m = max(m, op[3])
        return m + 1

    def ops(self) -> np.ndarray:
        return _cached_ops(self)

    def run(self, state: StateVector, exec_opts=None) -> StateVector:
        """Circuit::run (src/lib.rs:2786-2802), in place on the device state."""
        return state.apply_ops(self.ops(), exec_opts=exec_opts)

    def run_shots(self, initial_state, shots: int, seed: int, dtype="c128", backend: CudaBackend | None = None,
                  tie_eps: float = 0.0, exec_opts=None) -> ShotResult:
        """Circuit::run_shots (src/lib.rs:2822-2916) for terminal measurements."""
        return ShotResult.from_packed(*self.run_shots_packed(initial_state, shots, seed, dtype, backend, tie_eps, exec_opts))

    def run_density(self, state: "DensityMatrix", exec_opts=None) -> "DensityMatrix":
        """Circuit::run_density (src/lib.rs:2804-2818), in place on the device matrix."""
        return state.apply_ops(self.ops(), exec_opts)

    def run_shots_with_noise(self, initial_state, shots: int, seed: int, dtype="c128", backend: CudaBackend | None = None,
                             tie_eps: float = 0.0, exec_opts=None) -> ShotResult:
        """Circuit::run_shots_with_noise (src/lib.rs:2829-2840): channel
        trajectories, measurements and feed-forward per shot."""
        return ShotResult.from_packed(*self.run_shots_packed(initial_state, shots, seed, dtype, backend, tie_eps, exec_opts,
                                                             noise=True))

    def run_shots_packed(self, initial_state, shots: int, seed: int, dtype="c128", backend: CudaBackend | None = None,
                         tie_eps: float = 0.0, exec_opts=None, noise: bool = False):
        """The engine's qf_run_shots (qf_run_shots_with_noise when `noise`)
        result: (packed outcomes, one u64 per shot with classical bit c at
        bit c; register width; ties)."""
        backend = backend or default_backend()
        if isinstance(initial_state, StateVector):
            amps = initial_state.amplitudes()
        elif isinstance(initial_state, int):
            amps = np.zeros(1 << initial_state, dtype=np.complex128)
            amps[0] = 1
        else:
            amps = np.asarray(initial_state, dtype=np.complex128)
        n = amps.size.bit_length() - 1
        ops = self.ops()
        src = np.ascontiguousarray(amps).view(np.float64)
        out = np.empty(max(int(shots), 1), dtype=np.uint64)
        width = C.c_uint32()
        ties = C.c_uint64()
        fn = load().qf_run_shots_with_noise if noise else load().qf_run_shots
        check(fn(backend.handle, n, _dtype_code(dtype), ptr(ops), len(ops), ptr(src), int(shots), int(seed), float(tie_eps),
                 ptr(out), C.byref(width), C.byref(ties), _exec(exec_opts)))
        return out[: int(shots)], width.value, ties.value


@dataclass
class ShotConfig:
    """`ShotConfig` (src/lib.rs:3019-3026): shots per estimate and the seed."""

    shots: int
    seed: int = 0


def wilson_ci(successes: int, shots: int, confidence: float = 0.95):
    """Wilson score interval of a binomial proportion (src/lib.rs:2493-2513)."""
    if shots == 0:
        return 0.0, 1.0
    n = float(shots)
    p = successes / n
    z = 2.576 if confidence >= 0.99 else 1.96 if confidence >= 0.95 else 1.645 if confidence >= 0.90 else 1.96
    z2 = z * z
    denom = 1.0 + z2 / n
    center = (p + z2 / (2.0 * n)) / denom
    half = (z / denom) * math.sqrt(p * (1.0 - p) / n + z2 / (4.0 * n * n))
    return max(center - half, 0.0), min(center + half, 1.0)


def sample_expectation(expectation: float, sampling: "ShotConfig") -> float:
    """sample_expectation (src/lib.rs:4840-4850), computed by the library."""
    v = C.c_double()
    check(load().qf_sample_expectation(float(expectation), int(sampling.shots), int(sampling.seed), C.byref(v), None))
    return v.value


def parse_qasm_ops(source: str):
    """qf_parse_qasm: (op records, qubits declared, classical bits declared)."""
    data = source.encode()
    lib = load()
    n, nq, nc, line = C.c_uint64(), C.c_uint32(), C.c_uint32(), C.c_uint64()
    check(lib.qf_parse_qasm(data, len(data), None, 0, C.byref(n), C.byref(nq), C.byref(nc), C.byref(line)))
    ops = np.zeros(n.value, dtype=_abi.OP_DTYPE)
    check(lib.qf_parse_qasm(data, len(data), ptr(ops), n.value, C.byref(n), C.byref(nq), C.byref(nc), C.byref(line)))
    return ops, nq.value, nc.value


def parse_qasm(source: str) -> "Circuit":
    """qasm::parse_qasm (src/qasm.rs:73)."""
    return Circuit.from_qasm(source)


def export_qasm(circuit: "Circuit") -> str:
    """qasm_export::export_qasm."""
    return circuit.to_qasm()


def export_qasm_with_qubits(circuit: "Circuit", num_qubits: int) -> str:
    """qasm_export::export_qasm_with_qubits."""
    return circuit.to_qasm(num_qubits)


class ParameterizedCircuit:
    """`ParameterizedCircuit` (src/lib.rs:3008-3121, 3480-3704, 4651-4740)."""

    def __init__(self, parameter_count: int, input_count: int = 0):
        self.parameter_count_ = int(parameter_count)
        self.input_count_ = int(input_count)
        self.operations: list[tuple] = []

    @classmethod
    def new(cls, parameter_count: int) -> "ParameterizedCircuit":
        return cls(parameter_count)

    @classmethod
    def with_inputs(cls, parameter_count: int, input_count: int) -> "ParameterizedCircuit":
        return cls(parameter_count, input_count)

    @classmethod
    def from_ops(cls, ops: np.ndarray, parameter_count: int, input_count: int = 0) -> "ParameterizedCircuit":
        """A parameterized circuit from a ``qf_op`` record array."""
        c = cls(parameter_count, input_count)
        for r in ops:
            c.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), int(r["param"]),
                                 float(r["theta"])))
        return c

    def parameter_count(self) -> int:
        return self.parameter_count_

    def input_count(self) -> int:
        return self.input_count_

    def push(self, gate: Gate, target: int) -> None:
        self.operations.append((_abi.OP_GATE, gate.code, int(target), 0, 0, gate.theta))

    def rotation(self, axis: int, target: int, parameter: int) -> None:
        self.operations.append((_abi.OP_ROTATION, int(axis), int(target), 0, int(parameter), 0.0))

    def encode_rotation(self, axis: int, target: int, input: int) -> None:  # noqa: A002 - reference name
        self.operations.append((_abi.OP_ENCODING, int(axis), int(target), 0, int(input), 0.0))

    def cnot(self, control: int, target: int) -> None:
        self.operations.append((_abi.OP_CNOT, 0, int(control), int(target), 0, 0.0))

    def cz(self, first: int, second: int) -> None:
        self.operations.append((_abi.OP_CZ, 0, int(first), int(second), 0, 0.0))

    def swap(self, first: int, second: int) -> None:
        self.operations.append((_abi.OP_SWAP, 0, int(first), int(second), 0, 0.0))

    def channel(self, target: int, channel: NoiseChannel) -> None:
        self.operations.append(channel.record(int(target)))

    def ops(self) -> np.ndarray:
        return _cached_ops(self)

    # validate_parameters / validate_inputs (src/lib.rs:4651-4675)
    def _values(self, inputs, parameters):
        p = np.ascontiguousarray(parameters, dtype=np.float64).reshape(-1)
        i = np.ascontiguousarray(inputs if inputs is not None else [], dtype=np.float64).reshape(-1)
        if i.size != self.input_count_:
            raise QuantumError(_abi.STATUS_CODES["InvalidInputCount"],
                               f"expected {self.input_count_} encoded inputs, got {i.size}")
        if not np.all(np.isfinite(i)):
            raise QuantumError(_abi.STATUS_CODES["NonFiniteParameter"], "circuit parameters must be finite")
        if p.size != self.parameter_count_:
            raise QuantumError(_abi.STATUS_CODES["InvalidParameterCount"],
                               f"expected {self.parameter_count_} circuit parameters, got {p.size}")
        if not np.all(np.isfinite(p)):
            raise QuantumError(_abi.STATUS_CODES["NonFiniteParameter"], "circuit parameters must be finite")
        return i, p

    def run_with_inputs(self, inputs, parameters, qubits: int, dtype="c128", backend=None, exec_opts=None) -> StateVector:
        i, p = self._values(inputs, parameters)
        sv = StateVector.zero(qubits, dtype=dtype, backend=backend)
        return sv.apply_ops(self.ops(), params=p, inputs=i, exec_opts=exec_opts)

    def run(self, parameters, qubits: int, dtype="c128", backend=None, exec_opts=None) -> StateVector:
        return self.run_with_inputs([], parameters, qubits, dtype=dtype, backend=backend, exec_opts=exec_opts)

    # ---- finite-shot estimates (src/lib.rs:3323-3479, 4806-4838) ----
    def _shots_call(self, inputs, parameters, qubits, observable, observable_qubit, sampling, dtype, backend, exec_opts,
                    tie_eps):
        i, p = self._values(inputs, parameters)
        be = backend or default_backend()
        return i, p, be, self.ops(), _dtype_code(dtype), int(sampling.shots), int(sampling.seed)

    def expectation_with_inputs_shots_with_ci(self, inputs, parameters, qubits: int, observable: int,
                                              observable_qubit: int, sampling: "ShotConfig", dtype="c128",
                                              backend=None, exec_opts=None, tie_eps: float = 0.0):
        """(estimate, Wilson 95 % interval on the expectation) from `sampling`
        shots (src/lib.rs:3384-3405)."""
        i, p, be, ops, dc, shots, seed = self._shots_call(inputs, parameters, qubits, observable, observable_qubit, sampling,
                                                          dtype, backend, exec_opts, tie_eps)
        est, ok, ties = C.c_double(), C.c_uint64(), C.c_uint64()
        check(load().qf_expectation_shots(be.handle, int(qubits), dc, ptr(ops), len(ops), ptr(p), p.size, ptr(i), i.size,
                                          int(observable), int(observable_qubit), shots, seed, float(tie_eps),
                                          _exec(exec_opts), C.byref(est), C.byref(ok), C.byref(ties)))
        lo, hi = wilson_ci(ok.value, shots, 0.95)
        return est.value, (2.0 * lo - 1.0, 2.0 * hi - 1.0)

    def expectation_with_inputs_shots(self, inputs, parameters, qubits: int, observable: int, observable_qubit: int,
                                      sampling: "ShotConfig", **kw) -> float:
        """expectation_with_inputs_shots (src/lib.rs:3361-3382)."""
        return self.expectation_with_inputs_shots_with_ci(inputs, parameters, qubits, observable, observable_qubit,
                                                          sampling, **kw)[0]

    def expectation_shots(self, parameters, qubits: int, observable: int, observable_qubit: int, sampling, **kw) -> float:
        return self.expectation_with_inputs_shots([], parameters, qubits, observable, observable_qubit, sampling, **kw)

    def expectation_shots_with_ci(self, parameters, qubits: int, observable: int, observable_qubit: int, sampling, **kw):
        return self.expectation_with_inputs_shots_with_ci([], parameters, qubits, observable, observable_qubit, sampling,
                                                          **kw)

    def parameter_shift_gradient_with_inputs_shots(self, inputs, parameters, qubits: int, observable: int,
                                                   observable_qubit: int, sampling: "ShotConfig", dtype="c128",
                                                   backend=None, exec_opts=None, tie_eps: float = 0.0) -> np.ndarray:
        """parameter_shift_gradient_with_inputs_shots (src/lib.rs:3428-3479)."""
        i, p, be, ops, dc, shots, seed = self._shots_call(inputs, parameters, qubits, observable, observable_qubit, sampling,
                                                          dtype, backend, exec_opts, tie_eps)
        g = np.zeros(p.size, dtype=np.float64)
        ties = C.c_uint64()
        check(load().qf_parameter_shift_gradient_shots(be.handle, int(qubits), dc, ptr(ops), len(ops), ptr(p), p.size, ptr(i),
                                                       i.size, int(observable), int(observable_qubit), shots, seed,
                                                       float(tie_eps), _exec(exec_opts), ptr(g), C.byref(ties)))
        return g

    def parameter_shift_gradient_shots(self, parameters, qubits: int, observable: int, observable_qubit: int, sampling,
                                       **kw) -> np.ndarray:
        return self.parameter_shift_gradient_with_inputs_shots([], parameters, qubits, observable, observable_qubit,
                                                               sampling, **kw)

    # ---- the density-matrix path (channels; src/lib.rs:3125-3266, 3755-3800) ----
    def _resolved_ops(self, inputs, parameters) -> np.ndarray:
        """The op list with rotation and encoding angles bound to fixed gates."""
        i, p = self._values(inputs, parameters)
        ops = self.ops().copy()
        rot = {_abi.PAULI_X: _abi.GATE_RX, _abi.PAULI_Y: _abi.GATE_RY, _abi.PAULI_Z: _abi.GATE_RZ}
        for k in range(len(ops)):
            kind = int(ops[k]["kind"])
            if kind in (_abi.OP_ROTATION, _abi.OP_ENCODING):
                src = p if kind == _abi.OP_ROTATION else i
                idx = int(ops[k]["param"])
                if idx >= src.size:
                    name = "InvalidParameterCount" if kind == _abi.OP_ROTATION else "InvalidInputCount"
                    raise QuantumError(_abi.STATUS_CODES[name], f"index {idx} exceeds the {src.size} values given")
                ops[k]["theta"] = float(src[idx])
                ops[k]["gate"] = rot[int(ops[k]["gate"])]
                ops[k]["kind"] = _abi.OP_GATE
                ops[k]["param"] = 0
        return ops

    def run_density_with_inputs(self, inputs, parameters, qubits: int, dtype="c128", backend=None,
                                exec_opts=None) -> "DensityMatrix":
        """ParameterizedCircuit::run_density_with_inputs (src/lib.rs:3125-3132)."""
        rho = DensityMatrix.zero(qubits, dtype=dtype, backend=backend)
        return rho.apply_ops(self._resolved_ops(inputs, parameters), exec_opts)

    def run_density(self, parameters, qubits: int, **kw) -> "DensityMatrix":
        return self.run_density_with_inputs([], parameters, qubits, **kw)

    def expectation_density_with_inputs(self, inputs, parameters, qubits: int, observable: int, observable_qubit: int,
                                        dtype="c128", backend=None, exec_opts=None) -> float:
        """expectation_density_with_inputs (src/lib.rs:3175-3186)."""
        i, p = self._values(inputs, parameters)
        be = backend or default_backend()
        ops = self.ops()
        v = C.c_double()
        check(load().qf_expectation_density(be.handle, int(qubits), _dtype_code(dtype), ptr(ops), len(ops), ptr(p), p.size,
                                            ptr(i), i.size, int(observable), int(observable_qubit), _exec(exec_opts),
                                            C.byref(v)))
        return v.value

    def parameter_shift_gradient_density_with_inputs(self, inputs, parameters, qubits: int, observable: int,
                                                     observable_qubit: int, dtype="c128", backend=None,
                                                     exec_opts=None) -> np.ndarray:
        """parameter_shift_gradient_density_with_inputs (src/lib.rs:3235-3266)."""
        i, p = self._values(inputs, parameters)
        be = backend or default_backend()
        ops = self.ops()
        g = np.zeros(p.size, dtype=np.float64)
        check(load().qf_parameter_shift_gradient_density(be.handle, int(qubits), _dtype_code(dtype), ptr(ops), len(ops),
                                                         ptr(p), p.size, ptr(i), i.size, int(observable),
                                                         int(observable_qubit), _exec(exec_opts), None, ptr(g)))
        return g

    def mse_loss_and_gradient_density(self, data, parameters, qubits: int, observable: int, observable_qubit: int,
                                      **kw):
        """mse_loss_and_gradient_density (src/lib.rs:3755-3800): mean squared
        error of the density-matrix expectations and its parameter-shift gradient."""
        self._check_training_data(data)
        p = np.ascontiguousarray(parameters, dtype=np.float64)
        loss, grad = 0.0, np.zeros(self.parameter_count_)
        for x, y in data:
            r = self.expectation_density_with_inputs(x, p, qubits, observable, observable_qubit, **kw) - y
            loss += r * r
            grad += 2.0 * r * self.parameter_shift_gradient_density_with_inputs(x, p, qubits, observable, observable_qubit, **kw)
        return loss / len(data), grad / len(data)

    def _check_training_data(self, data):
        if not data or any(len(x) != self.input_count_ or not math.isfinite(y) or not all(math.isfinite(v) for v in x)
                           for x, y in data):
            raise QuantumError(_abi.STATUS_CODES["InvalidArgument"], "invalid training data")

    def expectation_density_with_inputs_shots_with_ci(self, inputs, parameters, qubits: int, observable: int,
                                                      observable_qubit: int, sampling: "ShotConfig", **kw):
        """(estimate, Wilson 95 % interval) of the density-matrix expectation
        from `sampling` shots (src/lib.rs:3208-3232): the exact expectation
        through sample_expectation, the interval from round(P(+1) * shots)."""
        if int(sampling.shots) == 0:
            raise QuantumError(_abi.STATUS_CODES["InvalidShotCount"], "shot count must be greater than zero")
        exact = self.expectation_density_with_inputs(inputs, parameters, qubits, observable, observable_qubit, **kw)
        est = sample_expectation(exact, sampling)
        p = min(max((1.0 + exact) * 0.5, 0.0), 1.0)
        lo, hi = wilson_ci(int(np.round(p * int(sampling.shots))), int(sampling.shots), 0.95)
        return est, (2.0 * lo - 1.0, 2.0 * hi - 1.0)

    def expectation_density_with_inputs_shots(self, inputs, parameters, qubits: int, observable: int,
                                              observable_qubit: int, sampling: "ShotConfig", **kw) -> float:
        """expectation_density_with_inputs_shots (src/lib.rs:3188-3206)."""
        if int(sampling.shots) == 0:
            raise QuantumError(_abi.STATUS_CODES["InvalidShotCount"], "shot count must be greater than zero")
        exact = self.expectation_density_with_inputs(inputs, parameters, qubits, observable, observable_qubit, **kw)
        return sample_expectation(exact, sampling)

    def parameter_shift_gradient_density_with_inputs_shots(self, inputs, parameters, qubits: int, observable: int,
                                                           observable_qubit: int, sampling: "ShotConfig", dtype="c128",
                                                           backend=None, exec_opts=None) -> np.ndarray:
        """parameter_shift_gradient_density_with_inputs_shots (src/lib.rs:3268-3320)."""
        i, p = self._values(inputs, parameters)
        be = backend or default_backend()
        ops = self.ops()
        g = np.zeros(p.size, dtype=np.float64)
        check(load().qf_parameter_shift_gradient_density_shots(be.handle, int(qubits), _dtype_code(dtype), ptr(ops),
                                                               len(ops), ptr(p), p.size, ptr(i), i.size, int(observable),
                                                               int(observable_qubit), int(sampling.shots),
                                                               int(sampling.seed), _exec(exec_opts), ptr(g)))
        return g

    def _mse_shots(self, data, parameters, sampling, predict, gradient):
        if int(sampling.shots) == 0:
            raise QuantumError(_abi.STATUS_CODES["InvalidShotCount"], "shot count must be greater than zero")
        self._check_training_data(data)
        p = np.ascontiguousarray(parameters, dtype=np.float64)
        loss, grad = 0.0, np.zeros(self.parameter_count_)
        for k, (x, y) in enumerate(data):
            seed = (int(sampling.seed) + k * 0x9E3779B9) & 0xFFFFFFFFFFFFFFFF
            r = predict(x, p, ShotConfig(int(sampling.shots), seed)) - y
            loss += r * r
            grad += 2.0 * r * gradient(x, p, ShotConfig(int(sampling.shots), (seed + 1) & 0xFFFFFFFFFFFFFFFF))
        return loss / len(data), grad / len(data)

    def mse_loss_and_gradient_shots(self, data, parameters, qubits: int, observable: int, observable_qubit: int,
                                    sampling: "ShotConfig", **kw):
        """mse_loss_and_gradient_shots (src/lib.rs:3866-3927): sample k uses
        seed + k * 0x9e3779b9 for its prediction and that + 1 for its gradient."""
        return self._mse_shots(
            data, parameters, sampling,
            lambda x, p, sc: self.expectation_with_inputs_shots(x, p, qubits, observable, observable_qubit, sc, **kw),
            lambda x, p, sc: self.parameter_shift_gradient_with_inputs_shots(x, p, qubits, observable, observable_qubit,
                                                                             sc, **kw))

    def mse_loss_and_gradient_density_shots(self, data, parameters, qubits: int, observable: int, observable_qubit: int,
                                            sampling: "ShotConfig", **kw):
        """mse_loss_and_gradient_density_shots (src/lib.rs:3802-3864)."""
        return self._mse_shots(
            data, parameters, sampling,
            lambda x, p, sc: self.expectation_density_with_inputs_shots(x, p, qubits, observable, observable_qubit, sc,
                                                                        **kw),
            lambda x, p, sc: self.parameter_shift_gradient_density_with_inputs_shots(x, p, qubits, observable,
                                                                                     observable_qubit, sc, **kw))

    def expectation_pauli_sum(self, parameters, qubits: int, hamiltonian, inputs=None, dtype="c128", backend=None,
                              exec_opts=None) -> float:
        i, p = self._values(inputs, parameters)
        backend = backend or default_backend()
        t = _as_terms(hamiltonian)
        ops = self.ops()
        v = C.c_double()
        check(load().qf_expectation(backend.handle, int(qubits), _dtype_code(dtype), ptr(ops), len(ops), ptr(p), p.size,
                                    ptr(i), i.size, ptr(t), len(t), _exec(exec_opts), C.byref(v)))
        return v.value

    # gradients: thin wrappers over gradients.gradient_with_inputs
    def circuit_profile(self):
        from .gradients import CircuitProfile

        prof = CircuitProfile(operations=len(self.operations), parameters=self.parameter_count_)
        for op in self.operations:
            if op[0] == _abi.OP_ROTATION:
                prof.parameterized_operations += 1
            elif op[0] == _abi.OP_CHANNEL:
                prof.has_channel = True
        return prof

    def gradient_with_inputs(self, options, inputs, parameters, qubits, observable, observable_qubit, **kw):
        from .gradients import gradient_with_inputs

        return gradient_with_inputs(self, options, inputs, parameters, qubits,
                                    PauliSum.single(observable, observable_qubit), **kw)

    def gradient(self, options, parameters, qubits, observable, observable_qubit, **kw):
        return self.gradient_with_inputs(options, [], parameters, qubits, observable, observable_qubit, **kw)

    def gradient_auto(self, parameters, qubits, observable, observable_qubit, **kw):
        from .gradients import GradientOptions

        return self.gradient(GradientOptions(), parameters, qubits, observable, observable_qubit, **kw)

    def _strategy_grad(self, strategy, inputs, parameters, qubits, observable, q, **kw):
        from .gradients import GradientOptions

        return self.gradient_with_inputs(GradientOptions(strategy=strategy), inputs, parameters, qubits, observable, q,
                                         **kw).gradient

    def parameter_shift_gradient_with_inputs(self, inputs, parameters, qubits, observable, observable_qubit, **kw):
        from .gradients import GradientStrategy

        return self._strategy_grad(GradientStrategy.ParameterShift, inputs, parameters, qubits, observable,
                                   observable_qubit, **kw)

    def parameter_shift_gradient_for(self, parameters, qubits, observable, observable_qubit, **kw):
        return self.parameter_shift_gradient_with_inputs([], parameters, qubits, observable, observable_qubit, **kw)

    def parameter_shift_gradient(self, parameters, qubits, observable_qubit, **kw):
        return self.parameter_shift_gradient_for(parameters, qubits, SingleQubitObservable.Z, observable_qubit, **kw)

    def adjoint_gradient_with_inputs(self, inputs, parameters, qubits, observable, observable_qubit, **kw):
        from .gradients import GradientStrategy

        return self._strategy_grad(GradientStrategy.Adjoint, inputs, parameters, qubits, observable, observable_qubit,
                                   **kw)

    def adjoint_gradient(self, parameters, qubits, observable, observable_qubit, **kw):
        return self.adjoint_gradient_with_inputs([], parameters, qubits, observable, observable_qubit, **kw)
