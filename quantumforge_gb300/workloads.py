"""Seeded synthetic workloads (random circuits, VQE ansatz, QAOA MaxCut).

Every generator draws from ``SmallRng`` so the oracle and the engine see the
same op list for the same seed. Ops are ``qf_op`` records (``_abi.OP_DTYPE``).

* ``random_circuit`` — layered random circuit: each layer applies H, RX, RY or
  RZ (uniform, angles uniform in [0, 2*pi)) to every qubit, then a two-qubit
  layer. ``two_qubit="ladder"`` is a CNOT ladder on (i, i+1) with alternating
  even/odd offsets; ``two_qubit="mixed"`` draws floor(n/2) disjoint pairs per
  layer, half from the alternating nearest-neighbour ladder and half
  long-range (|i-j| > 1, uniform over free qubits), each a CNOT, CZ or SWAP
  with equal probability.
* ``hea_vqe`` — hardware-efficient ansatz: per layer a rotation on every
  qubit for each axis in ``axes``, then a CZ or CNOT ring; parameters uniform
  in [-pi, pi).
* ``qaoa_maxcut`` — the reference's ``algorithms::qaoa_maxcut``
  (src/algorithms.rs:110-137) as a parameterised op list.
* ``inverse_circuit`` — C^dagger of a fixed gate list (round-trip checks at
  sizes the oracle cannot run).
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi
from .core import PauliSum, SmallRng

_ROT = {1: _abi.GATE_RX, 2: _abi.GATE_RY, 3: _abi.GATE_RZ}


def random_circuit(n: int, depth: int, seed: int, two_qubit: str = "ladder") -> np.ndarray:
    rng = SmallRng.seeded(seed)
    recs = []
    for layer in range(depth):
        for q in range(n):
            choice = rng.next_u64() % 4
            if choice == 0:
                recs.append((_abi.OP_GATE, _abi.GATE_H, q, 0, 0, 0.0))
            else:
                theta = 2.0 * math.pi * rng.next_f64()
                recs.append((_abi.OP_GATE, _ROT[choice], q, 0, 0, theta))
        if two_qubit == "ladder":
            for i in range(layer % 2, n - 1, 2):
                recs.append((_abi.OP_CNOT, 0, i, i + 1, 0, 0.0))
        elif two_qubit == "mixed":
            used = [False] * n
            n2 = n // 2
            n_nn = n2 // 2
            ladder = list(range(layer % 2, n - 1, 2))
            # Fisher-Yates over the ladder pairs, take n_nn of them
            for i in range(len(ladder) - 1, 0, -1):
                j = rng.next_u64() % (i + 1)
                ladder[i], ladder[j] = ladder[j], ladder[i]
            pairs = []
            for i in ladder[:n_nn]:
                pairs.append((i, i + 1))
                used[i] = used[i + 1] = True
            attempts = 0
            while len(pairs) < n2 and attempts < 64 * n:
                attempts += 1
                a = rng.next_u64() % n
                b = rng.next_u64() % n
                if a == b or abs(a - b) <= 1 or used[a] or used[b]:
                    continue
                used[a] = used[b] = True
                pairs.append((a, b))
            for a, b in pairs:
                kind = (_abi.OP_CNOT, _abi.OP_CZ, _abi.OP_SWAP)[rng.next_u64() % 3]
                recs.append((kind, 0, a, b, 0, 0.0))
        else:
            raise ValueError(two_qubit)
    return _abi.ops_array(recs)


def with_terminal_measurements(ops: np.ndarray, n: int) -> np.ndarray:
    """Append measure(q, q) for every qubit, as the CLI `shots` command does (src/bin/main.rs:593-597)."""
    meas = _abi.ops_array([(_abi.OP_MEASURE, 0, q, 0, q, 0.0) for q in range(n)])
    return np.concatenate([ops, meas])


def hea_vqe(n: int, layers: int, seed: int, axes=(_abi.PAULI_Y, _abi.PAULI_Z), entangler: str = "cz"):
    """Returns (ops, params): rotations use consecutive parameter indices."""
    rng = SmallRng.seeded(seed)
    recs = []
    p = 0
    for _ in range(layers):
        for ax in axes:
            for q in range(n):
                recs.append((_abi.OP_ROTATION, ax, q, 0, p, 0.0))
                p += 1
        for q in range(n):
            j = (q + 1) % n
            if j == q:
                continue
            if entangler == "cz":
                recs.append((_abi.OP_CZ, 0, q, j, 0, 0.0))
            else:
                recs.append((_abi.OP_CNOT, 0, q, j, 0, 0.0))
    params = np.array([-math.pi + 2.0 * math.pi * rng.next_f64() for _ in range(p)], dtype=np.float64)
    return _abi.ops_array(recs), params


def vqe_tfim(n: int = 24, layers: int = 8, seed: int = 3, h: float = 1.0):
    """24-qubit VQE workload: RY.RZ per qubit + CZ ring, TFIM ring Hamiltonian."""
    ops, params = hea_vqe(n, layers, seed, axes=(_abi.PAULI_Y, _abi.PAULI_Z), entangler="cz")
    return ops, params, PauliSum.tfim_ring(n, h)


def vqe_xxz(n: int = 32, layers: int = 4, seed: int = 5, delta: float = 0.5):
    """32-qubit checkpointed-adjoint workload: RX.RY per qubit + CNOT ring, XXZ ring."""
    ops, params = hea_vqe(n, layers, seed, axes=(_abi.PAULI_X, _abi.PAULI_Y), entangler="cnot")
    return ops, params, PauliSum.xxz_ring(n, delta)


def random_3_regular(n: int, seed: int):
    """MaxCutProblem::random_3_regular (src/mps_qaoa.rs:58-95): sorted (u, v, 1.0) edges."""
    assert n >= 4 and n % 2 == 0
    rng = SmallRng.seeded(seed)
    for _ in range(10_000):
        stubs = [v for v in range(n) for _ in range(3)]
        for i in range(len(stubs) - 1, 0, -1):
            j = rng.next_u64() % (i + 1)
            stubs[i], stubs[j] = stubs[j], stubs[i]
        edges = []
        ok = True
        for k in range(0, len(stubs), 2):
            a, b = stubs[k], stubs[k + 1]
            if a == b:
                ok = False
                break
            u, v = min(a, b), max(a, b)
            if any(eu == u and ev == v for eu, ev, _ in edges):
                ok = False
                break
            edges.append((u, v, 1.0))
        if ok:
            return sorted(edges, key=lambda e: (e[0], e[1]))
    raise RuntimeError("failed to sample a 3-regular graph")


def qaoa_param_circuit(n: int, edges, p: int) -> np.ndarray:
    """qaoa_maxcut as a parameterised op list for unit weights: parameter l is
    theta_l = 2*gamma_l (every Rz of layer l), parameter p + l is
    phi_l = 2*beta_l (every Rx of layer l); so dC/dgamma_l = 2 dC/dtheta_l."""
    recs = [(_abi.OP_GATE, _abi.GATE_H, q, 0, 0, 0.0) for q in range(n)]
    for layer in range(p):
        for u, v, _w in edges:
            recs.append((_abi.OP_CNOT, 0, u, v, 0, 0.0))
            recs.append((_abi.OP_ROTATION, _abi.PAULI_Z, v, 0, layer, 0.0))
            recs.append((_abi.OP_CNOT, 0, u, v, 0, 0.0))
        for q in range(n):
            recs.append((_abi.OP_ROTATION, _abi.PAULI_X, q, 0, p + layer, 0.0))
    return _abi.ops_array(recs)


def qaoa_batch_problems(count: int = 4096, sizes=(12, 14, 16, 18, 20), p: int = 4, seed: int = 11):
    """Batched QAOA workload: `count` random 3-regular MaxCut instances with n
    uniform over `sizes`, depth p, gamma uniform in [0, pi], beta in [0, pi/2]."""
    rng = SmallRng.seeded(seed)
    problems, gam, bet = [], [], []
    for i in range(count):
        n = sizes[rng.next_u64() % len(sizes)]
        problems.append((n, random_3_regular(n, seed * 1_000_003 + i)))
        gam.append([math.pi * rng.next_f64() for _ in range(p)])
        bet.append([0.5 * math.pi * rng.next_f64() for _ in range(p)])
    return problems, np.array(gam), np.array(bet)


def qaoa_maxcut(n: int, edges, p: int, betas, gammas) -> np.ndarray:
    """algorithms::qaoa_maxcut (src/algorithms.rs:110-137): H on all; per layer
    CNOT(u,v), Rz(2*gamma*w) on v, CNOT(u,v) for every edge, then Rx(2*beta)
    on every qubit."""
    recs = [(_abi.OP_GATE, _abi.GATE_H, q, 0, 0, 0.0) for q in range(n)]
    for layer in range(p):
        for u, v, w in edges:
            recs.append((_abi.OP_CNOT, 0, u, v, 0, 0.0))
            recs.append((_abi.OP_GATE, _abi.GATE_RZ, v, 0, 0, 2.0 * gammas[layer] * w))
            recs.append((_abi.OP_CNOT, 0, u, v, 0, 0.0))
        for q in range(n):
            recs.append((_abi.OP_GATE, _abi.GATE_RX, q, 0, 0, 2.0 * betas[layer]))
    return _abi.ops_array(recs)


def inverse_circuit(ops: np.ndarray) -> np.ndarray:
    """C^dagger of a fixed gate list: reversed, S/T swapped with their
    adjoints, rotation angles negated (``adjoint_gate``, src/lib.rs:2363-2382);
    CNOT, CZ, SWAP and the other gates are self-inverse."""
    inv = ops[::-1].copy()
    swap = {_abi.GATE_S: _abi.GATE_SDG, _abi.GATE_SDG: _abi.GATE_S, _abi.GATE_T: _abi.GATE_TDG,
            _abi.GATE_TDG: _abi.GATE_T}
    for r in inv:
        if int(r["kind"]) == _abi.OP_GATE:
            g = int(r["gate"])
            r["gate"] = swap.get(g, g)
            if g in (_abi.GATE_RX, _abi.GATE_RY, _abi.GATE_RZ):
                r["theta"] = -r["theta"]
    return inv
