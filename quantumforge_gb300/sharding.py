"""Sharding of independent work across ranks, one process per GPU.

The dense state vector of one circuit does not shard (it runs as replicas),
but two workloads are made of independent units:

* the instances of a batched QAOA MaxCut evaluation (cost and gradient per
  instance, ``maxcut_qaoa_expectation`` over ``qaoa_maxcut`` circuits,
  src/qaoa_transfer.rs:221-236, src/algorithms.rs:110-137);
* the +/- evaluations of a parameter-shift or central finite-difference
  gradient, one pair per rotation occurrence
  (``parameter_shift_gradient_with_inputs``, src/lib.rs:3516-3546, with
  ``run_with_shift``, src/lib.rs:4677-4740; FD: src/gradients.rs:344-375).

Units are assigned by a deterministic longest-processing-time rule on a cost
model (2^n times the gate count), every rank evaluates its share on its own
GPU, and one all-gather of the float64 result rows hands every rank the full
result in the original unit order. That gather is the only collective; no
state-vector data moves between ranks.
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi


def partition(costs, world: int) -> list[list[int]]:
    """Units by decreasing cost, each to the least-loaded rank (ties: lower
    unit index first, lower rank first); every part in increasing order."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    loads = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += float(costs[i])
    for p in parts:
        p.sort()
    return parts


def _rank_world(group=None):
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is a dependency of the package's tests
        return 0, 1
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def gather_rows(rows: np.ndarray, parts: list[list[int]], rank: int, width: int, group=None) -> np.ndarray:
    """Every rank's rows (len(parts[rank]) x width, float64) gathered into the
    full (units x width) array in unit order, on every rank."""
    total = sum(len(p) for p in parts)
    out = np.empty((total, width), dtype=np.float64)
    if len(parts) == 1:
        out[parts[0]] = rows
        return out
    import torch
    import torch.distributed as dist

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else torch.device("cpu")
    m = max(len(p) for p in parts)
    local = torch.zeros((m, width), dtype=torch.float64, device=dev)
    if len(parts[rank]):
        local[: len(parts[rank])] = torch.from_numpy(np.ascontiguousarray(rows, dtype=np.float64)).to(dev)
    bufs = [torch.empty((m, width), dtype=torch.float64, device=dev) for _ in parts]
    dist.all_gather(bufs, local, group=group)
    for r, p in enumerate(parts):
        if p:
            out[p] = bufs[r][: len(p)].cpu().numpy()
    return out


def run_sharded(costs, evaluate, width: int, group=None) -> np.ndarray:
    """evaluate(indices) -> (len(indices) x width) rows for this rank's units;
    returns the full result on every rank."""
    rank, world = _rank_world(group)
    parts = partition(costs, world)
    mine = parts[rank]
    rows = np.asarray(evaluate(mine) if mine else np.empty((0, width)), dtype=np.float64).reshape(len(mine), width)
    return gather_rows(rows, parts, rank, width, group)


def qaoa_cost_model(n: int, n_edges: int, p: int) -> float:
    """2^n times the gate count of qaoa_maxcut: n + p(3|E| + n)."""
    return float(2 ** n) * (n + p * (3 * n_edges + n))


def qaoa_maxcut_sharded(problems, p: int, gammas, betas, tile_qubits=None, backend=None, group=None, evaluate=None):
    """Batched QAOA MaxCut (cost, gradient[2p]) per instance, instances split
    across the group's ranks. `evaluate(indices, gammas, betas)` replaces the
    GPU batch (for host tests); it returns rows [cost, grad...]."""
    g = np.asarray(gammas, dtype=np.float64).reshape(len(problems), p)
    b = np.asarray(betas, dtype=np.float64).reshape(len(problems), p)

    def gpu_rows(idx):
        from .qaoa import QaoaBatch

        batch = QaoaBatch([problems[i] for i in idx], p, tile_qubits=tile_qubits, backend=backend)
        cost, grad = batch.run(g[idx], b[idx])
        return np.column_stack([cost, grad])

    fn = (lambda idx: evaluate(idx, g[idx], b[idx])) if evaluate is not None else gpu_rows
    costs = [qaoa_cost_model(int(n), len(es), p) for n, es in problems]
    out = run_sharded(costs, fn, 1 + 2 * p, group)
    return out[:, 0].copy(), out[:, 1:].copy()


_ROT_GATE = {_abi.PAULI_X: _abi.GATE_RX, _abi.PAULI_Y: _abi.GATE_RY, _abi.PAULI_Z: _abi.GATE_RZ}


def shifted_ops(ops: np.ndarray, k: int, params, delta: float) -> np.ndarray:
    """The op list with rotation occurrence k replaced by the fixed-angle gate
    R_axis(params[param_k] + delta): run_with_shift at one occurrence."""
    out = ops.copy()
    r = ops[k]
    if int(r["kind"]) != _abi.OP_ROTATION:
        raise ValueError(f"op {k} is not a parameterized rotation")
    out[k]["kind"] = _abi.OP_GATE
    out[k]["gate"] = _ROT_GATE[int(r["gate"])]
    out[k]["theta"] = float(params[int(r["param"])]) + delta
    out[k]["param"] = 0
    return out


def shift_gradient_sharded(ops: np.ndarray, qubits: int, params, hamiltonian, rule: str = "shift", h: float = 1e-4,
                           dtype: str = "c128", backend=None, group=None, energy=None, exec_opts=None):
    """Parameter-shift (rule "shift", +/- pi/2, factor 1/2) or central
    finite-difference (rule "fd", +/- h, factor 1/(2h)) gradient with the
    occurrences split across the group's ranks. `energy(ops, params)` replaces
    the GPU expectation (for host tests). Returns the gradient (float64)."""
    if rule not in ("shift", "fd"):
        raise ValueError("rule must be 'shift' or 'fd'")
    if rule == "fd" and not (math.isfinite(h) and h > 0):
        raise ValueError("the finite-difference step must be positive and finite")
    params = np.asarray(params, dtype=np.float64)
    occ = [k for k in range(len(ops)) if int(ops[k]["kind"]) == _abi.OP_ROTATION]
    delta = math.pi / 2 if rule == "shift" else h

    if energy is None:
        import ctypes as C

        from ._native import check, load, ptr
        from .core import _as_terms, _dtype_code, _exec, default_backend

        be = backend or default_backend()
        terms = _as_terms(hamiltonian)

        def energy(o, prm):
            v = C.c_double()
            empty = np.zeros(0, dtype=np.float64)
            check(load().qf_expectation(be.handle, int(qubits), _dtype_code(dtype), ptr(o), len(o), ptr(prm), prm.size,
                                        ptr(empty), 0, ptr(terms), len(terms), _exec(exec_opts), C.byref(v)))
            return v.value

    def rows(idx):
        return [[energy(shifted_ops(ops, occ[j], params, delta), params),
                 energy(shifted_ops(ops, occ[j], params, -delta), params)] for j in idx]

    out = run_sharded([1.0] * len(occ), rows, 2, group)
    grad = np.zeros(params.size, dtype=np.float64)
    for j, k in enumerate(occ):
        d = out[j, 0] - out[j, 1]
        grad[int(ops[k]["param"])] += 0.5 * d if rule == "shift" else d / (2.0 * h)
    return grad
