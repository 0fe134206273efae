"""Batched QAOA MaxCut on the GPU.

``QaoaBatch`` evaluates, for many MaxCut instances of uneven qubit counts, the
expected cut of the QAOA state
(``maxcut_qaoa_expectation``, src/qaoa_transfer.rs:221-236, on the circuit of
``algorithms::qaoa_maxcut``, src/algorithms.rs:110-137, unit weights) and its
exact gradient with respect to every gamma_l and beta_l: instances of up to 12
qubits one CTA each, larger ones (up to 24) as tile passes batched over all
instances of a qubit count, or one CTA each when asked. ``autotune_tiles``
picks, per qubit count, the shared-memory tile width of the small instances
and, above 12 qubits, batched passes or one CTA per instance, by timing
sub-batches; ``save_tiles`` / ``load_tiles`` persist the table.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from ._native import QuantumError, check, load, ptr
from .core import default_backend


class QaoaInstance(C.Structure):
    _fields_ = [("qubits", C.c_uint32), ("edge_begin", C.c_uint32), ("edge_count", C.c_uint32),
                ("tile_qubits", C.c_uint32)]


class QaoaOpts(C.Structure):
    _fields_ = [("use_graph", C.c_int32), ("tile_qubits", C.c_int32 * 33)]


_SIG_DONE = False


def _lib():
    global _SIG_DONE
    lib = load()
    if not _SIG_DONE:
        lib.qf_qaoa_maxcut_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_uint32,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.qf_qaoa_maxcut_batch.restype = C.c_int
        _SIG_DONE = True
    return lib


class QaoaBatch:
    """A fixed list of MaxCut problems [(n, [(u, v, w), ...]), ...] at depth p."""

    def __init__(self, problems, p: int, tile_qubits: dict | None = None, backend=None, use_graph: bool = True):
        self.p = int(p)
        self.backend = backend or default_backend()
        self.n_inst = len(problems)
        inst = (QaoaInstance * self.n_inst)()
        edges = []
        for i, (n, es) in enumerate(problems):
            for u, v, w in es:
                if w != 1.0:
                    raise QuantumError(17, "the batched QAOA kernel takes unit edge weights")
            inst[i].qubits = int(n)
            inst[i].edge_begin = len(edges)
            inst[i].edge_count = len(es)
            inst[i].tile_qubits = 0
            edges.extend((int(u), int(v)) for u, v, _ in es)
        self._inst = inst
        self._edges = np.ascontiguousarray(np.array(edges, dtype=np.uint32).reshape(-1))
        self.opts = QaoaOpts()
        self.opts.use_graph = 1 if use_graph else 0
        for n, k in (tile_qubits or {}).items():
            self.opts.tile_qubits[int(n)] = int(k)

    def run(self, gammas, betas):
        """Returns (cost[n_inst], grad[n_inst, 2p]) with grad rows [dC/dgamma_l..., dC/dbeta_l...]."""
        g = np.ascontiguousarray(gammas, dtype=np.float64).reshape(self.n_inst, self.p)
        b = np.ascontiguousarray(betas, dtype=np.float64).reshape(self.n_inst, self.p)
        cost = np.empty(self.n_inst, dtype=np.float64)
        grad = np.empty((self.n_inst, 2 * self.p), dtype=np.float64)
        check(_lib().qf_qaoa_maxcut_batch(self.backend.handle, C.cast(self._inst, C.c_void_p), self.n_inst,
                                          ptr(self._edges), self._edges.size // 2, self.p, ptr(g), ptr(b), ptr(cost),
                                          ptr(grad), C.byref(self.opts)))
        return cost, grad


def autotune_tiles(problems, p: int, candidates=(8, 9, 10, 11, 12), reps: int = 2, backend=None,
                   large_candidates=(0, 12, 11), max_large: int = 24) -> dict:
    """Best execution per qubit count, timed on the sub-batch of that count
    (at most 256 instances). Up to 12 qubits: the tile width of the
    one-CTA-per-instance kernel, from `candidates`. Above 12 (up to
    `max_large`): 0 = batched tile passes over every instance of the count, or
    one CTA per instance with tiles of a width in `large_candidates`."""
    rng = np.random.default_rng(0)
    best = {}
    by_n: dict[int, list] = {}
    for prob in problems:
        if int(prob[0]) <= max_large:
            by_n.setdefault(int(prob[0]), []).append(prob)
    for n, probs in sorted(by_n.items()):
        probs = probs[: max(8, min(len(probs), 256))]
        g = rng.uniform(0, np.pi, (len(probs), p))
        b = rng.uniform(0, np.pi / 2, (len(probs), p))
        timings = {}
        cands = candidates if n <= 12 else large_candidates
        for k in cands:
            if n <= 12 and k > n and k != cands[0]:
                continue
            batch = QaoaBatch(probs, p, tile_qubits={n: k}, backend=backend, use_graph=False)
            batch.run(g, b)
            t0 = time.perf_counter()
            for _ in range(reps):
                batch.run(g, b)
            timings[k] = (time.perf_counter() - t0) / reps
        best[n] = min(timings, key=timings.get)
    return best


def save_tiles(tiles: dict, path) -> None:
    """Persist an autotuned table ({qubits: tile}) as JSON."""
    import json
    from pathlib import Path

    Path(path).write_text(json.dumps({str(k): int(v) for k, v in sorted(tiles.items())}))


def load_tiles(path) -> dict:
    """A table written by save_tiles."""
    import json
    from pathlib import Path

    return {int(k): int(v) for k, v in json.loads(Path(path).read_text()).items()}
