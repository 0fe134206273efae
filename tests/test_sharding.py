"""Host logic of the multi-rank path: cost-balanced partition of independent
units (QAOA instances, shift/FD evaluations), the one all-gather, and the
occurrence shifts of run_with_shift (src/lib.rs:4677-4740). Two-rank runs use
gloo on CPU with the oracle as the per-unit evaluator."""
import socket

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import _abi
from quantumforge_gb300 import sharding as S
from quantumforge_gb300 import workloads as W


def test_partition_covers_every_unit_once_and_balances_cost():
    rng = np.random.default_rng(0)
    costs = [float(2 ** n) for n in rng.choice([12, 14, 16, 18, 20], size=257)]
    for world in (1, 2, 3, 8):
        parts = S.partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
        assert parts == S.partition(costs, world)  # deterministic: every rank computes the same split
        assert all(p == sorted(p) for p in parts)


def test_partition_of_fewer_units_than_ranks():
    parts = S.partition([3.0, 1.0], 4)
    assert parts == [[0], [1], [], []]
    with pytest.raises(ValueError):
        S.partition([1.0], 0)


def test_shifted_ops_replaces_one_occurrence_with_a_fixed_angle_gate():
    ops, params, _ = W.vqe_tfim(4, 1, seed=2)
    k = next(i for i in range(len(ops)) if ops[i]["kind"] == _abi.OP_ROTATION)
    sh = S.shifted_ops(ops, k, params, 0.25)
    assert sh[k]["kind"] == _abi.OP_GATE and sh[k]["gate"] == _abi.GATE_RY
    assert sh[k]["theta"] == params[ops[k]["param"]] + 0.25
    assert np.array_equal(np.delete(sh, k), np.delete(ops, k))
    with pytest.raises(ValueError):
        S.shifted_ops(ops, next(i for i in range(len(ops)) if ops[i]["kind"] != _abi.OP_ROTATION), params, 0.1)


def test_single_rank_shift_and_fd_match_the_oracle():
    n = 5
    ops, params, H = W.vqe_xxz(n, 2, seed=7)
    energy = lambda o, prm: O.energy(o, n, prm, H.array())  # noqa: E731
    g = S.shift_gradient_sharded(ops, n, params, H, rule="shift", energy=energy)
    assert np.abs(g - O.parameter_shift(ops, n, params, H.array())).max() < 1e-12
    g = S.shift_gradient_sharded(ops, n, params, H, rule="fd", h=1e-3, energy=energy)
    assert np.abs(g - O.finite_difference(ops, n, params, H.array(), 1e-3)).max() < 1e-12
    with pytest.raises(ValueError):
        S.shift_gradient_sharded(ops, n, params, H, rule="fd", h=0.0, energy=energy)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("case", ["shift", "qaoa"])
def test_two_gloo_ranks_gather_the_single_rank_result(tmp_path, case):
    torch_mp = pytest.importorskip("torch.multiprocessing")
    from _shard_worker import qaoa_rows, worker

    torch_mp.spawn(worker, args=(2, _free_port(), str(tmp_path), case), nprocs=2, join=True)
    r0, r1 = (np.load(tmp_path / f"{case}_{r}.npy") for r in (0, 1))
    assert np.array_equal(r0, r1)  # every rank holds the whole result
    if case == "shift":
        n = 6
        ops, params, H = W.vqe_xxz(n, 2, seed=4)
        assert np.abs(r0 - O.parameter_shift(ops, n, params, H.array())).max() < 1e-12
    else:
        problems, gam, bet = W.qaoa_batch_problems(count=9, sizes=(4, 6, 8), p=2, seed=3)
        want = qaoa_rows(problems, 2)(list(range(len(problems))), gam, bet)
        assert np.array_equal(r0, want)
