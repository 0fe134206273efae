"""Batched QAOA MaxCut against the oracle: the cost is maxcut_expectation of
the qaoa_maxcut circuit; the gradient is the oracle's parameter shift on the
same circuit with shared parameters theta_l = 2 gamma_l, phi_l = 2 beta_l.
complex64 state: cost within 1e-5 relative, gradient within 1e-4."""
import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import PauliSum
from quantumforge_gb300 import workloads as W
from quantumforge_gb300.qaoa import QaoaBatch, autotune_tiles

pytestmark = pytest.mark.gpu


def oracle_cost_grad(n, edges, gam, bet):
    p = len(gam)
    ops = W.qaoa_param_circuit(n, edges, p)
    params = np.concatenate([2 * np.asarray(gam), 2 * np.asarray(bet)])
    H = PauliSum.maxcut(edges).array()
    e, g = O.adjoint_uncompute(ops, n, params, H)
    return e, 2 * g


def test_param_circuit_matches_the_reference_builder():
    edges = O.random_3_regular(8, 3)
    gam, bet = [0.3, 1.1], [0.7, 0.2]
    a = O.run(W.qaoa_maxcut(8, edges, 2, bet, gam), 8)
    b = O.run(W.qaoa_param_circuit(8, edges, 2), 8, params=np.concatenate([2 * np.array(gam), 2 * np.array(bet)]))
    assert np.abs(a - b).max() < 1e-12
    assert abs(O.maxcut_expectation(a, edges) - O.pauli_expectation(a, PauliSum.maxcut(edges).array()).real) < 1e-12


@pytest.mark.parametrize("tiles", [None, {4: 4, 6: 4, 8: 5, 10: 6, 12: 7}])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_oracle(backend, tiles, graph):
    rng = np.random.default_rng(4)
    problems = []
    for i, n in enumerate([4, 6, 8, 10, 12, 12, 10, 8, 6, 4]):
        problems.append((n, O.random_3_regular(n, 100 + i)))
    p = 3
    gam = rng.uniform(0, np.pi, (len(problems), p))
    bet = rng.uniform(0, np.pi / 2, (len(problems), p))
    batch = QaoaBatch(problems, p, tile_qubits=tiles, backend=backend, use_graph=graph)
    cost, grad = batch.run(gam, bet)
    for i, (n, edges) in enumerate(problems):
        e_ref, g_ref = oracle_cost_grad(n, edges, gam[i], bet[i])
        assert abs(cost[i] - e_ref) < 1e-5 * max(1.0, abs(e_ref)), (i, cost[i], e_ref)
        assert np.abs(grad[i] - g_ref).max() < 1e-4, (i, grad[i], g_ref)
    # a second call with new angles (the graph is replayed)
    cost2, grad2 = batch.run(gam * 0.5, bet * 0.5)
    e_ref, g_ref = oracle_cost_grad(problems[3][0], problems[3][1], gam[3] * 0.5, bet[3] * 0.5)
    assert abs(cost2[3] - e_ref) < 1e-5 * max(1.0, abs(e_ref))
    assert np.abs(grad2[3] - g_ref).max() < 1e-4


@pytest.mark.parametrize("graph", [False, True])
def test_batched_passes_match_oracle(backend, graph):
    """Instances above 12 qubits run as batched tile passes per qubit count
    (several instances per count, mixed with per-CTA small instances)."""
    rng = np.random.default_rng(9)
    sizes = [14, 16, 18, 14, 10, 16, 12, 14]
    problems = [(n, O.random_3_regular(n, 300 + i)) for i, n in enumerate(sizes)]
    p = 2
    gam = rng.uniform(0, np.pi, (len(problems), p))
    bet = rng.uniform(0, np.pi / 2, (len(problems), p))
    batch = QaoaBatch(problems, p, backend=backend, use_graph=graph)
    for scale in (1.0, 0.6):  # the second call replays the graph with new angles
        cost, grad = batch.run(gam * scale, bet * scale)
        for i, (n, edges) in enumerate(problems):
            e_ref, g_ref = oracle_cost_grad(n, edges, gam[i] * scale, bet[i] * scale)
            assert abs(cost[i] - e_ref) < 1e-5 * max(1.0, abs(e_ref)), (i, n, cost[i], e_ref)
            assert np.abs(grad[i] - g_ref).max() < 1e-4 * max(1.0, np.abs(g_ref).max()), (i, n, grad[i], g_ref)


def test_config_sizes_at_depth_four_match_oracle(backend):
    """Every qubit count of the 4096-instance workload (12..20, p = 4, gamma in
    [0, pi], beta in [0, pi/2]), the 20-qubit class included, at non-zero
    angles against the oracle's complex128 adjoint; with and without the
    captured graph."""
    import os

    rng = np.random.default_rng(20)
    sizes = [20, 12, 14, 16, 18, 20]
    problems = [(n, O.random_3_regular(n, 900 + i)) for i, n in enumerate(sizes)]
    p = 4
    gam = rng.uniform(0, np.pi, (len(problems), p))
    bet = rng.uniform(0, np.pi / 2, (len(problems), p))
    threads = os.cpu_count() or 1
    refs = []
    for i, (n, edges) in enumerate(problems):
        ops = W.qaoa_param_circuit(n, edges, p)
        params = np.concatenate([2 * gam[i], 2 * bet[i]])
        e_ref, g_ref = O.adjoint_uncompute(ops, n, params, PauliSum.maxcut(edges).array(), threads=threads)
        refs.append((e_ref, 2 * g_ref))
    for graph in (False, True):
        cost, grad = QaoaBatch(problems, p, backend=backend, use_graph=graph).run(gam, bet)
        for i, (n, _) in enumerate(problems):
            e_ref, g_ref = refs[i]
            assert abs(cost[i] - e_ref) < 1e-5 * max(1.0, abs(e_ref)), (graph, i, n, cost[i], e_ref)
            assert np.abs(grad[i] - g_ref).max() < 1e-4 * max(1.0, np.abs(g_ref).max()), (graph, i, n, grad[i], g_ref)


def test_uniform_superposition_cuts_half_the_edges(backend):
    # gamma = beta = 0: the state is H^n |0>, every edge is cut with probability 1/2
    problems = [(n, O.random_3_regular(n, n)) for n in (12, 14, 16, 20, 22, 24)]
    batch = QaoaBatch(problems, 2, backend=backend)
    cost, grad = batch.run(np.zeros((len(problems), 2)), np.zeros((len(problems), 2)))
    for (n, edges), c in zip(problems, cost):
        assert abs(c - 0.5 * len(edges)) < 1e-5 * len(edges), (n, c)


def test_more_than_24_qubits_is_rejected(backend):
    from quantumforge_gb300 import QuantumError

    with pytest.raises(QuantumError):
        QaoaBatch([(26, O.random_3_regular(26, 1))], 1, backend=backend).run(np.zeros((1, 1)), np.zeros((1, 1)))


def test_autotune_returns_a_choice_per_size(backend, tmp_path):
    from quantumforge_gb300.qaoa import load_tiles, save_tiles

    problems = [(n, O.random_3_regular(n, n + 7)) for n in (10, 12, 14) for _ in range(8)]
    best = autotune_tiles(problems, 2, candidates=(8, 10, 12), large_candidates=(0, 12), reps=1, backend=backend)
    assert set(best) == {10, 12, 14} and best[10] in (8, 10, 12) and best[12] in (8, 10, 12) and best[14] in (0, 12)
    save_tiles(best, tmp_path / "tiles.json")
    assert load_tiles(tmp_path / "tiles.json") == best


@pytest.mark.parametrize("k", [12, 11])
def test_one_cta_per_large_instance_matches_oracle(backend, k):
    """Instances above 12 qubits on the one-CTA-per-instance kernel (a tile
    width given for their qubit count) instead of the batched passes."""
    rng = np.random.default_rng(31)
    sizes = [14, 16, 18, 12, 14]
    problems = [(n, O.random_3_regular(n, 500 + i)) for i, n in enumerate(sizes)]
    p = 2
    gam = rng.uniform(0, np.pi, (len(problems), p))
    bet = rng.uniform(0, np.pi / 2, (len(problems), p))
    batch = QaoaBatch(problems, p, tile_qubits={14: k, 16: k, 18: k}, backend=backend)
    cost, grad = batch.run(gam, bet)
    for i, (n, edges) in enumerate(problems):
        e_ref, g_ref = oracle_cost_grad(n, edges, gam[i], bet[i])
        assert abs(cost[i] - e_ref) < 1e-5 * max(1.0, abs(e_ref)), (i, n, cost[i], e_ref)
        assert np.abs(grad[i] - g_ref).max() < 1e-4 * max(1.0, np.abs(g_ref).max()), (i, n, grad[i], g_ref)


@pytest.mark.parametrize("graph", [False, True])
def test_dense_graphs_in_batched_passes_match_oracle(backend, graph):
    """Cut tables of graphs with many edges among the low qubits (edges inside
    qubits 0..3, from them to higher qubits and above them): the complete graph
    on 14 qubits (91 edges), a clique on qubits 0..7 with a path to qubit 12,
    a star from qubit 0 over 16 qubits with a ring."""
    k14 = [(u, v, 1.0) for u in range(14) for v in range(u + 1, 14)]
    clique = [(u, v, 1.0) for u in range(8) for v in range(u + 1, 8)] + [(q, q + 1, 1.0) for q in range(7, 12)]
    star = [(0, v, 1.0) for v in range(1, 16)] + [(q, q + 1, 1.0) for q in range(1, 15)]
    problems = [(14, k14), (13, clique), (16, star), (13, clique)]
    rng = np.random.default_rng(31)
    p = 2
    gam = rng.uniform(0, np.pi, (len(problems), p))
    bet = rng.uniform(0, np.pi / 2, (len(problems), p))
    cost, grad = QaoaBatch(problems, p, backend=backend, use_graph=graph).run(gam, bet)
    for i, (n, edges) in enumerate(problems):
        e_ref, g_ref = oracle_cost_grad(n, edges, gam[i], bet[i])
        assert abs(cost[i] - e_ref) < 1e-5 * max(1.0, abs(e_ref)), (i, n, cost[i], e_ref)
        assert np.abs(grad[i] - g_ref).max() < 1e-4 * max(1.0, np.abs(g_ref).max()), (i, n, grad[i], g_ref)


@pytest.mark.parametrize("n", [22, 24])
def test_batched_passes_above_twenty_qubits_match_oracle(backend, n):
    """Pass B of a 21..24-qubit class has windows at tile bits 8, 4 and 0 with
    the bits below L = 24 - n masked out (at 24 qubits, L = 0, its tiles load
    with plain copies): one instance at depth 1 against the oracle (22 qubits:
    a 3-regular graph; 24 qubits: a sparse graph with edges across pass A's and
    pass B's qubits, to keep the oracle's run short)."""
    import os

    rng = np.random.default_rng(40 + n)
    if n == 22:
        edges = O.random_3_regular(n, 1200)
    else:
        pairs = [(0, 23), (1, 12), (2, 20), (5, 17), (11, 12), (13, 22), (3, 7), (8, 15), (18, 21), (6, 9)]
        edges = [(u, v, 1.0) for u, v in pairs]
    p = 1
    gam = rng.uniform(0, np.pi, (1, p))
    bet = rng.uniform(0, np.pi / 2, (1, p))
    cost, grad = QaoaBatch([(n, edges)], p, backend=backend, use_graph=False).run(gam, bet)
    ops = W.qaoa_param_circuit(n, edges, p)
    params = np.concatenate([2 * gam[0], 2 * bet[0]])
    e_ref, g_ref = O.adjoint_uncompute(ops, n, params, PauliSum.maxcut(edges).array(), threads=os.cpu_count() or 1)
    assert abs(cost[0] - e_ref) < 1e-5 * max(1.0, abs(e_ref)), (cost[0], e_ref)
    assert np.abs(grad[0] - 2 * g_ref).max() < 1e-4 * max(1.0, np.abs(2 * g_ref).max()), (grad[0], 2 * g_ref)
