"""The sharded entry points with their GPU evaluators, on one rank: the same
numbers as the batch kernel and the engine's own parameter-shift gradient."""
import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import sharding as S
from quantumforge_gb300 import workloads as W
from quantumforge_gb300.qaoa import QaoaBatch

pytestmark = pytest.mark.gpu


def test_qaoa_sharded_equals_the_batch_kernel(backend):
    problems, gam, bet = W.qaoa_batch_problems(count=24, sizes=(6, 8, 10), p=2, seed=5)
    cost, grad = S.qaoa_maxcut_sharded(problems, 2, gam, bet, backend=backend)
    c2, g2 = QaoaBatch(problems, 2, backend=backend).run(gam, bet)
    assert np.array_equal(cost, c2) and np.array_equal(grad, g2)


@pytest.mark.parametrize("rule", ["shift", "fd"])
def test_shift_gradient_sharded_matches_the_oracle(backend, rule):
    n = 8
    ops, params, H = W.vqe_xxz(n, 2, seed=9)
    g = S.shift_gradient_sharded(ops, n, params, H, rule=rule, h=1e-3, dtype="c128", backend=backend)
    want = (O.parameter_shift(ops, n, params, H.array()) if rule == "shift"
            else O.finite_difference(ops, n, params, H.array(), 1e-3))
    assert np.abs(g - want).max() < 1e-10
