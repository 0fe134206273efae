"""Rank body of the two-process sharding tests (gloo, CPU): the oracle is the
per-unit evaluator, the sharding, partition and gather are the product's."""
import os

import numpy as np


def qaoa_rows(problems, p):
    import oracle as O
    from quantumforge_gb300 import workloads as W

    def evaluate(idx, g, b):
        rows = []
        for j, i in enumerate(idx):
            n, es = problems[i]
            a = O.run(W.qaoa_maxcut(n, es, p, b[j], g[j]), n)
            rows.append([O.maxcut_expectation(a, es)] + list(g[j]) + list(b[j]))
        return np.array(rows)

    return evaluate


def worker(rank, world, port, out_dir, case):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle as O
        from quantumforge_gb300 import sharding as S
        from quantumforge_gb300 import workloads as W

        if case == "shift":
            n = 6
            ops, params, H = W.vqe_xxz(n, 2, seed=4)
            g = S.shift_gradient_sharded(ops, n, params, H, rule="shift",
                                         energy=lambda o, prm: O.energy(o, n, prm, H.array()))
            np.save(os.path.join(out_dir, f"shift_{rank}.npy"), g)
        else:
            problems, gam, bet = W.qaoa_batch_problems(count=9, sizes=(4, 6, 8), p=2, seed=3)
            cost, grad = S.qaoa_maxcut_sharded(problems, 2, gam, bet, evaluate=qaoa_rows(problems, 2))
            np.save(os.path.join(out_dir, f"qaoa_{rank}.npy"), np.column_stack([cost, grad]))
        dist.barrier()
    finally:
        dist.destroy_process_group()
