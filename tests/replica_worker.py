"""One rank of the CPU replica test: solves its shard of a case118 batch with
the oracle (as the per-rank solver) and writes the gathered reports."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def run(rank: int, world: int, port: int, outdir: str, B: int) -> None:
    for p in (ROOT, os.path.join(ROOT, "oracle"), HERE):
        if p not in sys.path:
            sys.path.insert(0, p)
    import numpy as np
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", world_size=world,
                            rank=rank)
    try:
        import oracle as O
        from gridoxide_gb300 import grids as G
        from gridoxide_gb300 import replicas
        from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture

        fx = load_fixture("case118")
        g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
        ot = oracle_topology(O, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
        p, q = G.load_scenarios(g, B, 0.15, 21)

        def solve(p, q, vm0, va0, outage=None):
            r = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=1, outage=outage)
            return {"vm": r["vm"], "va": r["va"], "iters": r["iters"], "status": r["status"],
                    "max_mismatch": r["max_mis"]}

        rep = replicas.solve_replicas(solve, p, q, g.vm, g.va)
        tmax = replicas.max_over_ranks(10.0 * (rank + 1))
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), tmax=tmax, **rep)
    finally:
        dist.destroy_process_group()
