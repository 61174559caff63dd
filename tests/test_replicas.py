"""Replica sharding on CPU ranks (gloo, world size 2): every rank solves a
contiguous block of the batch and gathers the reports; the gathered
reports equal one process solving the whole batch, and the timing is the
max over ranks.  The per-rank solver here is the oracle (the GPU path uses
the same host logic with Topology.solve)."""
import os
import socket

import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from gridoxide_gb300 import replicas
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture


def test_shard_bounds_cover_the_batch():
    for B in (0, 1, 7, 32, 4096, 4097):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard_bounds(B, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == B
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard_bounds(10, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("B", [9, 16])
def test_two_gloo_ranks_gather_the_single_process_result(oracle_mod, tmp_path, B):
    import torch.multiprocessing as mp

    import replica_worker

    world = 2
    mp.spawn(replica_worker.run, args=(world, _free_port(), str(tmp_path), B), nprocs=world,
             join=True)
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    p, q = G.load_scenarios(g, B, 0.15, 21)
    ref = ot.batch_solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, threads=1)
    for r in range(world):
        with np.load(os.path.join(tmp_path, f"rank{r}.npz")) as z:
            np.testing.assert_array_equal(z["vm"], ref["vm"])
            np.testing.assert_array_equal(z["va"], ref["va"])
            np.testing.assert_array_equal(z["iters"], ref["iters"])
            np.testing.assert_array_equal(z["status"], ref["status"])
            np.testing.assert_array_equal(z["max_mismatch"], ref["max_mis"])
            assert float(z["tmax"]) == 10.0 * world
