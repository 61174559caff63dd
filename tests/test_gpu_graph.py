"""GPU: the Newton loop as one captured CUDA graph (conditional while / if
nodes; the iteration lives on the device).  The first solve of a
configuration runs the host-driven loop, a repeat of it runs the graph; both
give the same results bit for bit: mixed and FP64, with outages, with a
history, and with a budget that runs out (MaxIterations, the final
mismatch inside the graph)."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu


def _same(a, b):
    for x, y in ((a.voltage_mag, b.voltage_mag), (a.voltage_ang, b.voltage_ang),
                 (a.iterations, b.iterations), (a.status, b.status),
                 (a.max_mismatch, b.max_mismatch)):
        np.testing.assert_array_equal(x, y)
    if a.history is not None:
        np.testing.assert_array_equal(a.history, b.history)


@pytest.mark.parametrize("prec,outage,max_iter", [("mixed", False, 20), ("fp64", False, 20),
                                                  ("mixed", True, 20), ("fp64", False, 2)])
def test_graph_loop_equals_host_loop(gox, prec, outage, max_iter):
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 2048  # batches of 64+ groups of 32 scenarios use the graph
    p, q = G.load_scenarios(g, B, 0.15, 41)
    out = None
    if outage:
        rng = np.random.default_rng(42)
        out = G.outage_deltas(g, yb, rng.choice(np.flatnonzero(~G.bridges(g)), B))
    precision = gox.GOX_PRECISION_MIXED if prec == "mixed" else gox.GOX_PRECISION_FP64
    topo = gox.Topology(yb, g.bus_type)
    first = topo.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True,
                       max_iter=max_iter)
    assert topo.info()["graph_solves"] == 0
    again = topo.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True,
                       max_iter=max_iter)
    third = topo.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True,
                       max_iter=max_iter)
    assert topo.info()["graph_solves"] == 2
    _same(first, again)
    _same(first, third)
    if max_iter == 2:
        assert np.all(first.status == gox.GOX_MAX_ITERATIONS)
    else:
        assert np.all(first.status == gox.GOX_CONVERGED)
    # switched off, the same configuration stays on the host-driven loop
    off = gox.Topology(yb, g.bus_type)
    off.set_graph(False)
    for _ in range(3):
        r = off.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True,
                      max_iter=max_iter)
    assert off.info()["graph_solves"] == 0
    _same(first, r)
    # a small batch stays on the host-driven loop
    small = gox.Topology(yb, g.bus_type)
    for _ in range(3):
        small.solve(p[:64], q[:64], g.vm, g.va, precision=precision, max_iter=max_iter)
    assert small.info()["graph_solves"] == 0
