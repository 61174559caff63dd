"""GPU: split solves (gox_topo_set_split).  A batch of 4,096+ scenarios solved
as concurrent parts of whole groups (part k by the k-th clone of the topology
on its own stream) gives the unsplit results bit for bit: mixed precision,
with outages, 2, 3 (uneven parts) and 8 parts, through the host and the
device entries."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,outage,parts", [("mixed", False, 2), ("mixed", True, 2),
                                               ("mixed", True, 3), ("mixed", False, 8)])
def test_split_equals_unsplit(gox, prec, outage, parts):
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 4096 + 96  # 131 groups, the last one of 32: two parts of 2,112 and 2,080 scenarios
    p, q = G.load_scenarios(g, B, 0.15, 51)
    out = None
    if outage:
        rng = np.random.default_rng(52)
        out = G.outage_deltas(g, yb, rng.choice(np.flatnonzero(~G.bridges(g)), B))
    precision = gox.GOX_PRECISION_MIXED if prec == "mixed" else gox.GOX_PRECISION_FP64
    topo = gox.Topology(yb, g.bus_type)
    topo.set_split(1)
    ref = topo.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True)
    ref = topo.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True)
    for k in (parts, 0):  # the given parts, then parts by batch size (the default)
        topo.set_split(k)
        res = topo.solve(p, q, g.vm, g.va, precision=precision, outage=out, history=True)
        for a, b in ((res.voltage_mag, ref.voltage_mag), (res.voltage_ang, ref.voltage_ang),
                     (res.iterations, ref.iterations), (res.status, ref.status),
                     (res.max_mismatch, ref.max_mismatch), (res.history, ref.history)):
            np.testing.assert_array_equal(a, b)
    assert np.all(ref.status == gox.GOX_CONVERGED)
    for bad in (-1, 9):
        with pytest.raises(gox.GoxError):
            topo.set_split(bad)


def test_split_device_entry(gox):
    torch = pytest.importorskip("torch")
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 4096
    p, q = G.load_scenarios(g, B, 0.15, 53)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_split(1)
    ref = topo.solve(p, q, g.vm, g.va)
    topo.set_split(2)
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    n = g.n_bus
    vm = torch.empty((B, n), dtype=torch.float64, device="cuda")
    va = torch.empty_like(vm)
    it = torch.empty(B, dtype=torch.int32, device="cuda")
    st = torch.empty_like(it)
    mm = torch.empty(B, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        P, Q, V, A = d(p), d(q), d(g.vm), d(g.va)
        for _ in range(3):
            topo.solve_device(P, Q, V, A, vm, va, it, st, mm, stream=s)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(vm.cpu().numpy(), ref.voltage_mag)
    np.testing.assert_array_equal(it.cpu().numpy(), ref.iterations)
