"""GPU: many topologies solved together (gox_multi_solve).

Two forms: one persistent launch whose CTAs each run a (topology, group)
item's whole Newton loop, taken from a queue; and one Newton loop whose
phases are one launch each over every topology still running.  In both,
every scenario's result must equal, bit for bit, the same batch solved
alone by Topology.solve -- on three family grids of uneven size and batch
(one of them with several groups and stragglers), in both precisions --
and the FP64 results must match the oracle (the reference's algorithm)
within 1e-9 with equal iteration counts."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import oracle_topology

pytestmark = pytest.mark.gpu

# (buses, grid seed, scenarios)
SPECS = [(90, 5, 40), (1300, 6, 200), (6000, 7, 70)]


def _jobs(gox):
    out = []
    for n, gs, b in SPECS:
        g = G.family_grid(n, gs)
        yb = G.build_ybus(g)
        p, q = G.load_scenarios(g, b, 0.15, 100 + gs)
        out.append((g, yb, p, q))
    return out


def _same(a, b):
    np.testing.assert_array_equal(a.status, b.status)
    np.testing.assert_array_equal(a.iterations, b.iterations)
    np.testing.assert_array_equal(a.voltage_mag, b.voltage_mag)
    np.testing.assert_array_equal(a.voltage_ang, b.voltage_ang)
    np.testing.assert_array_equal(a.max_mismatch, b.max_mismatch)


@pytest.mark.parametrize("persistent", [True, False])
@pytest.mark.parametrize("precision", [0, 1])
def test_multi_equals_alone(gox, precision, persistent):
    from gridoxide_gb300 import solver as S
    data = _jobs(gox)
    kw = dict(tol=1e-8, max_iter=20, precision=precision)
    alone = [gox.Topology(yb, g.bus_type).solve(p, q, g.vm, g.va, **kw) for g, yb, p, q in data]
    topos = [gox.Topology(yb, g.bus_type) for g, yb, _, _ in data]
    S.set_multi_persistent(persistent)
    try:
        jobs = [(t, p, q, g.vm, g.va) for t, (g, yb, p, q) in zip(topos, data)]
        mixed = gox.multi_solve(jobs, **kw)
        for a, m in zip(alone, mixed):
            assert np.all(a.status == gox.GOX_CONVERGED)
            _same(a, m)
        # the same topologies again (fixed pivot orders, tuned plans), into
        # caller-given result arrays (filled with NaN first): same bits
        bufs = [gox.BatchResult(np.full(p.shape, np.nan), np.full(p.shape, np.nan),
                                np.full(p.shape[0], -7, np.int32),
                                np.full(p.shape[0], -7, np.int32),
                                np.full(p.shape[0], np.nan)) for g, yb, p, q in data]
        again = gox.multi_solve(jobs, out=bufs, **kw)
        for a, m, b in zip(alone, again, bufs):
            assert m is b
            _same(a, m)
        # a budget that runs out: MaxIterations reported as alone
        short = dict(kw, max_iter=2)
        alone2 = [gox.Topology(yb, g.bus_type).solve(p, q, g.vm, g.va, **short)
                  for g, yb, p, q in data]
        for a, m in zip(alone2, gox.multi_solve(jobs, **short)):
            assert np.any(a.status == gox.GOX_MAX_ITERATIONS)
            _same(a, m)
    finally:
        S.set_multi_persistent(False)  # the default


def test_multi_fp64_matches_oracle(gox, oracle_mod):
    data = _jobs(gox)
    topos = [gox.Topology(yb, g.bus_type) for g, yb, _, _ in data]
    res = gox.multi_solve([(t, p, q, g.vm, g.va) for t, (g, yb, p, q) in zip(topos, data)],
                          tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_FP64)
    g, yb, p, q = data[1]
    ot = oracle_topology(oracle_mod, yb, g.bus_type)
    ref = ot.batch_solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, threads=8)
    r = res[1]
    np.testing.assert_array_equal(r.iterations, ref["iters"])
    assert np.max(np.abs(r.voltage_mag - ref["vm"])) < 1e-9
    assert np.max(np.abs(r.voltage_ang - ref["va"])) < 1e-9


def test_multi_rejects_a_topology_twice(gox):
    g = G.family_grid(90, 5)
    yb = G.build_ybus(g)
    t = gox.Topology(yb, g.bus_type)
    p, q = G.load_scenarios(g, 4, 0.15, 1)
    with pytest.raises(gox.GoxError):
        gox.multi_solve([(t, p, q, g.vm, g.va), (t, p, q, g.vm, g.va)])
