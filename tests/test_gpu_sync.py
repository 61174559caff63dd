"""GPU: the refactor's two ways of ending a dependency level.

With progress flags each warp of the refactor CTA publishes the levels it
has done and waits only for the warps whose earlier work it reads or
overwrites (the waits the stream compiler found by analysing the barrier
form of the same schedule); with barriers every warp meets every other at
every level.  Both run the same operations on every value in the same
order, so the batched solves must agree bit for bit, in both precisions, on
a grid with hundreds of levels (case2000) and on the N-1 grid (case10000,
where the FP32 plan has one larger ring)."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from gridoxide_gb300 import solver as S
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu


def _solve_both(gox, yb, bus_type, args, kw):
    out = {}
    S.set_autotune(False)
    try:
        for flags in (True, False):
            S.set_refactor_sync(flags)
            topo = gox.Topology(yb, bus_type)
            out[flags] = topo.solve(*args, **kw)
            inf = topo.info()
            assert inf["rf32_progress_flags"] == int(flags)
            if flags:
                assert inf["rf32_flag_waits"] > 0
    finally:
        S.set_autotune(True)
        S.set_refactor_sync(False)  # the default
    return out


def _same(a, b):
    np.testing.assert_array_equal(a.status, b.status)
    np.testing.assert_array_equal(a.iterations, b.iterations)
    np.testing.assert_array_equal(a.voltage_mag, b.voltage_mag)
    np.testing.assert_array_equal(a.voltage_ang, b.voltage_ang)
    np.testing.assert_array_equal(a.max_mismatch, b.max_mismatch)


@pytest.mark.parametrize("precision", [0, 1])
def test_progress_flags_equal_barriers_case2000(gox, precision):
    fx = load_fixture("case2000")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    p, q = G.load_scenarios(g, 320, 0.15, 4242)
    r = _solve_both(gox, yb, g.bus_type, (p, q, g.vm, g.va),
                    dict(tol=1e-8, max_iter=20, precision=precision))
    assert np.all(r[True].status == gox.GOX_CONVERGED)
    _same(r[True], r[False])


def test_progress_flags_equal_barriers_case10000_outages(gox):
    g = G.config_grid("case10000")
    yb = G.build_ybus(g)
    B = 64
    p = np.tile(g.p_spec, (B, 1))
    q = np.tile(g.q_spec, (B, 1))
    rng = np.random.default_rng(9)
    outage = G.outage_deltas(g, yb, rng.choice(np.flatnonzero(~G.bridges(g)), size=B))
    r = _solve_both(gox, yb, g.bus_type, (p, q, g.vm, g.va),
                    dict(tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_MIXED, outage=outage))
    _same(r[True], r[False])
