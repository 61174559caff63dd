"""GPU: the refactor's plan forms give the same bits.

* How a dependency level ends: with CTA barriers every warp of the
  per-group refactor kernel meets every other at every level; with progress
  flags each warp publishes the levels it has done and waits only for the
  warps whose earlier work it reads or overwrites (the waits the stream
  compiler found by analysing the barrier form of the same schedule).
* Where the wide levels run: in the per-group kernel, or in the wide
  kernels -- one launch per leading refactor level (and, after the
  per-group kernel, per level of those columns' backward-substitution rows)
  with one warp per (column or row, group) across every SM.

Every form runs the same operations on every value in the same order, so
the batched solves must agree bit for bit, in both precisions, on a grid
with hundreds of levels (case2000) and on the N-1 grid (case10000, where
the FP32 plan has one larger ring)."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from gridoxide_gb300 import solver as S
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu

# (progress flags, narrowest level the wide kernels take; 0: none)
FORMS = [(False, 0), (True, 0), (False, 64), (True, 16)]


def _solve_forms(gox, yb, bus_type, args, kw):
    out = {}
    S.set_autotune(False)
    try:
        for flags, wide in FORMS:
            S.set_refactor_sync(flags)
            S.set_refactor_wide(wide)
            topo = gox.Topology(yb, bus_type)
            out[(flags, wide)] = topo.solve(*args, **kw)
            inf = topo.info()
            assert inf["rf32_progress_flags"] == int(flags)
            if flags:
                assert inf["rf32_flag_waits"] > 0
            assert (inf["rf32_wide_levels"] > 0) == (wide > 0)
    finally:
        S.set_autotune(True)
        S.set_refactor_sync(False)  # the defaults
        S.set_refactor_wide(0)
    return out


def _same(a, b):
    np.testing.assert_array_equal(a.status, b.status)
    np.testing.assert_array_equal(a.iterations, b.iterations)
    np.testing.assert_array_equal(a.voltage_mag, b.voltage_mag)
    np.testing.assert_array_equal(a.voltage_ang, b.voltage_ang)
    np.testing.assert_array_equal(a.max_mismatch, b.max_mismatch)


@pytest.mark.parametrize("precision", [0, 1])
def test_plan_forms_equal_case2000(gox, precision):
    fx = load_fixture("case2000")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    p, q = G.load_scenarios(g, 320, 0.15, 4242)
    r = _solve_forms(gox, yb, g.bus_type, (p, q, g.vm, g.va),
                     dict(tol=1e-8, max_iter=20, precision=precision))
    assert np.all(r[FORMS[0]].status == gox.GOX_CONVERGED)
    for f in FORMS[1:]:
        _same(r[FORMS[0]], r[f])


def test_plan_forms_equal_case10000_outages(gox):
    g = G.config_grid("case10000")
    yb = G.build_ybus(g)
    B = 64
    p = np.tile(g.p_spec, (B, 1))
    q = np.tile(g.q_spec, (B, 1))
    rng = np.random.default_rng(9)
    outage = G.outage_deltas(g, yb, rng.choice(np.flatnonzero(~G.bridges(g)), size=B))
    r = _solve_forms(gox, yb, g.bus_type, (p, q, g.vm, g.va),
                     dict(tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_MIXED, outage=outage))
    for f in FORMS[1:]:
        _same(r[FORMS[0]], r[f])


def test_wide_kernels_few_groups_big_grid(gox):
    """A grid of 12,000 buses with one group of scenarios (the serving
    case the wide kernels are for) gives the same bits both ways."""
    g = G.family_grid(12000, 77)
    yb = G.build_ybus(g)
    p, q = G.load_scenarios(g, 24, 0.15, 31)
    r = _solve_forms(gox, yb, g.bus_type, (p, q, g.vm, g.va),
                     dict(tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_MIXED))
    assert np.all(r[FORMS[0]].status == gox.GOX_CONVERGED)
    for f in FORMS[1:]:
        _same(r[FORMS[0]], r[f])
