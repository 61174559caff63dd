"""GPU: failure semantics, with every failure made on the host.

* A scenario that cannot converge (a load far beyond the grid's transfer
  capability) and one whose injections are not finite must not affect any
  other scenario of the batch -- the reference's
  divergent_scenario_does_not_poison_the_batch (tests/batch_solver_test.rs:
  153-183).  Both report a non-converged status; every other scenario,
  including the 31 other lanes of their groups, equals a batch without them
  bit for bit.
* A malformed command in the refactor's device stream (planted through the
  gox_topo_stream_word test hook) stops that warp: the kernel drains its
  copies, keeps the CTA's barriers (barrier plans) or makes the other warps'
  progress-flag waits give up (flag plans), and reports a device-wait
  error, so the solve returns GOX_E_DEVICE_WAIT promptly; with the word
  restored the next solve is correct again.  No wait is left to run out and
  nothing faults.
"""
import time

import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from gridoxide_gb300._lib import GoxError
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu


def _case118():
    fx = load_fixture("case118")
    return grid_from_fixture(fx), ybus_from_fixture(fx)


@pytest.mark.parametrize("precision", [0, 1])
def test_bad_scenarios_do_not_poison_the_batch(gox, precision):
    g, yb = _case118()
    B = 64
    p, q = G.load_scenarios(g, B, 0.15, 77)
    pq = np.flatnonzero(g.bus_type == G.BUS_PQ)
    bad_p, bad_q = p.copy(), q.copy()
    bad_p[5, pq[3]] = -1.0e6  # no solution exists
    bad_q[5, pq[3]] = -1.0e6
    bad_p[37, pq[10]] = np.nan  # not finite
    clean = gox.Topology(yb, g.bus_type).solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20,
                                                precision=precision)
    got = gox.Topology(yb, g.bus_type).solve(bad_p, bad_q, g.vm, g.va, tol=1e-8, max_iter=20,
                                              precision=precision)
    assert np.all(clean.status == gox.GOX_CONVERGED)
    assert got.status[5] != gox.GOX_CONVERGED and got.status[37] != gox.GOX_CONVERGED
    keep = np.setdiff1d(np.arange(B), [5, 37])
    np.testing.assert_array_equal(got.status[keep], clean.status[keep])
    np.testing.assert_array_equal(got.iterations[keep], clean.iterations[keep])
    np.testing.assert_array_equal(got.voltage_mag[keep], clean.voltage_mag[keep])
    np.testing.assert_array_equal(got.voltage_ang[keep], clean.voltage_ang[keep])
    np.testing.assert_array_equal(got.max_mismatch[keep], clean.max_mismatch[keep])


BAD_COMMAND = 15  # no command has this code


@pytest.mark.parametrize("progress_flags", [True, False])
@pytest.mark.parametrize("precision", [0, 1])
def test_malformed_stream_command_reports_device_wait(gox, precision, progress_flags):
    from gridoxide_gb300 import solver as S
    g, yb = _case118()
    p, q = G.load_scenarios(g, 96, 0.15, 78)
    # the default plan in either form (with progress flags, the other warps'
    # waits for the stopped warp give up at once instead of running out)
    S.set_autotune(False)
    S.set_refactor_sync(progress_flags)
    try:
        topo = gox.Topology(yb, g.bus_type)
        kw = dict(tol=1e-8, max_iter=20, precision=precision)
        good = topo.solve(p, q, g.vm, g.va, **kw)  # uploads the streams
    finally:
        S.set_autotune(True)
        S.set_refactor_sync(False)  # the default
    assert topo.info()["rf32_progress_flags"] == int(progress_flags)
    old = topo.stream_word(precision, 0, 0, BAD_COMMAND)
    try:
        t0 = time.perf_counter()
        with pytest.raises(GoxError) as ei:
            topo.solve(p, q, g.vm, g.va, **kw)
        assert ei.value.code == gox.GOX_E_DEVICE_WAIT
        assert time.perf_counter() - t0 < 10.0
    finally:
        assert topo.stream_word(precision, 0, 0, old) == BAD_COMMAND
    again = topo.solve(p, q, g.vm, g.va, **kw)
    np.testing.assert_array_equal(again.voltage_mag, good.voltage_mag)
    np.testing.assert_array_equal(again.iterations, good.iterations)
