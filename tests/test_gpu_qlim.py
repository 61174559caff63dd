"""GPU: reactive-power limits (gox_batch_solve_qlim, after
newton_raphson_enforcing_q_limits, src/solver.rs:545-618).

* the reference's 3-bus test (tests/q_limits_test.rs): bus 1 switches to PQ
  at Q = -0.25 and lands on the reference's voltages;
* case118, 48 scenarios, limits on six PV buses at quantiles of their
  unconstrained Q, so each scenario switches its own subset: per scenario the same switched
  buses, stabilized flag, status and iterations as the oracle's loop (FP64),
  |V| and theta within 1e-9; the mixed path switches the same buses and
  converges to within 1e-7 of it;
* max_outer = 1: no re-solve, the switching scenarios report stabilized =
  false with the unconstrained solve's voltages.
"""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import (grid_from_fixture, load_fixture, oracle_qlim, oracle_topology,
                     ybus_from_fixture)

pytestmark = pytest.mark.gpu


def test_qlim_network3(gox, oracle_mod):
    fx = load_fixture("network3")
    lines = [(int(a), int(b), r, x, bb) for a, b, r, x, bb in [tuple(r) for r in fx["lines"]]]
    yb = G.ybus_from_lines(3, lines)
    topo = gox.Topology(yb, fx["bus_type"])
    topo.set_initial_guess("linear")
    q_min = np.array([-999.0, -0.25, -999.0])
    q_max = np.array([999.0, 0.5, 999.0])
    res, sw, stab = topo.solve_qlim(fx["p_spec"][None], fx["q_spec"][None], fx["vm"], fx["va"],
                                    q_min, q_max, tol=1e-6, precision=gox.GOX_PRECISION_FP64)
    assert res.status[0] == gox.GOX_CONVERGED and stab[0]
    assert sw[0].tolist() == [False, True, False]
    vm, va = res.voltage_mag[0], res.voltage_ang[0]
    for i, (m, a) in {1: (1.043469, 0.013207), 2: (1.005454, -0.043577)}.items():
        assert abs(vm[i] - m) < 1e-5 and abs(va[i] - a) < 1e-5
    _, qc = oracle_mod.injections(yb, vm, va)
    assert abs(qc[1] + 0.25) < 1e-6


def _case118_limits(oracle_mod):
    """Limits on six PV buses at the 20 % (floor, the three lowest-Q buses)
    and 80 % (ceiling, the three highest) quantiles of their unconstrained Q
    over 48 load scenarios, so each scenario trips its own subset."""
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    p, q = G.load_scenarios(g, 48, 0.1, 77)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    base = ot.batch_solve(p, q, g.vm, g.va, tol=1e-10, max_iter=20, threads=8)
    qs = np.array([oracle_mod.injections(yb, base["vm"][s], base["va"][s])[1] for s in range(48)])
    pv = np.flatnonzero(g.bus_type == G.BUS_PV)
    order = pv[np.argsort(np.median(qs[:, pv], axis=0))]
    q_min = np.full(g.n_bus, -np.inf)
    q_max = np.full(g.n_bus, np.inf)
    q_min[order[:3]] = np.quantile(qs[:, order[:3]], 0.2, axis=0)
    q_max[order[-3:]] = np.quantile(qs[:, order[-3:]], 0.8, axis=0)
    return g, yb, q_min, q_max


def test_qlim_case118_matches_oracle(gox, oracle_mod):
    g, yb, q_min, q_max = _case118_limits(oracle_mod)
    B = 48
    p, q = G.load_scenarios(g, B, 0.1, 77)
    topo = gox.Topology(yb, g.bus_type)
    res, sw, stab = topo.solve_qlim(p, q, g.vm, g.va, q_min, q_max, tol=1e-8, max_iter=20,
                                    max_outer=10, precision=gox.GOX_PRECISION_FP64)
    n_groups = len({tuple(np.flatnonzero(r)) for r in sw})
    assert n_groups >= 4 and sw.any(axis=1).sum() > B // 4
    for s in range(B):
        ref, rsw, rstab = oracle_qlim(oracle_mod, yb, g.bus_type, p[s], q[s], g.vm, g.va, q_min,
                                      q_max, 1e-8, 20, 10)
        assert sorted(rsw) == np.flatnonzero(sw[s]).tolist()
        assert rstab == stab[s]
        assert res.status[s] == ref["status"][0]
        assert res.iterations[s] == ref["iters"][0]
        assert np.max(np.abs(res.voltage_mag[s] - ref["vm"][0])) < 1e-9
        assert np.max(np.abs(res.voltage_ang[s] - ref["va"][0])) < 1e-9
    mixed, msw, mstab = gox.Topology(yb, g.bus_type).solve_qlim(
        p, q, g.vm, g.va, q_min, q_max, tol=1e-8, max_iter=20, max_outer=10,
        precision=gox.GOX_PRECISION_MIXED)
    np.testing.assert_array_equal(msw, sw)
    assert np.all(mixed.status == gox.GOX_CONVERGED) and np.all(mstab)
    assert np.max(np.abs(mixed.voltage_mag - res.voltage_mag)) < 1e-7


def test_qlim_outer_budget(gox, oracle_mod):
    g, yb, q_min, q_max = _case118_limits(oracle_mod)
    p, q = G.load_scenarios(g, 32, 0.1, 78)
    topo = gox.Topology(yb, g.bus_type)
    res, sw, stab = topo.solve_qlim(p, q, g.vm, g.va, q_min, q_max, max_outer=1,
                                    precision=gox.GOX_PRECISION_FP64)
    plain = gox.Topology(yb, g.bus_type).solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64)
    hit = sw.any(axis=1)
    assert hit.any() and not hit.all()
    np.testing.assert_array_equal(stab, ~hit)
    np.testing.assert_array_equal(res.voltage_mag, plain.voltage_mag)
    np.testing.assert_array_equal(res.iterations, plain.iterations)
