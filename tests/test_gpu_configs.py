"""GPU parity on the workloads as the benchmark runs them.

* The 10,000-bus N-1 workload (one non-bridge branch out per scenario, warm
  start from the base case's solution): the FP64 path matches the oracle's
  iteration counts and status, |V| and theta within 1e-9 (the reference's
  KluNative path, src/solver.rs:639-736, restated by the oracle with the
  reference's own klu_analyze ordering); the mixed path converges and stays
  within 1e-7 pu of it (angles: 1e-7 of the grid's angle spread).
* The 2,000-bus x 4,096-scenario batch through the paths the benchmark
  times: the Newton loop as a captured CUDA graph (second solve of a
  configuration) and, for the mixed path, concurrent parts (two, four, five).  FP64
  matches the oracle as above; mixed converges, stays within 1e-7 of the
  oracle, and equals its first (unsplit, host-driven) solve bit for bit.
"""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G

pytestmark = pytest.mark.gpu

TOL_V = 1e-9
TOL_MIXED_V = 1e-7


def _oracle(O, yb, g, name):
    return O.Topology(yb, g.bus_type, *O.fixture_ordering(name, yb, g.bus_type))


def test_case10000_n1_warm_start_matches_oracle(gox, oracle_mod):
    O = oracle_mod
    g = G.config_grid("case10000")
    yb = G.build_ybus(g)
    ot = _oracle(O, yb, g, "case10000")
    base = ot.batch_solve(g.p_spec[None], g.q_spec[None], g.vm, g.va, tol=1e-8, max_iter=20)
    assert base["status"][0] == 0
    vm0, va0 = base["vm"][0], base["va"][0]
    B = 64
    p, q = G.load_scenarios(g, B, 0.15, 2025)
    rng = np.random.default_rng(2026)
    br = rng.choice(np.flatnonzero(~G.bridges(g)), size=B, replace=False)
    out = G.outage_deltas(g, yb, br)
    ref = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=16, outage=out)
    assert np.all(ref["status"] == 0)
    topo = gox.Topology(yb, g.bus_type)
    r64 = topo.solve(p, q, vm0, va0, tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_FP64,
                     outage=out)
    np.testing.assert_array_equal(r64.iterations, ref["iters"])
    np.testing.assert_array_equal(r64.status, ref["status"])
    assert np.max(np.abs(r64.voltage_mag - ref["vm"])) < TOL_V
    assert np.max(np.abs(r64.voltage_ang - ref["va"])) < TOL_V
    rmx = topo.solve(p, q, vm0, va0, tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_MIXED,
                     outage=out)
    assert np.all(rmx.status == 0) and np.all(rmx.max_mismatch < 1e-8)
    spread = float(np.ptp(ref["va"]))
    assert np.max(np.abs(rmx.voltage_mag - ref["vm"])) < TOL_MIXED_V
    assert np.max(np.abs(rmx.voltage_ang - ref["va"])) < TOL_MIXED_V * max(1.0, spread)


def test_case2000_full_batch_graph_and_split_match_oracle(gox, oracle_mod):
    O = oracle_mod
    g = G.config_grid("case2000")
    yb = G.build_ybus(g)
    B = 4096
    p, q = G.load_scenarios(g, B, 0.15, 2024)  # the benchmark's batch
    ref = _oracle(O, yb, g, "case2000").batch_solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20,
                                                      threads=16)
    assert np.all(ref["status"] == 0)
    topo = gox.Topology(yb, g.bus_type)
    solve = lambda prec: topo.solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, precision=prec)
    # FP64: the first solve fixes the pivot order (host-driven loop), the
    # second runs the captured graph
    first64 = solve(gox.GOX_PRECISION_FP64)
    n0 = topo.info()["graph_solves"]
    r64 = solve(gox.GOX_PRECISION_FP64)
    assert topo.info()["graph_solves"] == n0 + 1
    for r in (first64, r64):
        np.testing.assert_array_equal(r.iterations, ref["iters"])
        np.testing.assert_array_equal(r.status, ref["status"])
        assert np.max(np.abs(r.voltage_mag - ref["vm"])) < TOL_V
        assert np.max(np.abs(r.voltage_ang - ref["va"])) < TOL_V
    # mixed: with the pivot order fixed, 4,096 scenarios run as two
    # concurrent parts; the first mixed call captures its graphs, the next
    # ones run them
    rm = [solve(gox.GOX_PRECISION_MIXED) for _ in range(3)]
    # four staggered parts of 1,024 scenarios, then five uneven ones
    for parts in (4, 5):
        topo.set_split(parts)
        rm.append(solve(gox.GOX_PRECISION_MIXED))
    topo.set_split(1)
    topo.set_graph(False)
    plain = solve(gox.GOX_PRECISION_MIXED)
    for r in rm:
        assert np.all(r.status == 0) and np.all(r.max_mismatch < 1e-8)
        assert np.max(np.abs(r.voltage_mag - ref["vm"])) < TOL_MIXED_V
        assert np.max(np.abs(r.voltage_ang - ref["va"])) < TOL_MIXED_V
        np.testing.assert_array_equal(r.voltage_mag, plain.voltage_mag)
        np.testing.assert_array_equal(r.voltage_ang, plain.voltage_ang)
        np.testing.assert_array_equal(r.iterations, plain.iterations)
