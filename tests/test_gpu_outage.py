"""GPU: N-1 branch outages (the 10,000-bus workload's scenario kind), warm
start, and the mixed path's FP64 fallback.

An outage removes one non-bridge branch's series admittance and charging
from the Y-bus while keeping its pattern: a per-scenario delta on the
branch's four Y slots (the reference rejects outages,
src/batch.rs:207-209; the delta keeps the topology's factorization).
FP64 path: same iterations and status as the oracle, |V|, theta within
1e-9.  Mixed path: converges to max|F| < 1e-8 pu, within 1e-7 of the
oracle.  A scenario whose FP32 refactor meets a pivot below the threshold
times its column's largest L entry is solved again in FP64: with every
scenario sent there the mixed call must return the FP64 call's results
bit for bit.
"""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture

pytestmark = pytest.mark.gpu

TOL_V = 1e-9
TOL_MIXED_V = 1e-7


def _outages(g, yb, B, seed):
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(~G.bridges(g))
    br = rng.choice(cand, size=B, replace=True)
    return br, G.outage_deltas(g, yb, br)


def _fixture_grid(name):
    fx = load_fixture(name)
    return fx, grid_from_fixture(fx), ybus_from_fixture(fx)


@pytest.mark.parametrize("name,B", [("case118", 96), ("case2000", 64)])
def test_n1_fp64_matches_oracle(gox, oracle_mod, name, B):
    fx, g, yb = _fixture_grid(name)
    p, q = G.load_scenarios(g, B, 0.15, 11)
    _, out = _outages(g, yb, B, 12)
    topo = gox.Topology(yb, g.bus_type)
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64, outage=out)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ref = ot.batch_solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, threads=8, outage=out)
    np.testing.assert_array_equal(res.iterations, ref["iters"])
    np.testing.assert_array_equal(res.status, ref["status"])
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < TOL_V
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < TOL_V


def test_n1_mixed_warm_start_case2000(gox, oracle_mod):
    """Warm start from the base case's solution, one outage per scenario."""
    fx, g, yb = _fixture_grid("case2000")
    B = 64
    topo = gox.Topology(yb, g.bus_type)
    base = topo.solve(g.p_spec[None, :], g.q_spec[None, :], g.vm, g.va,
                      precision=gox.GOX_PRECISION_FP64)
    assert base.status[0] == gox.GOX_CONVERGED
    vm0, va0 = base.voltage_mag[0], base.voltage_ang[0]
    p, q = G.load_scenarios(g, B, 0.15, 13)
    _, out = _outages(g, yb, B, 14)
    res = topo.solve(p, q, vm0, va0, precision=gox.GOX_PRECISION_MIXED, outage=out)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ref = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=8, outage=out)
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    assert np.all(res.status[ok] == gox.GOX_CONVERGED)
    assert np.all(res.max_mismatch[ok] < 1e-8)
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < TOL_MIXED_V
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < TOL_MIXED_V


@pytest.mark.parametrize("name,B", [("case118", 80), ("case2000", 40)])
def test_fallback_every_scenario_equals_fp64(gox, name, B):
    _, g, yb = _fixture_grid(name)
    p, q = G.load_scenarios(g, B, 0.15, 15)
    _, out = _outages(g, yb, B, 16)
    topo = gox.Topology(yb, g.bus_type)
    fp64 = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64, outage=out,
                      history=True)
    topo.set_pivot_tolerance(1e300)  # every pivot trips: every scenario reruns in FP64
    mixed = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED, outage=out,
                       history=True)
    assert topo.last_fallbacks() == B
    # the re-solve factors every Newton step with partial pivoting: the FP64
    # path's results up to rounding, the same iterations and status
    np.testing.assert_array_equal(mixed.iterations, fp64.iterations)
    np.testing.assert_array_equal(mixed.status, fp64.status)
    assert np.max(np.abs(mixed.voltage_mag - fp64.voltage_mag)) < 1e-12
    assert np.max(np.abs(mixed.voltage_ang - fp64.voltage_ang)) < 1e-12
    it = fp64.iterations
    for s in range(B):
        h, hr = mixed.history[s, :it[s]], fp64.history[s, :it[s]]
        assert np.all(np.abs(h - hr) <= 1e-12 + 1e-6 * np.abs(hr))


def test_fallback_subset_keeps_other_scenarios(gox):
    """A threshold between the pivot ratios of two scenario families sends
    only some scenarios to the FP64 pivoting re-solve; the rest keep their
    mixed results (each result is bit for bit one of the two: scenarios are
    independent in both)."""
    _, g, yb = _fixture_grid("case118")
    B = 64
    p, q = G.load_scenarios(g, B, 0.15, 17)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_pivot_tolerance(0.0)
    plain = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    assert topo.last_fallbacks() == 0
    topo.set_pivot_tolerance(1e300)
    fp64 = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    assert topo.last_fallbacks() == B
    for tol in (1e-3, 1e-2, 1e-1, 0.5):
        topo.set_pivot_tolerance(tol)
        res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
        nf = topo.last_fallbacks()
        same64 = np.all(res.voltage_mag == fp64.voltage_mag, axis=1)
        same32 = np.all(res.voltage_mag == plain.voltage_mag, axis=1)
        assert np.all(same64 | same32)
        assert same64.sum() >= nf
        assert np.all(res.status == gox.GOX_CONVERGED)
    topo.set_pivot_tolerance(1e-6)


def test_n1_case10000_mixed_warm_start(gox, oracle_mod):
    """The 10,000-bus grid with one non-bridge outage per scenario, warm
    started from the base case, mixed precision.  The contract is the
    mismatch (< 1e-8 pu).  This grid's angles spread over ~38 rad along long
    chains and its Jacobian is ill-conditioned there, so two 1e-8-pu
    solutions differ in angle by ~1e-7 of that spread (5e-6 rad observed
    between the mixed path and the oracle): angles are bounded at 1e-6 of
    the spread, |V| at 1e-7."""
    g = G.config_grid("case10000")
    yb = G.build_ybus(g)
    B = 32
    topo = gox.Topology(yb, g.bus_type)
    base = topo.solve(g.p_spec[None, :], g.q_spec[None, :], g.vm, g.va,
                      precision=gox.GOX_PRECISION_FP64)
    assert base.status[0] == gox.GOX_CONVERGED
    vm0, va0 = base.voltage_mag[0], base.voltage_ang[0]
    p, q = G.load_scenarios(g, B, 0.15, 19)
    _, out = _outages(g, yb, B, 20)
    res = topo.solve(p, q, vm0, va0, precision=gox.GOX_PRECISION_MIXED, outage=out)
    ot = oracle_topology(oracle_mod, yb, g.bus_type)
    ref = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=8, outage=out)
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    assert np.all(res.status[ok] == gox.GOX_CONVERGED)
    assert np.all(res.max_mismatch[ok] < 1e-8)
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < TOL_MIXED_V
    spread = np.max(np.abs(ref["va"][ok]))
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < 1e-6 * max(1.0, spread)
