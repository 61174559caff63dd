"""GPU: the linear initial guess (src/network.rs:627-678), which the
reference's BatchSolver runs before every scenario (src/batch.rs:268).

The GPU computes it for the whole batch (FP64 refactor of the guess system's
real 2x2-block form with a fixed pivot order); the oracle restates it with
a complex sparse LU (scipy's splu standing in for faer).  Both start points
agree to rounding, so the Newton runs from them must agree like any two FP64
runs: same iterations and status, |V| and theta within 1e-9.  The 3-bus
snapshot the reference's own tests solve this way (tol 1e-6, linear guess:
powerflow_test.rs:17-31) pins the whole path.
"""
import dataclasses

import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture

pytestmark = pytest.mark.gpu

TOL_V = 1e-9


def _oracle_starts(O, yb, bus_type, p, q, vm, va, outage=None):
    vm0 = np.zeros_like(p)
    va0 = np.zeros_like(p)
    for s in range(p.shape[0]):
        y = yb
        if outage is not None and outage[0][s][0] >= 0:
            re, im = yb.re.copy(), yb.im.copy()
            for c in range(4):
                re[outage[0][s][c]] += outage[1][s][c]
                im[outage[0][s][c]] += outage[2][s][c]
            y = dataclasses.replace(yb, re=re, im=im)
        vm0[s], va0[s] = O.linear_initial_guess(y, bus_type, p[s], q[s], vm, va)
    return vm0, va0


def test_network3_snapshot_linear_guess(gox, oracle_mod):
    fx = load_fixture("network3")
    lines = [(int(a), int(b), r, x, bb) for a, b, r, x, bb in [tuple(r) for r in fx["lines"]]]
    yb = G.ybus_from_lines(3, lines)
    topo = gox.Topology(yb, fx["bus_type"])
    topo.set_initial_guess("linear")
    res = topo.solve(fx["p_spec"][None], fx["q_spec"][None], fx["vm"], fx["va"], tol=1e-6,
                     precision=gox.GOX_PRECISION_FP64)
    expected = [(1.06, 0.0), (1.04, 0.014349), (1.003358, -0.043141)]
    assert res.status[0] == gox.GOX_CONVERGED
    for i, (vm, va) in enumerate(expected):
        assert abs(res.voltage_mag[0][i] - vm) < 1e-5
        assert abs(res.voltage_ang[0][i] - va) < 1e-5
    vm0, va0 = _oracle_starts(oracle_mod, yb, fx["bus_type"], fx["p_spec"][None], fx["q_spec"][None],
                              fx["vm"], fx["va"])
    ot = oracle_topology(oracle_mod, yb, fx["bus_type"])
    ref = ot.batch_solve(fx["p_spec"][None], fx["q_spec"][None], vm0, va0, tol=1e-6, max_iter=20)
    assert res.iterations[0] == ref["iters"][0]


@pytest.mark.parametrize("name,B,outages", [("case118", 64, False), ("case2000", 40, False),
                                            ("case118", 48, True)])
def test_linear_guess_fp64_matches_oracle(gox, oracle_mod, name, B, outages):
    fx = load_fixture(name)
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    p, q = G.load_scenarios(g, B, 0.15, 21)
    out = None
    if outages:
        rng = np.random.default_rng(22)
        br = rng.choice(np.flatnonzero(~G.bridges(g)), size=B, replace=True)
        out = G.outage_deltas(g, yb, br)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_initial_guess("linear")
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64, outage=out)
    vm0, va0 = _oracle_starts(oracle_mod, yb, g.bus_type, p, q, g.vm, g.va, out)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ref = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=8, outage=out)
    np.testing.assert_array_equal(res.iterations, ref["iters"])
    np.testing.assert_array_equal(res.status, ref["status"])
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < TOL_V
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < TOL_V


def test_linear_guess_mixed_case2000(gox, oracle_mod):
    fx = load_fixture("case2000")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 64
    p, q = G.load_scenarios(g, B, 0.15, 23)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_initial_guess("linear")
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    vm0, va0 = _oracle_starts(oracle_mod, yb, g.bus_type, p, q, g.vm, g.va)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ref = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=8)
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    assert np.all(res.status[ok] == gox.GOX_CONVERGED)
    assert np.all(res.max_mismatch[ok] < 1e-8)
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < 1e-7
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < 1e-7
    # the given start is still the default, and switching back restores it
    topo.set_initial_guess("given")
    flat = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    assert np.all(flat.status[ok] == gox.GOX_CONVERGED)


def test_linear_guess_large_batch(gox, oracle_mod):
    """A batch whose scenarios x buses exceed the capped launch grid of the
    start-point kernels (4,864 blocks x 256 threads): every scenario gets
    its own guess and converges."""
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 12000
    assert B * g.n_bus > 4864 * 256
    p, q = G.load_scenarios(g, B, 0.15, 29)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_initial_guess("linear")
    gvm, gva = topo.initial_guess(p, q, g.vm, g.va)
    for s in (0, B // 2, B - 1):
        vm0, va0 = oracle_mod.linear_initial_guess(yb, g.bus_type, p[s], q[s], g.vm, g.va)
        assert np.max(np.abs(gvm[s] - vm0)) < 1e-12
        assert np.max(np.abs(gva[s] - va0)) < 1e-12
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    assert np.all(res.status == gox.GOX_CONVERGED)
    ref = topo.solve(p[-32:], q[-32:], g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    np.testing.assert_array_equal(res.iterations[-32:], ref.iterations)
