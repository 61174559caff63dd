"""GPU: ZIP terms of the effective injection (src/network.rs:600-611) in
every mismatch, not differentiated in the Jacobian (src/jacobian.rs:224-243),
as the reference's inexact Newton does.  FP64 path: same iterations and
status as the oracle with the same terms, |V| and theta within 1e-9; mixed
path: converges to max|F| < 1e-8 pu (F with the ZIP terms), within 1e-7 of
the oracle; and with the linear initial guess, whose load admittance uses
the effective injection at the start |V|."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture
from test_zip_oracle import _zip_terms

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,B", [("case118", 64), ("case2000", 40)])
def test_zip_fp64_and_mixed_match_oracle(gox, oracle_mod, name, B):
    fx = load_fixture(name)
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    p, q = G.load_scenarios(g, B, 0.1, 33)
    imp, cur = _zip_terms(g, 34)
    if name == "case2000":  # the scaled-down loads of this grid: smaller terms
        imp, cur = 0.1 * imp, 0.1 * cur
    topo = gox.Topology(yb, g.bus_type)
    topo.set_zip(imp, cur)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ot.set_zip(imp, cur)
    ref = ot.batch_solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, threads=8)
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64)
    np.testing.assert_array_equal(res.iterations, ref["iters"])
    np.testing.assert_array_equal(res.status, ref["status"])
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < 1e-9
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < 1e-9
    mix = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED)
    assert np.all(mix.status[ok] == gox.GOX_CONVERGED)
    assert np.all(mix.max_mismatch[ok] < 1e-8)
    assert np.max(np.abs(mix.voltage_mag[ok] - ref["vm"][ok])) < 1e-7
    assert np.max(np.abs(mix.voltage_ang[ok] - ref["va"][ok])) < 1e-7
    # clearing the terms returns to constant power
    topo.set_zip()
    plain = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64)
    assert np.max(np.abs(plain.voltage_mag[ok] - res.voltage_mag[ok])) > 1e-6


def test_zip_with_linear_guess(gox, oracle_mod):
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 32
    p, q = G.load_scenarios(g, B, 0.1, 35)
    imp, cur = _zip_terms(g, 36)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_zip(imp, cur)
    topo.set_initial_guess("linear")
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64)
    vm0 = np.zeros_like(p)
    va0 = np.zeros_like(p)
    for s in range(B):
        vm0[s], va0[s] = oracle_mod.linear_initial_guess(yb, g.bus_type, p[s], q[s], g.vm, g.va,
                                                         imp, cur)
    ot = oracle_topology(oracle_mod, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ot.set_zip(imp, cur)
    ref = ot.batch_solve(p, q, vm0, va0, tol=1e-8, max_iter=20, threads=8)
    ok = ref["status"] == gox.GOX_CONVERGED
    assert ok.sum() > B // 2
    np.testing.assert_array_equal(res.iterations, ref["iters"])
    assert np.max(np.abs(res.voltage_mag[ok] - ref["vm"][ok])) < 1e-9
    assert np.max(np.abs(res.voltage_ang[ok] - ref["va"][ok])) < 1e-9
