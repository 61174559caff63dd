"""GPU parity: the CUDA batched Newton-Raphson path against the oracle.

FP64 path: same iteration counts and status as the oracle (the reference's
algorithm), |V| and theta within 1e-9 pu / 1e-9 rad.
Mixed path (FP32 refactor/solve, FP64 mismatch): every scenario converges
to max|F| < 1e-8 pu (its own FP64 mismatch), and its voltages stay within
1e-7 of the FP64 oracle's (both are 1e-8-pu solutions of the same system).
"""
import numpy as np
import pytest

from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture

pytestmark = pytest.mark.gpu

TOL_V = 1e-9
TOL_MIXED_V = 1e-7


def _run_both(gox, O, fx, p, q, precision, outage=None, threads=8):
    g = grid_from_fixture(fx)
    yb = ybus_from_fixture(fx)
    topo = gox.Topology(yb, g.bus_type)
    res = topo.solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, precision=precision,
                     outage=outage, history=True)
    ot = oracle_topology(O, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    ref = ot.batch_solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, threads=threads,
                         outage=outage, history=True)
    return topo, res, ref


@pytest.mark.parametrize("name", ["case118", "case2000"])
def test_fp64_matches_oracle_on_golden_scenarios(gox, oracle_mod, name):
    fx = load_fixture(name)
    topo, res, ref = _run_both(gox, oracle_mod, fx, fx["scen_p"], fx["scen_q"],
                               gox.GOX_PRECISION_FP64)
    # the oracle reproduces the committed golden vectors exactly
    np.testing.assert_array_equal(ref["vm"], fx["nr_vm"])
    np.testing.assert_array_equal(ref["iters"], fx["nr_iters"])
    np.testing.assert_array_equal(res.iterations, fx["nr_iters"])
    np.testing.assert_array_equal(res.status, fx["nr_status"])
    assert np.max(np.abs(res.voltage_mag - fx["nr_vm"])) < TOL_V
    assert np.max(np.abs(res.voltage_ang - fx["nr_va"])) < TOL_V
    # mismatch history: same length, same decades
    for s in range(len(res.iterations)):
        it = res.iterations[s]
        h, hr = res.history[s, :it], fx["nr_hist"][s, :it]
        assert np.all(np.abs(h - hr) <= 1e-9 + 1e-6 * np.abs(hr))


@pytest.mark.parametrize("name", ["case118", "case2000"])
def test_static_pivots_match_reference_ordering(gox, oracle_mod, name):
    fx = load_fixture(name)
    topo, res, ref = _run_both(gox, oracle_mod, fx, fx["scen_p"][:1], fx["scen_q"][:1],
                               gox.GOX_PRECISION_FP64)
    st = topo.structure()
    np.testing.assert_array_equal(st["Q"], fx["ref_Q"])
    np.testing.assert_array_equal(st["R"], fx["ref_R"])
    if "ref_factor_P" in fx:
        np.testing.assert_array_equal(st["P"], fx["ref_factor_P"])


@pytest.mark.parametrize("name,B", [("case118", 300), ("case2000", 96)])
def test_fp64_batch_matches_oracle(gox, oracle_mod, name, B):
    from gridoxide_gb300 import grids as G
    fx = load_fixture(name)
    g = grid_from_fixture(fx)
    p, q = G.load_scenarios(g, B, 0.15, 7)
    topo, res, ref = _run_both(gox, oracle_mod, fx, p, q, gox.GOX_PRECISION_FP64)
    np.testing.assert_array_equal(res.iterations, ref["iters"])
    np.testing.assert_array_equal(res.status, ref["status"])
    assert np.max(np.abs(res.voltage_mag - ref["vm"])) < TOL_V
    assert np.max(np.abs(res.voltage_ang - ref["va"])) < TOL_V


@pytest.mark.parametrize("name,B", [("case118", 300), ("case2000", 96)])
def test_mixed_converges_to_fp64_solution(gox, oracle_mod, name, B):
    from gridoxide_gb300 import grids as G
    fx = load_fixture(name)
    g = grid_from_fixture(fx)
    p, q = G.load_scenarios(g, B, 0.15, 8)
    topo, res, ref = _run_both(gox, oracle_mod, fx, p, q, gox.GOX_PRECISION_MIXED)
    assert np.all(res.status == gox.GOX_CONVERGED)
    assert np.all(res.max_mismatch < 1e-8)
    assert np.max(np.abs(res.voltage_mag - ref["vm"])) < TOL_MIXED_V
    assert np.max(np.abs(res.voltage_ang - ref["va"])) < TOL_MIXED_V


def test_masked_scenarios_are_frozen(gox, oracle_mod):
    """A scenario that converges early keeps its voltages bit for bit while
    the rest of its 32-lane group iterates (bde.rs:254-259 semantics)."""
    fx = load_fixture("case118")
    g = grid_from_fixture(fx)
    yb = ybus_from_fixture(fx)
    B = 40
    p = np.tile(g.p_spec, (B, 1))
    q = np.tile(g.q_spec, (B, 1))
    p[1::2] *= 1.3  # odd scenarios need more iterations
    q[1::2] *= 1.3
    topo = gox.Topology(yb, g.bus_type)
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64)
    alone = topo.solve(p[:1], q[:1], g.vm, g.va, precision=gox.GOX_PRECISION_FP64)
    for s in range(0, B, 2):
        np.testing.assert_array_equal(res.voltage_mag[s], alone.voltage_mag[0])
        np.testing.assert_array_equal(res.voltage_ang[s], alone.voltage_ang[0])


def test_linear_solver_dropin(gox, oracle_mod):
    """LinearSolver semantics (src/klu_native/mod.rs:219-241)."""
    S = gox.Gb300LinearSolver
    a = [(0, 0, 2.0), (0, 1, 1.0), (1, 0, 1.0), (1, 1, 3.0)]
    ls = S.new(2, a)
    x = ls.factor_and_solve(a, [5.0, 10.0])
    assert abs(x[0] - 1.0) < 1e-10 and abs(x[1] - 3.0) < 1e-10
    b = [(0, 0, 4.0), (0, 1, 1.0), (1, 0, 1.0), (1, 1, 2.0)]
    x2 = ls.factor_and_solve(b, [6.0, 5.0])
    assert abs(x2[0] - 1.0) < 1e-10 and abs(x2[1] - 2.0) < 1e-10
    assert S.new(2, [(0, 0, 1.0), (0, 1, 1.0), (1, 0, 2.0), (1, 1, 2.0)]) is None


def test_linear_solver_matches_oracle_on_jacobian(gox, oracle_mod):
    O = oracle_mod
    fx = load_fixture("case2000")
    g = grid_from_fixture(fx)
    yb = ybus_from_fixture(fx)
    jac = O.Jacobian(yb, g.bus_type)
    p, q = O.injections(yb, g.vm, g.va)
    vals = jac.fill(g.vm, g.va, p, q)
    ent = list(zip(jac.rows.tolist(), jac.cols.tolist(), vals.tolist()))
    ls = gox.Gb300LinearSolver.new(jac.n_u, ent)
    lu = O.LU(jac.n_u, jac.rows, jac.cols, vals, fx["ref_P"], fx["ref_Q"], fx["ref_R"])
    rng = np.random.default_rng(3)
    for _ in range(3):
        v2 = vals * (1 + 0.01 * rng.standard_normal(vals.size))
        rhs = rng.standard_normal(jac.n_u)
        x = ls.factor_and_solve_values(v2, rhs)
        xr = lu.factor_solve(v2, rhs)
        assert np.max(np.abs(x - xr)) <= 1e-10 * max(1.0, np.max(np.abs(xr)))
