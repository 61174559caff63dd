"""GPU: the mixed path's repair of a poor static pivot order.

A scenario whose FP32 refactor meets a pivot below the pivot-ratio threshold
is solved again in FP64, each Newton step factoring its Jacobian afresh
with threshold partial pivoting on the GPU (KLU's lpivot, tol 0.001 with
diagonal preference: src/klu_native/kernel.rs:187-262, factor_block
:341-416).

* One Jacobian whose static pivot order meets a pivot 1e-12 times its
  column (the first factor column's pivot entry scaled down on the host):
  the GPU's pivoting solve equals the oracle's fresh klu_factor + solve of
  that Jacobian within 1e-9 (relative to the solution), while the static
  order's pivot ratio is below 1e-6.
* Whole batches with every scenario sent to the pivoting re-solve (a
  threshold above 1): every report equals the oracle's FP64 result --
  iterations, status, |V| and theta within 1e-9."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture

pytestmark = pytest.mark.gpu


def test_pivot_solve_repairs_a_tiny_static_pivot(gox, oracle_mod):
    O = oracle_mod
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    topo = gox.Topology(yb, g.bus_type)
    assert topo.prepare(g.p_spec[None], g.q_spec[None], g.vm, g.va)
    st = topo.structure()
    jac = O.Jacobian(yb, g.bus_type)
    p0, q0 = O.injections(yb, g.vm, g.va)
    J0 = jac.fill(g.vm, g.va, p0, q0)
    rng = np.random.default_rng(9)
    vm = g.vm * (1.0 + 0.01 * rng.standard_normal(g.n_bus))
    va = g.va + 0.02 * rng.standard_normal(g.n_bus)
    pc, qc = O.injections(yb, vm, va)
    J1 = jac.fill(vm, va, pc, qc)
    # the static pivot of the first factor column (no update reaches it):
    # the entry at (Pnum[0], Q[0]), made 1e-12 times the column's largest
    e = int(np.flatnonzero((jac.rows == st["P"][0]) & (jac.cols == st["Q"][0]))[0])
    col = np.abs(J1[jac.cols == st["Q"][0]])
    J1[e] = 1e-12 * col.max()
    # the static order on these values: its pivot ratio is tiny
    static = O.LU(jac.n_u, jac.rows, jac.cols, J0, fx["ref_P"], fx["ref_Q"], fx["ref_R"])
    assert static.refactor(J1) == 0
    ex = static.extract()
    u00 = ex["Ux"][ex["Up"][1] - 1]
    lmax = np.max(np.abs(ex["Lx"][ex["Lp"][0] + 1:ex["Lp"][1]] * u00))
    assert abs(u00) < 1e-6 * max(abs(u00), lmax)
    # a fresh factorization with partial pivoting of J1 (the oracle's KLU)
    fresh = O.LU(jac.n_u, jac.rows, jac.cols, J1, fx["ref_P"], fx["ref_Q"], fx["ref_R"])
    rhs = rng.standard_normal(jac.n_u)
    x_ref = fresh.factor_solve(J1, rhs)
    dx = topo.pivot_solve(J1, rhs)
    assert dx is not None and x_ref is not None
    scale = float(np.max(np.abs(x_ref)))
    assert np.max(np.abs(dx - x_ref)) <= 1e-9 * scale
    # and it solves the system
    import scipy.sparse as sp
    A = sp.csr_matrix((J1, (jac.rows, jac.cols)), shape=(jac.n_u, jac.n_u))
    assert np.max(np.abs(A @ dx - rhs)) <= 1e-9 * max(1.0, float(np.max(np.abs(rhs))))


@pytest.mark.parametrize("name", ["case118", "case2000"])
def test_every_flagged_scenario_resolved_with_pivoting_matches_oracle(gox, oracle_mod, name):
    fx = load_fixture(name)
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    B = 64
    p, q = G.load_scenarios(g, B, 0.15, 404)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_pivot_tolerance(2.0)  # |u_kk| < 2 max(|u_kk|, |l_ik|): every scenario trips
    res = topo.solve(p, q, g.vm, g.va, tol=1e-8, max_iter=20, precision=gox.GOX_PRECISION_MIXED)
    assert topo.last_fallbacks() == B
    ref = oracle_topology(oracle_mod, yb, g.bus_type).batch_solve(p, q, g.vm, g.va, tol=1e-8,
                                                                  max_iter=20, threads=16)
    np.testing.assert_array_equal(res.status, ref["status"])
    np.testing.assert_array_equal(res.iterations, ref["iters"])
    assert np.max(np.abs(res.voltage_mag - ref["vm"])) < 1e-9
    assert np.max(np.abs(res.voltage_ang - ref["va"])) < 1e-9
