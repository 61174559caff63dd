"""Pins the oracle (CPU restatement of the reference path) against the
reference's own known answers and its compiled C.

* 3-bus snapshot of tests/data/network.json (powerflow_test.rs:17-31,
  persistent_solver_test.rs:33-37): V = (1.06, 0), (1.04, 0.014349),
  (1.003358, -0.043141) within 1e-5.
* Jacobian pattern and values equal, bit for bit, to an independent
  restatement of the reference's naive `build_jacobian_triplets`
  (src/solver.rs:815-888) at the 4 operating points of jacobian.rs:297-368.
* KLU factorization equal, bit for bit, to the reference's compiled
  klu_factor/klu_extract (golden fixture), and NR results equal to the
  committed golden vectors (made with the reference's KLU in the loop).
* BatchSolver semantics (tests/batch_solver_test.rs): thread-count
  invariance, divergent scenarios isolated, empty batch.
"""
import math

import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture


def _ordering_for(O, yb, bus_type):
    from gridoxide_gb300 import solver as S
    jac = O.Jacobian(yb, bus_type)
    Ap, Ai, _ = jac.csc_pattern()
    return S.analyze(jac.n_u, Ap, Ai)


def test_network3_snapshot(oracle_mod):
    O = oracle_mod
    fx = load_fixture("network3")
    lines = [tuple(r) for r in fx["lines"]]
    lines = [(int(a), int(b), r, x, bb) for a, b, r, x, bb in lines]
    yb = G.ybus_from_lines(3, lines)
    topo = oracle_topology(O, yb, fx["bus_type"], _ordering_for(O, yb, fx["bus_type"]))
    res = topo.batch_solve(fx["p_spec"][None], fx["q_spec"][None], fx["vm"], fx["va"], tol=1e-6,
                           max_iter=20)
    expected = [(1.06, 0.0), (1.04, 0.014349), (1.003358, -0.043141)]
    assert res["status"][0] == 0
    for i, (vm, va) in enumerate(expected):
        assert abs(res["vm"][0][i] - vm) < 1e-5
        assert abs(res["va"][0][i] - va) < 1e-5


def test_network3_snapshot_linear_guess(oracle_mod):
    """The reference's own setup for the snapshot: the linear initial guess
    (src/network.rs:627-678) before NR, tol 1e-6."""
    O = oracle_mod
    fx = load_fixture("network3")
    lines = [(int(a), int(b), r, x, bb) for a, b, r, x, bb in [tuple(r) for r in fx["lines"]]]
    yb = G.ybus_from_lines(3, lines)
    vm0, va0 = O.linear_initial_guess(yb, fx["bus_type"], fx["p_spec"], fx["q_spec"], fx["vm"], fx["va"])
    assert vm0[0] == fx["vm"][0] and vm0[1] == fx["vm"][1]  # slack and PV keep their voltage
    topo = oracle_topology(O, yb, fx["bus_type"], _ordering_for(O, yb, fx["bus_type"]))
    res = topo.batch_solve(fx["p_spec"][None], fx["q_spec"][None], vm0[None], va0[None], tol=1e-6,
                           max_iter=20)
    expected = [(1.06, 0.0), (1.04, 0.014349), (1.003358, -0.043141)]
    assert res["status"][0] == 0
    for i, (vm, va) in enumerate(expected):
        assert abs(res["vm"][0][i] - vm) < 1e-5
        assert abs(res["va"][0][i] - va) < 1e-5


def _mixed_network():
    """jacobian.rs:300-333: bus 0 Slack, bus 1 PV, buses 2-4 PQ."""
    bus_type = np.array([G.BUS_SLACK, G.BUS_PV, G.BUS_PQ, G.BUS_PQ, G.BUS_PQ], np.int32)
    vm = np.array([1.06, 1.04, 1.0, 1.0, 1.0])
    lines = [(0, 1, 0.02, 0.06, 0.03), (0, 2, 0.08, 0.24, 0.025), (1, 2, 0.06, 0.18, 0.02),
             (1, 3, 0.06, 0.18, 0.02), (2, 4, 0.04, 0.12, 0.015), (3, 4, 0.01, 0.03, 0.01)]
    return bus_type, vm, G.ybus_from_lines(5, lines)


def _naive_jacobian(bus_type, yb, vm, va, p, q):
    """Independent restatement of build_jacobian_triplets (src/solver.rs:815-888)."""
    n = len(bus_type)
    ns = [i for i in range(n) if bus_type[i] != G.BUS_SLACK]
    pq = [i for i in range(n) if bus_type[i] == G.BUS_PQ]
    nsp = {b: k for k, b in enumerate(ns)}
    pqp = {b: k for k, b in enumerate(pq)}
    na = len(ns)
    out = []

    def row(i):
        s, e = yb.indptr[i], yb.indptr[i + 1]
        return [(int(yb.indices[t]), float(yb.re[t]), float(yb.im[t])) for t in range(s, e)]

    for r, i in enumerate(ns):
        for k, g, b in row(i):
            if k == i:
                out.append((r, r, -q[i] - (vm[i] * vm[i]) * b))
                if i in pqp:
                    out.append((r, na + pqp[i], p[i] / vm[i] + vm[i] * g))
                continue
            ang = va[i] - va[k]
            if k in nsp:
                out.append((r, nsp[k], vm[i] * vm[k] * (g * math.sin(ang) - b * math.cos(ang))))
            if k in pqp:
                out.append((r, na + pqp[k], vm[i] * (g * math.cos(ang) + b * math.sin(ang))))
    for r, i in enumerate(pq):
        for k, g, b in row(i):
            if k == i:
                out.append((na + r, nsp[i], p[i] - (vm[i] * vm[i]) * g))
                out.append((na + r, na + r, q[i] / vm[i] - vm[i] * b))
                continue
            ang = va[i] - va[k]
            if k in nsp:
                out.append((na + r, nsp[k], -vm[i] * vm[k] * (g * math.cos(ang) + b * math.sin(ang))))
            if k in pqp:
                out.append((na + r, na + pqp[k], vm[i] * (g * math.sin(ang) - b * math.cos(ang))))
    return out


def test_jacobian_bit_exact_at_four_operating_points(oracle_mod):
    O = oracle_mod
    bus_type, vm0, yb = _mixed_network()
    jac = O.Jacobian(yb, bus_type)
    for step in range(4):
        va = np.array([-0.01 * (step * (j + 1)) for j in range(5)])
        vm = vm0.copy()
        for j in range(5):
            if bus_type[j] == G.BUS_PQ:
                vm[j] = 1.0 - 0.013 * step * (j + 1)
        p, q = O.injections(yb, vm, va)
        vals = jac.fill(vm, va, p, q)
        exp = _naive_jacobian(bus_type, yb, vm.tolist(), va.tolist(), p.tolist(), q.tolist())
        assert len(exp) == jac.nnz
        for e, (r, c, v) in enumerate(exp):
            assert (jac.rows[e], jac.cols[e]) == (r, c)
            assert np.float64(vals[e]).tobytes() == np.float64(v).tobytes(), (step, e)


def test_jacobian_pattern_network3(oracle_mod):
    O = oracle_mod
    fx = load_fixture("network3")
    lines = [(int(a), int(b), r, x, bb) for a, b, r, x, bb in fx["lines"]]
    yb = G.ybus_from_lines(3, lines)
    jac = O.Jacobian(yb, fx["bus_type"])
    p, q = O.injections(yb, fx["vm"], fx["va"])
    vals = jac.fill(fx["vm"], fx["va"], p, q)
    exp = _naive_jacobian(fx["bus_type"], yb, fx["vm"].tolist(), fx["va"].tolist(), p.tolist(),
                          q.tolist())
    assert [(r, c) for r, c, _ in exp] == list(zip(jac.rows.tolist(), jac.cols.tolist()))
    assert all(np.float64(v).tobytes() == np.float64(x).tobytes() for (_, _, v), x in zip(exp, vals))


@pytest.mark.parametrize("name", ["case118", "case2000"])
def test_oracle_ybus_matches_generator(oracle_mod, name):
    fx = load_fixture(name)
    g = grid_from_fixture(fx)
    rp, ci, yr, yi = oracle_mod.ybus_build(g)
    yb = G.build_ybus(g)
    np.testing.assert_array_equal(rp, yb.indptr)
    np.testing.assert_array_equal(ci, yb.indices)
    assert yr.tobytes() == yb.re.tobytes() and yi.tobytes() == yb.im.tobytes()
    np.testing.assert_array_equal(yb.indptr, fx["y_indptr"])
    assert yb.re.tobytes() == fx["y_re"].tobytes()


def test_oracle_factor_equals_reference_klu(oracle_mod):
    O = oracle_mod
    fx = load_fixture("case118")
    yb = ybus_from_fixture(fx)
    jac = O.Jacobian(yb, fx["bus_type"])
    lu = O.LU(jac.n_u, jac.rows, jac.cols, fx["jac_vals_flat"], fx["ref_P"], fx["ref_Q"],
              fx["ref_R"])
    ex = lu.extract()
    for k in ("Lp", "Li", "Lx", "Up", "Ui", "Ux", "P", "Q", "R"):
        assert ex[k].tobytes() == fx["ref_factor_" + k].tobytes(), k


@pytest.mark.parametrize("name", ["case118", "case2000"])
def test_oracle_reproduces_golden_nr(oracle_mod, name):
    O = oracle_mod
    fx = load_fixture(name)
    g = grid_from_fixture(fx)
    topo = oracle_topology(O, ybus_from_fixture(fx), g.bus_type,
                           (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    res = topo.batch_solve(fx["scen_p"], fx["scen_q"], g.vm, g.va, tol=1e-8, max_iter=20,
                           history=True)
    assert res["vm"].tobytes() == fx["nr_vm"].tobytes()
    assert res["va"].tobytes() == fx["nr_va"].tobytes()
    np.testing.assert_array_equal(res["iters"], fx["nr_iters"])
    np.testing.assert_array_equal(res["status"], fx["nr_status"])


def test_batch_thread_invariance_and_isolation(oracle_mod):
    O = oracle_mod
    fx = load_fixture("case118")
    g = grid_from_fixture(fx)
    topo = oracle_topology(O, ybus_from_fixture(fx), g.bus_type,
                           (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    p, q = G.load_scenarios(g, 32, 0.15, 5)
    p[7] *= 40.0  # a divergent scenario (batch_solver_test.rs:153-183)
    q[7] *= 40.0
    a = topo.batch_solve(p, q, g.vm, g.va, threads=1, history=True)
    b = topo.batch_solve(p, q, g.vm, g.va, threads=8, history=True)
    assert a["vm"].tobytes() == b["vm"].tobytes()
    np.testing.assert_array_equal(a["iters"], b["iters"])
    assert a["status"][7] != 0
    keep = [s for s in range(32) if s != 7]
    c = topo.batch_solve(p[keep], q[keep], g.vm, g.va, threads=3)
    assert c["vm"].tobytes() == a["vm"][keep].tobytes()
    empty = topo.batch_solve(np.zeros((0, g.n_bus)), np.zeros((0, g.n_bus)), g.vm, g.va)
    assert empty["vm"].shape == (0, g.n_bus)
