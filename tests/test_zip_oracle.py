"""The oracle's ZIP terms of the effective injection (src/network.rs:600-611):
at a converged point the computed injections equal p_spec + j q_spec +
s_imp |V|^2 + s_cur |V| (an independent evaluation of the formula), and with
all ZIP terms zero the results equal the constant-power run bit for bit."""
import numpy as np

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture


def _zip_terms(g, seed):
    rng = np.random.default_rng(seed)
    pq = g.bus_type == G.BUS_PQ
    imp = np.zeros(g.n_bus, np.complex128)
    cur = np.zeros(g.n_bus, np.complex128)
    sel = pq & (rng.random(g.n_bus) < 0.3)
    imp[sel] = -(0.02 + 0.05 * rng.random(sel.sum())) * (1 + 0.3j)
    sel = pq & (rng.random(g.n_bus) < 0.3)
    cur[sel] = -(0.02 + 0.05 * rng.random(sel.sum())) * (1 + 0.2j)
    return imp, cur


def test_zip_residual_and_zero_terms(oracle_mod):
    O = oracle_mod
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    p, q = G.load_scenarios(g, 8, 0.1, 31)
    ot = oracle_topology(O, yb, g.bus_type, (fx["ref_P"], fx["ref_Q"], fx["ref_R"]))
    plain = ot.batch_solve(p, q, g.vm, g.va, tol=1e-10, max_iter=20)
    ot.set_zip(np.zeros(g.n_bus), np.zeros(g.n_bus))
    zero = ot.batch_solve(p, q, g.vm, g.va, tol=1e-10, max_iter=20)
    np.testing.assert_array_equal(plain["vm"], zero["vm"])
    np.testing.assert_array_equal(plain["va"], zero["va"])
    imp, cur = _zip_terms(g, 32)
    ot.set_zip(imp, cur)
    res = ot.batch_solve(p, q, g.vm, g.va, tol=1e-10, max_iter=20)
    assert np.all(res["status"] == 0)
    ns = g.bus_type != G.BUS_SLACK
    pqb = g.bus_type == G.BUS_PQ
    for s in range(p.shape[0]):
        vm, va = res["vm"][s], res["va"][s]
        pc, qc = O.injections(yb, vm, va)
        pe = p[s] + (imp.real * vm) * vm + cur.real * vm
        qe = q[s] + (imp.imag * vm) * vm + cur.imag * vm
        assert np.max(np.abs(pe[ns] - pc[ns])) < 1e-9
        assert np.max(np.abs(qe[pqb] - qc[pqb])) < 1e-9
    # the loads changed the solution
    assert np.max(np.abs(res["vm"] - plain["vm"])) > 1e-4
