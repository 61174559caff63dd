"""PGM conversion (gridoxide_gb300.pgm, after src/pgm.rs:347-595 and the
Y-bus stamping of src/network.rs) pinned against power-grid-model's own
results: every symmetric fixture the reference tests, converted, started from
the linear initial guess and solved by the oracle's Newton-Raphson with
tol 1e-6 / 20 iterations, matches the expected node voltages within the
reference test's tolerance (tests/klu_native_jacobian_test.rs:26-126,
tests/pgm_three_winding_transformer_test.rs)."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from gridoxide_gb300 import pgm
from helpers import PGM_CASES, oracle_topology, pgm_oracle_start, pgm_runs, pgm_worst


@pytest.mark.parametrize("case", sorted(PGM_CASES))
def test_pgm_case_oracle(oracle_mod, case):
    O = oracle_mod
    for doc, nodes in pgm_runs(case):
        net = pgm.convert(doc)
        vm0, va0 = pgm_oracle_start(O, net)
        ot = oracle_topology(O, net.ybus, net.bus_type)
        ot.set_zip(net.zip_imp, net.zip_cur)
        r = ot.batch_solve(net.p_spec[None], net.q_spec[None], vm0, va0, tol=1e-6, max_iter=20)
        assert r["status"][0] == 0
        assert pgm_worst(net, r["vm"][0], r["va"][0], nodes) < PGM_CASES[case]


def test_pgm_conversion_pieces():
    """Source impedance, island marking and the bus layout of a converted input."""
    r, x = pgm.source_impedance_pu(1e10, 0.1, 1e6)
    assert abs(np.hypot(r, x) - 1e-4) < 1e-18 and abs(r / x - 0.1) < 1e-15
    (doc, _), = pgm_runs("basic-node")
    net = pgm.convert(doc)
    # node_1 (PQ), node_2 (no source: a slack at V = 0), the source's slack bus
    assert list(net.bus_type) == [G.BUS_PQ, G.BUS_SLACK, G.BUS_SLACK]
    assert net.vm[1] == 0.0 and net.vm[2] == doc["data"]["source"][0]["u_ref"]
    (doc, _), = pgm_runs("three_winding_transformer")[:1]
    net = pgm.convert(doc)
    n_nodes = len(doc["data"]["node"])
    assert net.n_bus == n_nodes + 1 + len(doc["data"]["source"])
    star = n_nodes
    assert net.bus_type[star] == G.BUS_PQ
    # the star bus connects to the three windings' nodes only
    cols = set(net.ybus.indices[net.ybus.indptr[star]:net.ybus.indptr[star + 1]])
    assert cols == {star} | {net.id_to_idx[int(doc["data"]["three_winding_transformer"][0][k])]
                             for k in ("node_1", "node_2", "node_3")}


def test_from_grid_round_trip(oracle_mod):
    """A generated grid written as a PGM document and converted back: the
    same Y-bus between the grid's buses (to rounding; the slack bus's
    diagonal gains the source admittance), injections, PV set-points and bus
    types, one extra slack bus for the source; and it solves."""
    g = G.config_grid("case118")
    net = pgm.convert(pgm.from_grid(g))
    n = g.n_bus
    assert net.n_bus == n + 1 and net.bus_type[n] == G.BUS_SLACK and net.vm[n] == g.vm[0]
    a = G.build_ybus(g).dense()
    b = net.ybus.dense()[:n, :n]
    d = np.abs(a - b)
    z_s = complex(*pgm.source_impedance_pu(1e10, 0.1, pgm.S_BASE_VA))
    assert abs(d[0, 0] - abs(1.0 / z_s)) < 1e-6 * abs(1.0 / z_s)
    d[0, 0] = 0.0
    assert d.max() < 1e-14 * np.abs(a).max()
    expect_type = np.where(g.bus_type == G.BUS_SLACK, G.BUS_PQ, g.bus_type)
    np.testing.assert_array_equal(net.bus_type[:n], expect_type)
    ns = g.bus_type != G.BUS_SLACK
    pq = g.bus_type == G.BUS_PQ
    assert np.max(np.abs(net.p_spec[:n][ns] - g.p_spec[ns])) < 1e-15
    assert np.max(np.abs(net.q_spec[:n][pq] - g.q_spec[pq])) < 1e-15
    np.testing.assert_array_equal(net.vm[:n][g.bus_type == G.BUS_PV], g.vm[g.bus_type == G.BUS_PV])
    ot = oracle_topology(oracle_mod, net.ybus, net.bus_type)
    r = ot.batch_solve(net.p_spec[None], net.q_spec[None], net.vm, net.va, tol=1e-8, max_iter=20)
    assert r["status"][0] == 0


def test_voltage_regulator_limits():
    """A voltage regulator's q_min / q_max become the PV bus's reactive limits
    in per unit (src/pgm.rs:431-441); NaN or absent means none."""
    g = G.config_grid("case118")
    doc = pgm.from_grid(g)
    regs = doc["data"]["voltage_regulator"]
    regs[0]["q_min"], regs[0]["q_max"] = -5e6, 7e6
    regs[1]["q_min"], regs[1]["q_max"] = float("nan"), 2e6
    net = pgm.convert(doc)
    gen_node = {x["id"]: x["node"] for x in doc["data"]["sym_gen"]}
    k0 = net.id_to_idx[gen_node[regs[0]["regulated_object"]]]
    k1 = net.id_to_idx[gen_node[regs[1]["regulated_object"]]]
    assert (net.q_min[k0], net.q_max[k0]) == (-5.0, 7.0)
    assert net.q_min[k1] == -np.inf and net.q_max[k1] == 2.0
    assert np.isfinite(net.q_min).sum() == 1 and np.isfinite(net.q_max).sum() == 2
