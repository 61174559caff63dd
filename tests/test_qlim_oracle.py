"""The oracle's Q-limit loop pinned against the reference's own test
(tests/q_limits_test.rs): the 3-bus slack/PV/PQ network with bus 1's q_min
tightened to -0.25 switches bus 1 to PQ at Q = -0.25 and lands on the
reference's voltages; with q_min = -0.5 nothing switches and the voltages
are the unconstrained ones."""
import numpy as np

from gridoxide_gb300 import grids as G
from helpers import load_fixture, oracle_qlim


def _network3():
    fx = load_fixture("network3")
    lines = [(int(a), int(b), r, x, bb) for a, b, r, x, bb in [tuple(r) for r in fx["lines"]]]
    return fx, G.ybus_from_lines(3, lines)


def test_qlim_switches_pv_to_pq(oracle_mod):
    O = oracle_mod
    fx, yb = _network3()
    vm0, va0 = O.linear_initial_guess(yb, fx["bus_type"], fx["p_spec"], fx["q_spec"], fx["vm"], fx["va"])
    q_min = np.array([-999.0, -0.25, -999.0])
    q_max = np.array([999.0, 0.5, 999.0])
    r, sw, stab = oracle_qlim(O, yb, fx["bus_type"], fx["p_spec"], fx["q_spec"], vm0, va0, q_min,
                              q_max, 1e-6, 20, 10)
    assert r["status"][0] == 0 and sw == [1] and stab
    vm, va = r["vm"][0], r["va"][0]
    pc, qc = O.injections(yb, vm, va)
    assert abs(pc[1] - 0.5) < 1e-6 and abs(qc[1] + 0.25) < 1e-6
    for i, (m, a) in {1: (1.043469, 0.013207), 2: (1.005454, -0.043577)}.items():
        assert abs(vm[i] - m) < 1e-5 and abs(va[i] - a) < 1e-5


def test_qlim_no_violation_matches_unconstrained(oracle_mod):
    O = oracle_mod
    fx, yb = _network3()
    vm0, va0 = O.linear_initial_guess(yb, fx["bus_type"], fx["p_spec"], fx["q_spec"], fx["vm"], fx["va"])
    r, sw, stab = oracle_qlim(O, yb, fx["bus_type"], fx["p_spec"], fx["q_spec"], vm0, va0,
                              np.array([-999.0, -0.5, -999.0]), np.array([999.0, 0.5, 999.0]),
                              1e-6, 20, 10)
    assert sw == [] and stab
    vm, va = r["vm"][0], r["va"][0]
    for i, (m, a) in {1: (1.04, 0.014349), 2: (1.003358, -0.043141)}.items():
        assert abs(vm[i] - m) < 1e-5 and abs(va[i] - a) < 1e-5
