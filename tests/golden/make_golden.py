"""Generates the committed golden fixtures (run where the reference tree is
mounted; the GPU tests only read the .npz files).

    python tests/golden/make_golden.py

For each workload grid it stores
  * the grid itself (bus and branch arrays) and its Y-bus,
  * the reference's symbolic ordering of the Jacobian (klu_analyze of the
    vendored SuiteSparse KLU, compiled by oracle/Makefile into oracle/_ref),
  * Newton-Raphson results for a few scenarios, computed by the oracle and
    cross-checked, bit for bit, against an NR loop whose linear solves are
    the reference's own compiled klu_factor / klu_refactor / klu_solve.
It also stores the reference's 3-bus network (tests/data/network.json of
the reference) as arrays.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from gridoxide_gb300 import grids as G  # noqa: E402
import oracle as O  # noqa: E402

REF_NETWORK = os.path.join(O.REF_ROOT, "tests", "data", "network.json")


def nr_with_ref_klu(yb, bus_type, jac, Ap, Ai, order, p_spec, q_spec, vm0, va0, tol, max_iter):
    """newton_raphson_cached (src/solver.rs:639-736) with the reference's
    compiled KLU as the LinearSolver (one persistent solver)."""
    vm, va = vm0.copy(), va0.copy()
    ns = np.flatnonzero(bus_type != G.BUS_SLACK)
    pq = np.flatnonzero(bus_type == G.BUS_PQ)
    hist = []
    klu = None
    for _ in range(max_iter):
        p, q = O.injections(yb, vm, va)
        F = np.concatenate([p_spec[ns] - p[ns], q_spec[pq] - q[pq]])
        m = 0.0
        for v in np.abs(F):
            m = max(m, v)
        hist.append(m)
        if m < tol:
            return vm, va, hist, 0
        vals = jac.fill(vm, va, p, q)
        if klu is None:
            klu = O.RefKLU(jac.n_u, Ap, Ai, vals[order])
        st, dx = klu.refactor_solve(vals[order], F)
        if st != 0 or not np.all(np.isfinite(dx)):
            return vm, va, hist, 2
        va[ns] += dx[:ns.size]
        vm[pq] += dx[ns.size:]
    return vm, va, hist, 1


def grid_fixture(name: str, n_scen: int, sigma: float, seed: int):
    g = G.config_grid(name)
    yb = G.build_ybus(g)
    jac = O.Jacobian(yb, g.bus_type)
    Ap, Ai, order = jac.csc_pattern()
    P, Q, R = O.ref_analyze(jac.n_u, Ap, Ai)
    p_s, q_s = G.load_scenarios(g, n_scen, sigma, seed)
    p_s[0], q_s[0] = g.p_spec, g.q_spec  # scenario 0 = base case
    topo = O.Topology(yb, g.bus_type, P, Q, R)
    res = topo.batch_solve(p_s, q_s, g.vm, g.va, tol=1e-8, max_iter=20, threads=1, history=True)
    for s in range(n_scen):
        vm, va, hist, st = nr_with_ref_klu(yb, g.bus_type, jac, Ap, Ai, order, p_s[s], q_s[s],
                                           g.vm, g.va, 1e-8, 20)
        it = res["iters"][s]
        assert st == res["status"][s] and len(hist) == it, (name, s)
        assert np.array_equal(vm, res["vm"][s]) and np.array_equal(va, res["va"][s]), (name, s)
        assert np.array_equal(np.array(hist), res["hist"][s][:it]), (name, s)
    out = dict(
        n_bus=g.n_bus, bus_type=g.bus_type, vm=g.vm, va=g.va, p_spec=g.p_spec, q_spec=g.q_spec,
        br_from=g.br_from, br_to=g.br_to, br_r=g.br_r, br_x=g.br_x, br_b=g.br_b,
        br_tap=g.br_tap, br_is_trafo=g.br_is_trafo, load_p=g.load_p, load_q=g.load_q,
        pv_weight=g.pv_weight,
        y_indptr=yb.indptr, y_indices=yb.indices, y_re=yb.re, y_im=yb.im,
        jac_rows=jac.rows, jac_cols=jac.cols,
        ref_P=P, ref_Q=Q, ref_R=R,
        scen_p=p_s, scen_q=q_s,
        nr_vm=res["vm"], nr_va=res["va"], nr_iters=res["iters"], nr_status=res["status"],
        nr_hist=res["hist"],
    )
    if name == "case118":
        p, q = O.injections(yb, g.vm, g.va)
        vals = jac.fill(g.vm, g.va, p, q)
        ex = O.RefKLU(jac.n_u, Ap, Ai, vals[order]).extract()
        out["jac_vals_flat"] = vals
        for k, v in ex.items():
            out["ref_factor_" + k] = v
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, "iters", res["iters"], "status", res["status"])


def ordering_fixture(name: str):
    """Only the reference's klu_analyze ordering of a grid too large to
    store whole, with a fingerprint of the pattern it belongs to."""
    g = G.config_grid(name)
    yb = G.build_ybus(g)
    jac = O.Jacobian(yb, g.bus_type)
    Ap, Ai, _ = jac.csc_pattern()
    P, Q, R = O.ref_analyze(jac.n_u, Ap, Ai)
    np.savez_compressed(os.path.join(HERE, f"{name}_order.npz"), ref_P=P, ref_Q=Q, ref_R=R,
                        pattern_sha256=O.pattern_fingerprint(yb, g.bus_type))
    print(name, "ordering: blocks", len(R) - 1)


def network3_fixture():
    with open(REF_NETWORK) as fh:
        net = json.load(fh)
    types = {"PQ": G.BUS_PQ, "PV": G.BUS_PV, "Slack": G.BUS_SLACK}
    buses = net["buses"]
    lines = net["lines"]
    np.savez_compressed(
        os.path.join(HERE, "network3.npz"),
        bus_type=np.array([types[b["bus_type"]] for b in buses], np.int32),
        vm=np.array([b["voltage_mag"] for b in buses]),
        va=np.array([b["voltage_ang"] for b in buses]),
        p_spec=np.array([b["p_spec"] for b in buses]),
        q_spec=np.array([b["q_spec"] for b in buses]),
        lines=np.array([[ln["from"], ln["to"], ln["r"], ln["x"], ln["b_shunt"]] for ln in lines]),
    )


if __name__ == "__main__":
    O.build(ref=True)
    network3_fixture()
    grid_fixture("case118", 8, 0.15, 101)
    grid_fixture("case2000", 4, 0.15, 102)
    ordering_fixture("case10000")
