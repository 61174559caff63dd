"""Test helpers: fixture loading and oracle runs (oracle = test infrastructure)."""
from __future__ import annotations

import os

import numpy as np

from gridoxide_gb300 import grids as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def grid_from_fixture(fx: dict) -> G.Grid:
    return G.Grid(n_bus=int(fx["n_bus"]), bus_type=fx["bus_type"], vm=fx["vm"], va=fx["va"],
                  p_spec=fx["p_spec"], q_spec=fx["q_spec"], br_from=fx["br_from"],
                  br_to=fx["br_to"], br_r=fx["br_r"], br_x=fx["br_x"], br_b=fx["br_b"],
                  br_tap=fx["br_tap"], br_is_trafo=fx["br_is_trafo"], load_p=fx["load_p"],
                  load_q=fx["load_q"], pv_weight=fx["pv_weight"])


def ybus_from_fixture(fx: dict) -> G.YBus:
    return G.YBus(n=int(fx["n_bus"]), indptr=fx["y_indptr"], indices=fx["y_indices"],
                  re=fx["y_re"], im=fx["y_im"])


def reference_ordering(O, yb, bus_type):
    """The reference's compiled klu_analyze ordering of one of the workload
    grids (committed fixture), or None for other grids."""
    for name in ("case118", "case2000", "case10000"):
        try:
            return O.fixture_ordering(name, yb, bus_type)
        except ValueError:
            continue
    return None


def oracle_topology(O, yb, bus_type, ordering=None):
    """Oracle topology.  The symbolic ordering is an input of the oracle: the
    reference's own (a committed fixture) for the workload grids, else the
    library's klu_analyze, whose output the CPU tests pin bit for bit
    against the reference's compiled KLU."""
    if ordering is None:
        ordering = reference_ordering(O, yb, bus_type)
    if ordering is None:
        from gridoxide_gb300 import solver as S
        jac = O.Jacobian(yb, bus_type)
        Ap, Ai, _ = jac.csc_pattern()
        ordering = S.analyze(jac.n_u, Ap, Ai)
    P, Q, R = ordering
    return O.Topology(yb, bus_type, P, Q, R)


# power-grid-model fixtures (tests/golden/pgm/<case>, copied from the
# reference's tests/data/pgm/powerflow/symmetric by make_pgm_fixtures.py) and
# the tolerances the reference's own tests give them
# (tests/klu_native_jacobian_test.rs, tests/pgm_three_winding_transformer_test.rs)
PGM_CASES = {"basic-node": 1e-5, "node": 1e-5, "line": 1e-5, "shunt": 1e-5, "sym_load": 1e-5,
             "sym_gen": 1e-5, "source": 1e-5, "transmission-case": 1e-5, "transformer": 1e-4,
             "distribution-case": 1e-5, "three_winding_transformer": 1e-4}


def pgm_runs(case: str):
    """[(input document, expected node outputs)] of one case: the single input,
    or every scenario of the update batch merged into the base input."""
    from gridoxide_gb300 import pgm
    d = os.path.join(GOLDEN, "pgm", case)
    base = pgm.load(os.path.join(d, "input.json"))
    if os.path.exists(os.path.join(d, "sym_output.json")):
        return [(base, pgm.load(os.path.join(d, "sym_output.json"))["data"]["node"])]
    upd = pgm.load(os.path.join(d, "update_batch.json"))["data"]
    exp = pgm.load(os.path.join(d, "sym_output_batch.json"))["data"]
    return [(pgm.apply_batch_scenario(base, u), e["node"]) for u, e in zip(upd, exp)]


def pgm_worst(net, vm, va, nodes) -> float:
    """Largest |u_pu - vm| or |u_angle - va| over the expected nodes."""
    worst = 0.0
    for nd in nodes:
        k = net.id_to_idx[int(nd["id"])]
        worst = max(worst, abs(vm[k] - nd["u_pu"]), abs(va[k] - nd["u_angle"]))
    return worst


def pgm_oracle_start(O, net):
    """The oracle's start point for a converted network: its linear guess,
    or the given voltages where the reference's guess would be singular."""
    if net.guess_singular:
        return net.vm.copy(), net.va.copy()
    return O.linear_initial_guess(net.ybus, net.bus_type, net.p_spec, net.q_spec, net.vm, net.va,
                                  net.zip_imp, net.zip_cur)


def oracle_qlim(O, yb, bus_type, p, q, vm0, va0, q_min, q_max, tol, max_iter, max_outer):
    """newton_raphson_enforcing_q_limits_with_stats (src/solver.rs:569-618)
    for one scenario on the oracle: solve; stop unless converged; switch
    every PV bus whose computed Q (src/network.rs power_injections) leaves
    [q_min, q_max] to PQ with Q pinned at the limit; solve again from the
    converged state with a fresh pivot order (PersistentSolver::reset);
    repeat until nothing switches or max_outer solves ran.  Returns
    (report dict of the last solve, switched buses, stabilized)."""
    types = np.array(bus_type, np.int32).copy()
    q = np.array(q, np.float64).copy()
    vm, va = np.array(vm0, np.float64), np.array(va0, np.float64)
    switches = []
    r = None
    for _ in range(max_outer):
        ot = oracle_topology(O, yb, types)
        r = ot.batch_solve(np.asarray(p)[None], q[None], vm, va, tol=tol, max_iter=max_iter)
        vm, va = r["vm"][0], r["va"][0]
        if r["status"][0] != 0:
            return r, switches, True
        _, qc = O.injections(yb, vm, va)
        switched = False
        for b in range(len(types)):
            if types[b] != G.BUS_PV:
                continue
            if qc[b] < q_min[b]:
                types[b], q[b] = G.BUS_PQ, q_min[b]
            elif qc[b] > q_max[b]:
                types[b], q[b] = G.BUS_PQ, q_max[b]
            else:
                continue
            switches.append(b)
            switched = True
        if not switched:
            return r, switches, True
    return r, switches, False
