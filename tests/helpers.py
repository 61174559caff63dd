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


def oracle_topology(O, yb, bus_type, ordering=None):
    """Oracle topology.  The symbolic ordering is an input of the oracle;
    by default it is taken from the library's klu_analyze, whose output the
    CPU tests pin bit for bit against the reference's compiled KLU."""
    if ordering is None:
        from gridoxide_gb300 import solver as S
        jac = O.Jacobian(yb, bus_type)
        Ap, Ai, _ = jac.csc_pattern()
        ordering = S.analyze(jac.n_u, Ap, Ai)
    P, Q, R = ordering
    return O.Topology(yb, bus_type, P, Q, R)
