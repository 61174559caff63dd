"""GPU: the Jacobian fill (K2) and the refactor (K3) checked entry by entry.

The reference pins its Jacobian bit for bit against a naive assembly
(src/jacobian.rs:297-368) and its factor against dense LU fixtures
(src/klu_native/kernel.rs:606-812, refactor.rs:223-301).  Here the device
path's own values are read back (gox_topo_factor_values: one injection,
fill and refactor of the batch kernels at given voltages) and compared with
the oracle's Jacobian.fill and with the oracle's KLU refactor + klu_extract
of the same Jacobian, on case118 at 40 perturbed operating points.

Errors are measured against the largest entry of the same column.  FP64:
the Jacobian within 1e-13 (the device sums the injections in another
order), every L and U entry within 1e-10.  Mixed: the FP32 Jacobian within
1e-5, the FP32 factor within 2e-4."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu


def _setup(gox, O, B=40, seed=3):
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    topo = gox.Topology(yb, g.bus_type)
    # the pivot order: the first factorization of the base case at its start
    assert topo.prepare(g.p_spec[None], g.q_spec[None], g.vm, g.va)
    jac = O.Jacobian(yb, g.bus_type)
    Ap, Ai, order = jac.csc_pattern()
    p0, q0 = O.injections(yb, g.vm, g.va)
    lu = O.LU(jac.n_u, jac.rows, jac.cols, jac.fill(g.vm, g.va, p0, q0), fx["ref_P"], fx["ref_Q"],
              fx["ref_R"])
    rng = np.random.default_rng(seed)
    vm = np.tile(g.vm, (B, 1))
    va = np.tile(g.va, (B, 1))
    pq = g.bus_type == G.BUS_PQ
    vm[:, pq] *= 1.0 + 0.02 * rng.standard_normal((B, int(pq.sum())))
    va[:, 1:] += 0.05 * rng.standard_normal((B, g.n_bus - 1))
    p, q = G.load_scenarios(g, B, 0.15, seed)
    return topo, jac, lu, g, yb, p, q, vm, va


def _entries_dev(st, lu_row):
    """{(row, col): value} of the device factor in its slot layout."""
    n = len(st["Lp"]) - 1
    out, base = {}, 0
    for k in range(n):
        ul = st["Up"][k + 1] - st["Up"][k]
        ll = st["Lp"][k + 1] - st["Lp"][k]
        for p_ in range(ul):
            out[(int(st["Ui"][st["Up"][k] + p_]), k)] = lu_row[base + p_]
        out[(k, k)] = lu_row[base + ul]
        for t in range(ll):
            out[("L", int(st["Li"][st["Lp"][k] + t]), k)] = lu_row[base + ul + 1 + t]
        base += ul + 1 + ll
    return out


def _entries_oracle(ex):
    """The same keys from klu_extract's layout (L columns open with the unit
    diagonal, U columns close with the pivot)."""
    n = len(ex["Lp"]) - 1
    out = {}
    for k in range(n):
        for j in range(ex["Lp"][k] + 1, ex["Lp"][k + 1]):
            out[("L", int(ex["Li"][j]), k)] = ex["Lx"][j]
        for j in range(ex["Up"][k], ex["Up"][k + 1]):
            out[(int(ex["Ui"][j]), k)] = ex["Ux"][j]
    return out


def _col_scale(ref):
    sc = {}
    for key, v in ref.items():
        c = key[-1]
        sc[c] = max(sc.get(c, 0.0), abs(v))
    return sc


@pytest.mark.parametrize("precision", [0, 1])
def test_fill_and_factor_match_the_oracle_entry_by_entry(gox, oracle_mod, precision):
    O = oracle_mod
    topo, jac, lu, g, yb, p, q, vm, va = _setup(gox, O)
    jd, ld = topo.factor_values(p, q, vm, va, precision=precision)
    st = topo.structure()
    fp64 = precision == gox.GOX_PRECISION_FP64
    worst_j = worst_lu = 0.0
    for s in range(p.shape[0]):
        pc, qc = O.injections(yb, vm[s], va[s])
        J = jac.fill(vm[s], va[s], pc, qc)
        # against the largest entry of the same Jacobian column (the
        # rectangular form's differences of products cancel where angles
        # are close, so small entries carry the column's rounding)
        cmax = np.zeros(jac.n_u)
        np.maximum.at(cmax, jac.cols, np.abs(J))
        worst_j = max(worst_j, float(np.max(np.abs(jd[s] - J) / cmax[jac.cols])))
        assert lu.refactor(J) == 0
        ex = lu.extract()
        if s == 0:
            np.testing.assert_array_equal(ex["P"], st["P"])
        ref = _entries_oracle(ex)
        dev = _entries_dev(st, ld[s])
        assert set(ref) == set(dev), "factor patterns differ"
        sc = _col_scale(ref)
        for key, v in ref.items():
            worst_lu = max(worst_lu, abs(dev[key] - v) / sc[key[-1]])
    if fp64:
        assert worst_j < 1e-13, worst_j
        assert worst_lu < 1e-10, worst_lu
    else:
        assert worst_j < 1e-5, worst_j
        assert worst_lu < 2e-4, worst_lu
