"""The device refactor / substitution schedule (hazard-free update batches,
stage positions, dependency levels, fused forward substitution, backward
phases), run by its host FP64 mirror and compared with the oracle's KLU
refactor + solve -- no GPU needed.

Same-entry updates keep their order, so the refactor's rounding is KLU's;
the solution is compared at 1e-10 relative (the row-oriented substitution
sums in another order than KLU's column sweep)."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture


@pytest.mark.parametrize("progress_flags,wide", [(False, 0), (True, 0), (False, 16), (True, 16)])
@pytest.mark.parametrize("name", ["case118", "case2000", "case10000"])
def test_schedule_mirror_matches_oracle_lu(gox, oracle_mod, name, progress_flags, wide):
    """Both forms of the levels' synchronization, without and with the wide
    kernels' levels (run by the host mirror before and after the stream):
    with progress flags the host interpreter also checks, before the stream
    is accepted, that every conflicting pair of accesses by two warps is
    ordered by a flag wait and that every wait is for a level published
    earlier in level order."""
    from gridoxide_gb300 import solver as S
    O = oracle_mod
    if name == "case10000":
        g = G.config_grid(name)
        yb = G.build_ybus(g)
    else:
        fx = load_fixture(name)
        g = grid_from_fixture(fx)
        yb = ybus_from_fixture(fx)
    S.set_refactor_sync(progress_flags)
    S.set_refactor_wide(wide)
    try:
        topo = gox.Topology(yb, g.bus_type)
        assert topo.prepare(g.p_spec, g.q_spec, g.vm, g.va)
    finally:
        S.set_refactor_sync(False)
        S.set_refactor_wide(0)
    info = topo.info()
    assert info["rf32_progress_flags"] == int(progress_flags)
    if wide:
        assert info["rf32_wide_levels"] > 0
        assert name == "case118" or info["rf32_wide_phases"] > 0
    if progress_flags:
        assert 0 < info["rf32_flag_waits"] <= info["rf32_flag_warps_waited"]
    jac = O.Jacobian(yb, g.bus_type)
    st = topo.structure()
    Ap, Ai, _ = jac.csc_pattern()
    from gridoxide_gb300 import solver as S
    Pq, Qq, Rq = S.analyze(jac.n_u, Ap, Ai)
    p0, q0 = O.injections(yb, g.vm, g.va)
    v0 = jac.fill(g.vm, g.va, p0, q0)
    lu = O.LU(jac.n_u, jac.rows, jac.cols, v0, Pq, Qq, Rq)
    np.testing.assert_array_equal(lu.extract()["P"], st["P"])
    rng = np.random.default_rng(4)
    for _ in range(3):
        vm = g.vm.copy()
        pq = g.bus_type == G.BUS_PQ
        vm[pq] *= 1.0 + 0.02 * rng.standard_normal(pq.sum())
        va = 0.03 * rng.standard_normal(g.n_bus)
        va[0] = 0.0
        p, q = O.injections(yb, vm, va)
        vals = jac.fill(vm, va, p, q)
        rhs = rng.standard_normal(jac.n_u)
        x_ref = lu.factor_solve(vals, rhs)
        x = topo.emulate_step(vals, rhs)
        assert np.max(np.abs(x - x_ref)) <= 1e-10 * max(1.0, np.max(np.abs(x_ref)))
    assert info["levels"] > 0 and info["lu_slots"] == info["nnz_l"] + info["nnz_u"] + info["n_u"]
