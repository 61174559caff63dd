"""The LinearSolver refactor + solve without device allocation.

Some callers cannot allocate device memory when they solve: a process
whose device memory another allocator's pool already holds (cudaMalloc
would fail or take memory the pool counted on), or a control loop with a
deadline per Newton step (cudaMalloc and cudaFree synchronize the device
and take unbounded time).  For them
gox_ls_factor_solve_values_static keeps its scratch in a fixed array inside
the library.  Its results must equal gox_ls_factor_solve_values' on the same
handle, call after call (the array keeps the previous call's contents, so
two different systems are solved back to back).  This file is collected
last so that a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

from gridoxide_gb300 import _lib
from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10  # the tolerance of the other LinearSolver tests


def _jacobian(O, name, seed):
    fx = load_fixture(name)
    g = grid_from_fixture(fx)
    yb = ybus_from_fixture(fx)
    jac = O.Jacobian(yb, g.bus_type)
    rng = np.random.default_rng(seed)
    vm = g.vm.copy()
    pq = g.bus_type == G.BUS_PQ
    vm[pq] *= 1.0 + 0.01 * rng.standard_normal(pq.sum())
    va = 0.02 * rng.standard_normal(g.n_bus)
    va[0] = 0.0
    p, q = O.injections(yb, vm, va)
    return jac, jac.fill(vm, va, p, q), rng


@pytest.mark.parametrize("name", ["case118", "case2000"])
def test_static_variant_matches_allocating_call_twice(gox, oracle_mod, name):
    jac, vals, rng = _jacobian(oracle_mod, name, 5)
    ent = list(zip(jac.rows.tolist(), jac.cols.tolist(), vals.tolist()))
    ls = gox.Gb300LinearSolver.new(jac.n_u, ent)
    for call in range(2):
        v = vals * (1.0 + 0.02 * rng.standard_normal(vals.size))
        rhs = rng.standard_normal(jac.n_u)
        x_static = ls.factor_and_solve_values_static(v, rhs)
        x_ref = ls.factor_and_solve_values(v, rhs)
        assert x_static is not None and x_ref is not None, call
        scale = max(1.0, float(np.max(np.abs(x_ref))))
        assert np.max(np.abs(x_static - x_ref)) <= REL_TOL * scale, call


def test_static_variant_reports_singular_and_too_large(gox):
    ls = gox.Gb300LinearSolver.new(2, [(0, 0, 2.0), (0, 1, 1.0), (1, 0, 1.0), (1, 1, 3.0)])
    x = ls.factor_and_solve_values_static([2.0, 1.0, 1.0, 3.0], [5.0, 10.0])
    assert abs(x[0] - 1.0) < 1e-12 and abs(x[1] - 3.0) < 1e-12
    assert ls.factor_and_solve_values_static([1.0, 1.0, 2.0, 2.0], [1.0, 1.0]) is None
    n = 300_000  # 300k factor entries x 32 lanes x 8 B > the fixed array
    big = gox.Gb300LinearSolver.new(n, [(i, i, 1.0 + i % 7) for i in range(n)])
    L = _lib.load()
    xs = np.zeros(n)
    rc = L.gox_ls_factor_solve_values_static(
        big._h, np.ones(n).ctypes.data_as(_lib.f64p), np.ones(n).ctypes.data_as(_lib.f64p),
        xs.ctypes.data_as(_lib.f64p))
    assert rc == _lib.GOX_E_TOO_LARGE
