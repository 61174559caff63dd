"""GPU: PowerFlowModel (src/python.rs:99-478) end to end.

* `solve()` on every single-input power-grid-model fixture matches
  power-grid-model's node voltages within the reference test's tolerance;
* `initial_guess()` equals the oracle's linear guess within 1e-9;
* `solve_batch_scaled` (what scripts/bench/bench_batch.py times) over the
  11-node transmission case: FP64 runs equal the oracle's per scenario (same
  iterations, |V| and theta within 1e-9), results do not depend on `threads`,
  and the mixed backend converges to the same voltages within 1e-7;
* `solve_batch` overrides equal the same loads given through the scaled call.
"""
import os
import random

import numpy as np
import pytest

from gridoxide_gb300 import pgm
from helpers import GOLDEN, PGM_CASES, oracle_topology, pgm_oracle_start, pgm_runs, pgm_worst

pytestmark = pytest.mark.gpu

SINGLE = [c for c in sorted(PGM_CASES)
          if os.path.exists(os.path.join(GOLDEN, "pgm", c, "sym_output.json"))]


def _path(case):
    return os.path.join(GOLDEN, "pgm", case, "input.json")


@pytest.mark.parametrize("case", SINGLE)
def test_model_solve_matches_pgm(gox, oracle_mod, case):
    m = gox.PowerFlowModel.from_pgm_json(_path(case))
    m.solve()
    (doc, nodes), = pgm_runs(case)
    net = pgm.convert(doc)
    assert pgm_worst(net, np.array(m.voltage_mag()), np.array(m.voltage_ang()), nodes) < PGM_CASES[case]
    vm0, va0 = pgm_oracle_start(oracle_mod, net)
    gvm, gva = m.initial_guess()
    assert np.max(np.abs(np.array(gvm) - vm0)) < 1e-9
    assert np.max(np.abs(np.array(gva) - va0)) < 1e-9
    m.reset()
    m.solve()


def test_model_batch_scaled(gox, oracle_mod):
    O = oracle_mod
    path = _path("transmission-case")
    rng = random.Random(20260726)
    scales = [rng.uniform(0.8, 1.2) for _ in range(64)]
    m = gox.PowerFlowModel.from_pgm_json(path, backend="klu_native")
    out = m.solve_batch_scaled(scales, threads=1)
    again = m.solve_batch_scaled(scales, threads=8)
    assert all(r.converged for r in out)
    for a, b in zip(out, again):
        np.testing.assert_array_equal(a.voltage_mag, b.voltage_mag)
    net = pgm.convert(pgm.load(path))
    ot = oracle_topology(O, net.ybus, net.bus_type)
    for s, f in enumerate(scales):
        p, q = net.p_spec * f, net.q_spec * f
        vm0, va0 = O.linear_initial_guess(net.ybus, net.bus_type, p, q, net.vm, net.va)
        ref = ot.batch_solve(p[None], q[None], vm0, va0, tol=1e-6, max_iter=20)
        assert out[s].iterations == ref["iters"][0]
        assert out[s].max_mismatch < 1e-6
        assert np.max(np.abs(out[s].voltage_mag - ref["vm"][0])) < 1e-9
        assert np.max(np.abs(out[s].voltage_ang - ref["va"][0])) < 1e-9
    mixed = gox.PowerFlowModel.from_pgm_json(path, backend="gb300").solve_batch_scaled(scales)
    for a, b in zip(mixed, out):
        assert a.converged
        assert np.max(np.abs(a.voltage_mag - b.voltage_mag)) < 1e-7
    # the same loads as explicit overrides
    kinds, p0, q0 = m.bus_spec()
    sc = [[(i, p0[i] * f, q0[i] * f) for i in range(m.n_nodes) if p0[i] != 0.0 or q0[i] != 0.0]
          for f in scales[:8]]
    ov = m.solve_batch(sc)
    for a, b in zip(ov, out[:8]):
        np.testing.assert_array_equal(a.voltage_mag, b.voltage_mag)


def test_solve_scaled_equals_explicit(gox):
    """gox_batch_solve_scaled (scenarios expanded on the device) gives the
    results of gox_batch_solve on the same scaled arrays, bit for bit."""
    from gridoxide_gb300 import grids as G
    from helpers import grid_from_fixture, load_fixture, ybus_from_fixture
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    f = np.random.default_rng(5).uniform(0.8, 1.2, 200)
    for prec in (gox.GOX_PRECISION_FP64, gox.GOX_PRECISION_MIXED):
        topo = gox.Topology(yb, g.bus_type)
        a = topo.solve_scaled(f, g.p_spec, g.q_spec, g.vm, g.va, precision=prec, history=True)
        b = topo.solve(g.p_spec[None] * f[:, None], g.q_spec[None] * f[:, None], g.vm, g.va,
                       precision=prec, history=True)
        for x, y in ((a.voltage_mag, b.voltage_mag), (a.voltage_ang, b.voltage_ang),
                     (a.iterations, b.iterations), (a.status, b.status), (a.history, b.history)):
            np.testing.assert_array_equal(x, y)
        assert np.all(a.status == gox.GOX_CONVERGED)
