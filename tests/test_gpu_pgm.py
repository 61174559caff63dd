"""GPU: power-grid-model inputs end to end.  Every symmetric fixture the
reference tests (tests/klu_native_jacobian_test.rs:26-126,
tests/pgm_three_winding_transformer_test.rs) is converted on the host
(gridoxide_gb300.pgm), registered as a topology with its ZIP terms, started
from the GPU's linear initial guess and solved with tol 1e-6 / 20 iterations:

* FP64: the node voltages match power-grid-model's within the reference
  test's tolerance, and the oracle's run from its own linear guess (same
  iterations and status, |V| and theta within 1e-9);
* mixed precision: converged, and within the same power-grid-model tolerance.
"""
import numpy as np
import pytest

from gridoxide_gb300 import pgm
from helpers import PGM_CASES, oracle_topology, pgm_oracle_start, pgm_runs, pgm_worst

pytestmark = pytest.mark.gpu

TOL_V = 1e-9


@pytest.mark.parametrize("case", sorted(PGM_CASES))
def test_pgm_case_gpu(gox, oracle_mod, case):
    O = oracle_mod
    for doc, nodes in pgm_runs(case):
        net = pgm.convert(doc)
        res = pgm.solve(gox, net, precision=gox.GOX_PRECISION_FP64)
        assert res.status[0] == gox.GOX_CONVERGED
        assert pgm_worst(net, res.voltage_mag[0], res.voltage_ang[0], nodes) < PGM_CASES[case]
        vm0, va0 = pgm_oracle_start(O, net)
        ot = oracle_topology(O, net.ybus, net.bus_type)
        ot.set_zip(net.zip_imp, net.zip_cur)
        ref = ot.batch_solve(net.p_spec[None], net.q_spec[None], vm0, va0, tol=1e-6, max_iter=20)
        assert res.iterations[0] == ref["iters"][0]
        assert np.max(np.abs(res.voltage_mag[0] - ref["vm"][0])) < TOL_V
        assert np.max(np.abs(res.voltage_ang[0] - ref["va"][0])) < TOL_V
        mixed = pgm.solve(gox, net, precision=gox.GOX_PRECISION_MIXED)
        assert mixed.status[0] == gox.GOX_CONVERGED
        assert pgm_worst(net, mixed.voltage_mag[0], mixed.voltage_ang[0], nodes) < PGM_CASES[case]
