"""gridoxide_gb300: GB300-native batched Newton-Raphson AC power flow.

The GPU engine lives in ``libgridoxide_gb300.so`` (C ABI:
``include/gridoxide_gb300.h``); this package is its Python face:

* :mod:`gridoxide_gb300.solver` -- LinearSolver / Topology / BatchSolver,
  mirroring the reference's plugin surface;
* :mod:`gridoxide_gb300.model` -- the reference's ``PowerFlowModel`` /
  ``BatchResult`` Python surface over the engine;
* :mod:`gridoxide_gb300.pgm` -- power-grid-model JSON to buses and Y-bus;
* :mod:`gridoxide_gb300.grids` -- seeded synthetic grids and the Y-bus;
* :mod:`gridoxide_gb300.build` -- in-tree build of the library (sm_103a).
"""
from . import build, grids, pgm, replicas  # noqa: F401
from ._lib import (GOX_CONVERGED, GOX_MAX_ITERATIONS, GOX_PRECISION_FP64,  # noqa: F401
                   GOX_E_DEVICE_WAIT, GOX_PRECISION_MIXED, GOX_SINGULAR_SCENARIO, GoxError)
from .solver import (BatchError, BatchResult, BatchSolver, Buses, BusOverride,  # noqa: F401
                     Gb300LinearSolver, JacobianBackend, PowerFlowReport, Scenario, Server,
                     SolveStatus, Topology, analyze, factor_host, multi_solve,
                     uniform_load_scaling)

from .model import PowerFlowModel  # noqa: F401,E402

__version__ = "0.1.0"
