"""The reference's Python model surface over the GPU engine.

`PowerFlowModel` and `BatchResult` follow the reference's PyO3 classes of the
same names (src/python.rs:63-478): a model loaded from a power-grid-model
JSON file, solved once (`solve`) or as a batch of injection scenarios
(`solve_batch`, `solve_batch_scaled`, the call the reference's
scripts/bench/bench_batch.py times), plus the inspection methods its oracle
scripts use (`ybus_triplets`, `bus_spec`, `initial_guess`,
`zip_term_counts`).  Every numeric call runs on the GPU through
libgridoxide_gb300 (linear initial guess, then batched Newton-Raphson).

Backends: the reference's names ("scalar", "block", "klu", "klu_native",
"pardiso") select the FP64 GPU path, the arithmetic they share; "gb300"
selects the mixed path (FP32 refactor and solves, FP64 mismatch and update,
FP64 fallback per scenario) and "gb300_fp64" the FP64 path by name.
"""
from __future__ import annotations

import copy
import os
from dataclasses import dataclass

import numpy as np

from . import grids as G
from . import pgm
from ._lib import GOX_CONVERGED, GOX_MAX_ITERATIONS, GOX_PRECISION_FP64, GOX_PRECISION_MIXED
from .solver import Topology

_BACKENDS = {"scalar": GOX_PRECISION_FP64, "block": GOX_PRECISION_FP64, "klu": GOX_PRECISION_FP64,
             "klu_native": GOX_PRECISION_FP64, "pardiso": GOX_PRECISION_FP64,
             "gb300_fp64": GOX_PRECISION_FP64, "gb300": GOX_PRECISION_MIXED}


@dataclass
class BatchResult:
    """python.rs:63-78: one scenario of a batch."""

    voltage_mag: np.ndarray
    voltage_ang: np.ndarray
    iterations: int
    converged: bool
    max_mismatch: float


class PowerFlowModel:
    """python.rs:99-478 with the GPU engine as its solver."""

    def __init__(self, net: pgm.Network, backend: str = "scalar", tol: float = 1e-6,
                 max_iter: int = 20):
        if backend not in _BACKENDS:
            raise ValueError(f"unknown backend {backend!r}; expected one of {sorted(_BACKENDS)}")
        self._template = net                      # the converted buses, islands not yet marked
        self._net = copy.deepcopy(net)            # what the solver sees (python.rs solve path)
        pgm.mark_unreferenced_islands(self._net)
        self._precision = _BACKENDS[backend]
        self.backend = backend
        self.tol = float(tol)
        self.max_iter = int(max_iter)
        self._topo = None
        self._vm = net.vm.copy()
        self._va = net.va.copy()

    @staticmethod
    def from_pgm_json(path: str, backend: str = "scalar", tol: float = 1e-6, max_iter: int = 20,
                      s_base_va: float = 1e6, freq_hz: float = 50.0) -> "PowerFlowModel":
        """python.rs:123-168."""
        try:
            doc = pgm.load(path)
        except OSError as e:
            raise RuntimeError(f"reading {path}: {e}") from e
        except ValueError as e:
            raise ValueError(f"parsing {path} as PGM JSON: {e}") from e
        net = pgm.convert(doc, s_base_va, freq_hz, mark_islands=False)
        return PowerFlowModel(net, backend, tol, max_iter)

    def _topology(self) -> Topology:
        if self._topo is None:
            # the ZIP terms and the start-point rule of the converted network
            self._topo = pgm.topology(_gox(), self._net)
        return self._topo

    @property
    def n_nodes(self) -> int:
        """python.rs:220-225: buses, the sources' slack buses included."""
        return self._template.n_bus

    @staticmethod
    def default_threads() -> int:
        """python.rs:345-349.  The GPU batch has no worker pool; `threads`
        arguments are accepted and do not change the results."""
        return os.cpu_count() or 1

    def solve(self) -> None:
        """python.rs:245-268: linear guess, Newton-Raphson; raises RuntimeError
        when it did not converge or met a singular Jacobian."""
        net = self._net
        res = self._topology().solve(net.p_spec[None], net.q_spec[None], net.vm, net.va,
                                     tol=self.tol, max_iter=self.max_iter,
                                     precision=self._precision)
        self._vm = res.voltage_mag[0].copy()
        self._va = res.voltage_ang[0].copy()
        st = int(res.status[0])
        if st == GOX_MAX_ITERATIONS:
            raise RuntimeError(f"power flow did not converge within {self.max_iter} iterations")
        if st != GOX_CONVERGED:
            raise RuntimeError("Jacobian is singular")

    def reset(self) -> None:
        """python.rs:270-277: forget the cached factorization."""
        if self._topo is not None:
            self._topo.reset()

    def _run_batch(self, p: np.ndarray, q: np.ndarray) -> list:
        net = self._net
        res = self._topology().solve(p, q, net.vm, net.va, tol=self.tol, max_iter=self.max_iter,
                                     precision=self._precision)
        return _results(res)

    def solve_batch(self, scenarios, threads=None) -> list:
        """python.rs:279-321: per scenario a list of (bus, p_spec, q_spec)
        overrides in per unit; results in scenario order.  A bus index out of
        range raises RuntimeError (the reference's BatchError::BusOutOfRange)."""
        n = self._net.n_bus
        B = len(scenarios)
        if B == 0:
            return []
        p = np.tile(self._net.p_spec, (B, 1))
        q = np.tile(self._net.q_spec, (B, 1))
        for s, overrides in enumerate(scenarios):
            for bus, ps, qs in overrides:
                if bus < 0 or bus >= n:
                    raise RuntimeError(f"scenario {s} overrides bus {bus}, but the bus template "
                                       f"only has {n} buses")
                p[s, bus] = ps
                q[s, bus] = qs
        return self._run_batch(p, q)

    def solve_batch_scaled(self, scales, threads=None) -> list:
        """python.rs:323-343: every scale one scenario with the loaded buses'
        p_spec and q_spec multiplied by it (uniform_load_scaling,
        src/batch.rs:98-106)."""
        f = np.asarray(scales, np.float64).ravel()
        if f.shape[0] == 0:
            return []
        net = self._net
        res = self._topology().solve_scaled(f, net.p_spec, net.q_spec, net.vm, net.va, tol=self.tol,
                                            max_iter=self.max_iter, precision=self._precision)
        return _results(res)

    def ybus_triplets(self):
        """python.rs:351-377: (rows, cols, g, b), row-major, columns ascending."""
        yb = self._net.ybus
        rows = np.repeat(np.arange(yb.n), np.diff(yb.indptr)).tolist()
        return rows, yb.indices.tolist(), yb.re.tolist(), yb.im.tolist()

    def bus_spec(self):
        """python.rs:379-393: (kind, p_spec, q_spec) per bus of the template,
        kind 0 = Slack, 1 = PV, 2 = PQ."""
        kind = {G.BUS_SLACK: 0, G.BUS_PV: 1, G.BUS_PQ: 2}
        t = self._template
        return [kind[int(b)] for b in t.bus_type], t.p_spec.tolist(), t.q_spec.tolist()

    def initial_guess(self):
        """python.rs:395-406: the state Newton starts from, from the GPU."""
        net = self._net
        if net.guess_singular:
            return net.vm.tolist(), net.va.tolist()
        vm, va = self._topology().initial_guess(net.p_spec[None], net.q_spec[None], net.vm, net.va)
        return vm[0].tolist(), va[0].tolist()

    def zip_term_counts(self):
        """python.rs:408-415."""
        return self._template.zip_terms.tolist()

    def voltage_mag(self):
        """python.rs:417-421: per unit, after the last solve()."""
        return self._vm.tolist()

    def voltage_ang(self):
        """python.rs:423-426: radians."""
        return self._va.tolist()

    def voltage_kv(self):
        """python.rs:428-434: |V| times the bus's rated voltage, in kV."""
        return (self._vm * self._template.u_rated / 1e3).tolist()


def _results(res) -> list:
    """One BatchResult per scenario (rows of the batch's arrays)."""
    return list(map(BatchResult, res.voltage_mag, res.voltage_ang, res.iterations.tolist(),
                    (res.status == GOX_CONVERGED).tolist(), res.max_mismatch.tolist()))


def _gox():
    import gridoxide_gb300
    return gridoxide_gb300
