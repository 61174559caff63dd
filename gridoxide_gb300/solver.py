"""Host-side mirror of the reference's linear-solver plugin surface.

* :class:`Gb300LinearSolver` -- the ``solver::LinearSolver`` trait
  (gridoxide src/solver.rs:35-57): ``new`` / ``factor_and_solve`` /
  ``factor_and_solve_values``, ``None`` on a singular matrix.
* :class:`Topology` -- one registered topology on the GPU, the state a
  ``PersistentSolver`` keeps (src/solver.rs:395-494): Jacobian pattern,
  symbolic ordering, pivot order (fixed by the first Jacobian factored),
  ``reset``.
* :class:`BatchSolver` -- ``batch::BatchSolver::solve`` (src/batch.rs:198-289)
  with :class:`Scenario` / :class:`BusOverride` / :func:`uniform_load_scaling`
  (src/batch.rs:40-106) and :class:`BatchError` (src/batch.rs:108-135).

Every numeric call goes through ``libgridoxide_gb300.so``; there is no CPU
path here.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (GOX_CONVERGED, GOX_MAX_ITERATIONS, GOX_PRECISION_FP64, GOX_PRECISION_MIXED,
                   GOX_SINGULAR, GOX_SINGULAR_SCENARIO, check)


class SolveStatus:
    """solver::SolveStatus (src/solver.rs:162-171)."""

    Converged = GOX_CONVERGED
    MaxIterationsReached = GOX_MAX_ITERATIONS
    Singular = GOX_SINGULAR_SCENARIO


class JacobianBackend:
    """The two GB300 entries added beside Scalar/Block/Klu/KluNative/Pardiso
    (src/solver.rs:62-108)."""

    Gb300 = GOX_PRECISION_MIXED       # FP32 refactor/solve, FP64 mismatch/update
    Gb300Fp64 = GOX_PRECISION_FP64    # plain FP64 on the GPU


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


# ---------------------------------------------------------------------------
# LinearSolver

class Gb300LinearSolver:
    """LinearSolver on the GPU: symbolic + first factor on the host, FP64
    refactor and solves on the device with the fixed pivot order."""

    def __init__(self, handle, n, rows, cols):
        self._h = handle
        self.n = n
        self._rows = rows
        self._cols = cols

    @classmethod
    def new(cls, n: int, entries: Sequence) -> Optional["Gb300LinearSolver"]:
        """``LinearSolver::new``: ``None`` if singular (src/solver.rs:38-41)."""
        L = _lib.load()
        ent = list(entries)
        rows = _i32([e[0] for e in ent])
        cols = _i32([e[1] for e in ent])
        vals = _f64([e[2] for e in ent])
        h = C.c_void_p()
        rc = L.gox_ls_create(n, len(ent), _p(rows, _lib.i32p), _p(cols, _lib.i32p),
                             _p(vals, _lib.f64p), C.byref(h))
        if rc == GOX_SINGULAR:
            return None
        check(rc, "gox_ls_create")
        return cls(h, n, rows, cols)

    def factor_and_solve_values(self, values, rhs) -> Optional[np.ndarray]:
        L = _lib.load()
        x = np.zeros(self.n)
        rc = L.gox_ls_factor_solve_values(self._h, _p(_f64(values), _lib.f64p),
                                          _p(_f64(rhs), _lib.f64p), _p(x, _lib.f64p))
        if rc == GOX_SINGULAR:
            return None
        check(rc, "gox_ls_factor_solve_values")
        return x

    def factor_and_solve_values_static(self, values, rhs) -> Optional[np.ndarray]:
        """As factor_and_solve_values, allocating no device memory: for callers
        that cannot allocate at solve time (a process whose device memory is
        held by another allocator's pool, or a control loop with a deadline
        per Newton step, where cudaMalloc/cudaFree synchronize the device).
        Its scratch is a fixed array inside the library, shared by every call
        (serialize calls; see gox_ls_factor_solve_values_static)."""
        L = _lib.load()
        x = np.zeros(self.n)
        rc = L.gox_ls_factor_solve_values_static(self._h, _p(_f64(values), _lib.f64p),
                                                 _p(_f64(rhs), _lib.f64p), _p(x, _lib.f64p))
        if rc == GOX_SINGULAR:
            return None
        check(rc, "gox_ls_factor_solve_values_static")
        return x

    def factor_and_solve(self, entries, rhs) -> Optional[np.ndarray]:
        L = _lib.load()
        ent = list(entries)
        rows = _i32([e[0] for e in ent])
        cols = _i32([e[1] for e in ent])
        vals = _f64([e[2] for e in ent])
        x = np.zeros(self.n)
        rc = L.gox_ls_factor_solve(self._h, len(ent), _p(rows, _lib.i32p), _p(cols, _lib.i32p),
                                   _p(vals, _lib.f64p), _p(_f64(rhs), _lib.f64p),
                                   _p(x, _lib.f64p))
        if rc == GOX_SINGULAR:
            return None
        check(rc, "gox_ls_factor_solve")
        return x

    def __del__(self):
        try:
            if self._h:
                _lib.load().gox_ls_destroy(self._h)
                self._h = None
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Topology (PersistentSolver state) and batched solves

@dataclass
class BatchResult:
    """BatchResult of the reference's Python surface (src/python.rs:63-78)."""

    voltage_mag: np.ndarray
    voltage_ang: np.ndarray
    iterations: np.ndarray
    status: np.ndarray
    max_mismatch: np.ndarray
    history: Optional[np.ndarray] = None

    @property
    def converged(self) -> np.ndarray:
        return self.status == GOX_CONVERGED


def set_autotune(on: bool) -> None:
    """Turn the refactor-plan autotuner on (default) or off, process-wide."""
    check(_lib.load().gox_set_autotune(1 if on else 0), "gox_set_autotune")


def set_refactor_sync(progress_flags: bool) -> None:
    """How the default refactor plan of topologies analysed from now on ends
    its dependency levels: per-warp progress flags or CTA barriers (the
    default; gox_set_refactor_sync); the results are the same bit for bit."""
    check(_lib.load().gox_set_refactor_sync(1 if progress_flags else 0), "gox_set_refactor_sync")


def set_multi_persistent(on: bool) -> None:
    """multi_solve's form: one Newton loop whose phases are one launch each
    over every topology still running (default), or one persistent launch
    in which each CTA runs whole Newton loops of (topology, group) items."""
    check(_lib.load().gox_set_multi_persistent(1 if on else 0), "gox_set_multi_persistent")


def multi_solve(jobs, tol=1e-8, max_iter=20, precision=GOX_PRECISION_MIXED,
                out: Optional[list] = None) -> list:
    """Many topologies' batches solved together (gox_multi_solve): one
    Newton loop with one launch per phase over every topology still running,
    or (set_multi_persistent(True)) one persistent launch whose CTAs run
    whole Newton loops of (topology, group) items.  `jobs`: (Topology, p_spec [B, N], q_spec [B, N], vm0, va0) with
    vm0 / va0 [N] (shared) or [B, N]; each topology at most once.  Returns
    one BatchResult per job, equal bit for bit to Topology.solve on that job
    alone.  out: one BatchResult per job to write into (e.g. over pinned
    memory, reused across calls) instead of fresh arrays."""
    n = len(jobs)
    if out is not None and len(out) != n:
        raise ValueError("out must hold one BatchResult per job")
    keep, outs = [], []
    topo_a = (C.c_void_p * n)()
    arr = {k: (C.c_void_p * n)() for k in ("p", "q", "vm", "va", "ovm", "ova", "it", "st", "mm")}
    batch = np.zeros(n, np.int32)
    vstride = np.zeros(n, np.int32)
    for j, (topo, p, q, vm0, va0) in enumerate(jobs):
        p, q = _f64(p), _f64(q)
        B, N = p.shape
        vm0, va0 = _f64(vm0), _f64(va0)
        batch[j] = B
        vstride[j] = N if vm0.ndim == 2 else 0
        if out is not None:
            res = out[j]
            ok = (res.voltage_mag.shape == (B, N) and res.voltage_ang.shape == (B, N) and
                  res.iterations.shape == (B,) and res.status.shape == (B,) and
                  res.max_mismatch.shape == (B,) and res.voltage_mag.dtype == np.float64 and
                  res.voltage_ang.dtype == np.float64 and res.iterations.dtype == np.int32 and
                  res.status.dtype == np.int32 and res.max_mismatch.dtype == np.float64 and
                  all(a.flags.c_contiguous for a in (res.voltage_mag, res.voltage_ang,
                                                     res.iterations, res.status,
                                                     res.max_mismatch)))
            if not ok:
                raise ValueError("out arrays do not match the batch")
        else:
            res = BatchResult(np.empty((B, N)), np.empty((B, N)), np.zeros(B, np.int32),
                              np.zeros(B, np.int32), np.zeros(B))
        keep += [p, q, vm0, va0]
        outs.append(res)
        topo_a[j] = topo.handle.value
        for k, a in (("p", p), ("q", q), ("vm", vm0), ("va", va0), ("ovm", res.voltage_mag),
                     ("ova", res.voltage_ang), ("it", res.iterations), ("st", res.status),
                     ("mm", res.max_mismatch)):
            arr[k][j] = a.ctypes.data
    check(_lib.load().gox_multi_solve(
        n, topo_a, _p(batch, _lib.i32p), arr["p"], arr["q"], arr["vm"], arr["va"],
        _p(vstride, _lib.i32p), float(tol), int(max_iter), int(precision), arr["ovm"], arr["ova"],
        arr["it"], arr["st"], arr["mm"]), "gox_multi_solve")
    return outs


def set_repack(on: bool) -> None:
    """Re-packing of running scenarios into fewer groups in the host-driven
    Newton loop (default on; gox_set_repack); same results bit for bit."""
    check(_lib.load().gox_set_repack(1 if on else 0), "gox_set_repack")


def set_refactor_wide(min_width: int) -> None:
    """The wide kernels in the default refactor plan of topologies analysed
    from now on: leading refactor levels / trailing backward phases with at
    least `min_width` columns / rows run one level per launch across every
    SM (0, the default: none; gox_set_refactor_wide); same results bit for
    bit."""
    check(_lib.load().gox_set_refactor_wide(int(min_width)), "gox_set_refactor_wide")


class Topology:
    """A registered topology: Y-bus (CSR) + bus types, resident on the GPU."""

    def __init__(self, ybus, bus_type):
        L = _lib.load()
        self.n_bus = int(ybus.n)
        self.ybus = ybus
        self.bus_type = _i32(bus_type)
        h = C.c_void_p()
        check(L.gox_topo_register(self.n_bus, _p(_i32(ybus.indptr), _lib.i32p),
                                  _p(_i32(ybus.indices), _lib.i32p), _p(_f64(ybus.re), _lib.f64p),
                                  _p(_f64(ybus.im), _lib.f64p), _p(self.bus_type, _lib.i32p),
                                  C.byref(h)), "gox_topo_register")
        self._h = h

    @property
    def handle(self):
        return self._h

    def reset(self):
        """PersistentSolver::reset: forget the fixed pivot order."""
        check(_lib.load().gox_topo_reset(self._h), "gox_topo_reset")

    def solve(self, p_spec, q_spec, vm0, va0, tol=1e-8, max_iter=20,
              precision=GOX_PRECISION_MIXED, outage=None, history=False,
              out: Optional[BatchResult] = None) -> BatchResult:
        """Batched NR on host arrays (inputs/outputs copied to/from the GPU).

        p_spec/q_spec [B, N]; vm0/va0 [N] (shared) or [B, N];
        outage = (slots [B,4], dre [B,4], dim [B,4]) or None.
        out: a BatchResult of the right shapes to write into (e.g. over
        pinned memory, reused across calls) instead of fresh arrays."""
        L = _lib.load()
        p_spec = _f64(np.atleast_2d(p_spec))
        q_spec = _f64(np.atleast_2d(q_spec))
        B, n = p_spec.shape
        if n != self.n_bus or q_spec.shape != p_spec.shape:
            raise ValueError("p_spec/q_spec must be [B, n_bus]")
        vm0 = _f64(vm0)
        va0 = _f64(va0)
        stride = n if vm0.ndim == 2 else 0
        if out is not None:
            vm, va, iters, status, mis = (out.voltage_mag, out.voltage_ang, out.iterations,
                                          out.status, out.max_mismatch)
            hist = out.history if history else None
            ok = (vm.shape == (B, n) and va.shape == (B, n) and iters.shape == (B,) and
                  status.shape == (B,) and mis.shape == (B,) and vm.dtype == np.float64 and
                  va.dtype == np.float64 and iters.dtype == np.int32 and status.dtype == np.int32 and
                  mis.dtype == np.float64 and all(a.flags.c_contiguous for a in (vm, va, iters, status, mis)) and
                  (not history or (hist is not None and hist.shape == (B, max_iter) and
                                   hist.dtype == np.float64 and hist.flags.c_contiguous)))
            if not ok:
                raise ValueError("out arrays do not match the batch")
        else:
            vm = np.empty((B, n))
            va = np.empty((B, n))
            iters = np.zeros(B, np.int32)
            status = np.zeros(B, np.int32)
            mis = np.zeros(B)
            hist = np.zeros((B, max_iter)) if history else None
        if outage is not None:
            sl, dr, di = _i32(outage[0]), _f64(outage[1]), _f64(outage[2])
        else:
            sl = dr = di = None
        rc = L.gox_batch_solve(self._h, B, _p(p_spec, _lib.f64p), _p(q_spec, _lib.f64p),
                               _p(vm0, _lib.f64p), _p(va0, _lib.f64p), stride,
                               _p(sl, _lib.i32p), _p(dr, _lib.f64p), _p(di, _lib.f64p),
                               float(tol), int(max_iter), int(precision), _p(vm, _lib.f64p),
                               _p(va, _lib.f64p), _p(iters, _lib.i32p), _p(status, _lib.i32p),
                               _p(mis, _lib.f64p), _p(hist, _lib.f64p))
        if rc == _lib.GOX_E_BUS_RANGE:
            raise BatchError("BusOutOfRange", rc)
        check(rc, "gox_batch_solve")
        return BatchResult(vm, va, iters, status, mis, hist)

    def outage_islands(self, outage):
        """Components of each outage scenario's grid (gox_outage_islands):
        (n_islands [B], island_of [B, N], verdict [B, N]) with verdict 0 =
        one slack bus, 1 = none (pinned to V = 0 by the solves), 2 = several."""
        sl, dr, di = _i32(outage[0]), _f64(outage[1]), _f64(outage[2])
        B, n = sl.shape[0], self.n_bus
        nis = np.zeros(B, np.int32)
        lab = np.zeros((B, n), np.int32)
        ver = np.zeros((B, n), np.int32)
        check(_lib.load().gox_outage_islands(self._h, B, _p(sl, _lib.i32p), _p(dr, _lib.f64p),
                                             _p(di, _lib.f64p), _p(nis, _lib.i32p),
                                             _p(lab, _lib.i32p), _p(ver, _lib.i32p)),
              "gox_outage_islands")
        return nis, lab, ver

    def solve_qlim(self, p_spec, q_spec, vm0, va0, q_min, q_max, tol=1e-8, max_iter=20,
                   max_outer=10, precision=GOX_PRECISION_MIXED):
        """Batched NR enforcing the PV buses' reactive limits
        (gox_batch_solve_qlim; newton_raphson_enforcing_q_limits,
        src/solver.rs:545-618).  q_min/q_max [N] per unit.  Returns
        (BatchResult of the last solves, switched [B, N] bool,
        stabilized [B] bool)."""
        L = _lib.load()
        p_spec = _f64(np.atleast_2d(p_spec))
        q_spec = _f64(np.atleast_2d(q_spec))
        B, n = p_spec.shape
        if n != self.n_bus or q_spec.shape != p_spec.shape:
            raise ValueError("p_spec/q_spec must be [B, n_bus]")
        vm0, va0, q_min, q_max = _f64(vm0), _f64(va0), _f64(q_min), _f64(q_max)
        if q_min.shape != (n,) or q_max.shape != (n,):
            raise ValueError("q_min/q_max must be [n_bus]")
        vm, va = np.empty((B, n)), np.empty((B, n))
        iters, status, mis = np.zeros(B, np.int32), np.zeros(B, np.int32), np.zeros(B)
        nsw, stab = np.zeros(B, np.int32), np.zeros(B, np.int32)
        sw = np.zeros((B, n), np.uint8)
        check(L.gox_batch_solve_qlim(self._h, B, _p(p_spec, _lib.f64p), _p(q_spec, _lib.f64p),
                                     _p(vm0, _lib.f64p), _p(va0, _lib.f64p),
                                     n if vm0.ndim == 2 else 0, _p(q_min, _lib.f64p),
                                     _p(q_max, _lib.f64p), float(tol), int(max_iter),
                                     int(max_outer), int(precision), _p(vm, _lib.f64p),
                                     _p(va, _lib.f64p), _p(iters, _lib.i32p), _p(status, _lib.i32p),
                                     _p(mis, _lib.f64p), _p(nsw, _lib.i32p),
                                     sw.ctypes.data_as(C.POINTER(C.c_uint8)), _p(stab, _lib.i32p)),
              "gox_batch_solve_qlim")
        assert np.array_equal(nsw, sw.sum(axis=1))
        return BatchResult(vm, va, iters, status, mis, None), sw.astype(bool), stab.astype(bool)

    def solve_scaled(self, scales, p_base, q_base, vm0, va0, tol=1e-8, max_iter=20,
                     precision=GOX_PRECISION_MIXED, history=False) -> BatchResult:
        """Batched NR over uniformly scaled injections (gox_batch_solve_scaled):
        scenario s has p_base * scales[s], q_base * scales[s]; vm0/va0 [N]."""
        L = _lib.load()
        scales = _f64(np.ravel(scales))
        p_base, q_base, vm0, va0 = _f64(p_base), _f64(q_base), _f64(vm0), _f64(va0)
        B, n = scales.shape[0], self.n_bus
        if any(a.shape != (n,) for a in (p_base, q_base, vm0, va0)):
            raise ValueError("p_base/q_base/vm0/va0 must be [n_bus]")
        vm, va = np.empty((B, n)), np.empty((B, n))
        iters, status, mis = np.zeros(B, np.int32), np.zeros(B, np.int32), np.zeros(B)
        hist = np.zeros((B, max_iter)) if history else None
        check(L.gox_batch_solve_scaled(self._h, B, _p(scales, _lib.f64p), _p(p_base, _lib.f64p),
                                       _p(q_base, _lib.f64p), _p(vm0, _lib.f64p),
                                       _p(va0, _lib.f64p), float(tol), int(max_iter),
                                       int(precision), _p(vm, _lib.f64p), _p(va, _lib.f64p),
                                       _p(iters, _lib.i32p), _p(status, _lib.i32p),
                                       _p(mis, _lib.f64p), _p(hist, _lib.f64p)),
              "gox_batch_solve_scaled")
        return BatchResult(vm, va, iters, status, mis, hist)

    def solve_device(self, p_spec, q_spec, vm0, va0, vm_out, va_out, iters, status, max_mis,
                     tol=1e-8, max_iter=20, precision=GOX_PRECISION_MIXED, outage=None,
                     history=None, stream=None):
        """Batched NR on device tensors (torch CUDA tensors, contiguous):
        p/q/vm_out/va_out float64 [B, N]; vm0/va0 float64 [N] or [B, N];
        iters/status int32 [B]; max_mis float64 [B]; outage = (slots int32
        [B,4], dre, dim float64 [B,4]) or None; history float64 [B, max_iter]
        or None.  Work is enqueued on `stream` (a torch.cuda.Stream or None)."""
        L = _lib.load()
        B, n = p_spec.shape
        stride = n if vm0.dim() == 2 else 0
        ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())
        sl, dr, di = outage if outage is not None else (None, None, None)
        st = None if stream is None else C.c_void_p(stream.cuda_stream)
        rc = L.gox_batch_solve_device(self._h, B, ptr(p_spec), ptr(q_spec), ptr(vm0), ptr(va0),
                                      stride, ptr(sl), ptr(dr), ptr(di), float(tol),
                                      int(max_iter), int(precision), ptr(vm_out), ptr(va_out),
                                      ptr(iters), ptr(status), ptr(max_mis), ptr(history), st)
        if rc == _lib.GOX_E_BUS_RANGE:
            raise BatchError("BusOutOfRange", rc)
        check(rc, "gox_batch_solve_device")

    def prepare(self, p_spec, q_spec, vm0, va0, tol=1e-8, outage=None):
        """Fix the pivot order on the host (no GPU needed); see gox_topo_prepare."""
        L = _lib.load()
        p_spec = _f64(np.atleast_2d(p_spec))
        q_spec = _f64(np.atleast_2d(q_spec))
        vm0, va0 = _f64(vm0), _f64(va0)
        stride = self.n_bus if vm0.ndim == 2 else 0
        sl, dr, di = (None, None, None) if outage is None else (
            _i32(outage[0]), _f64(outage[1]), _f64(outage[2]))
        rc = L.gox_topo_prepare(self._h, p_spec.shape[0], _p(p_spec, _lib.f64p),
                                _p(q_spec, _lib.f64p), _p(vm0, _lib.f64p), _p(va0, _lib.f64p),
                                stride, _p(sl, _lib.i32p), _p(dr, _lib.f64p), _p(di, _lib.f64p),
                                float(tol))
        if rc == GOX_SINGULAR:
            return False
        check(rc, "gox_topo_prepare")
        return True

    def emulate_step(self, jac_vals, rhs) -> Optional[np.ndarray]:
        """Host FP64 mirror of the device refactor + solve schedule."""
        L = _lib.load()
        dx = np.zeros(len(rhs))
        rc = L.gox_topo_emulate_step(self._h, _p(_f64(jac_vals), _lib.f64p),
                                     _p(_f64(rhs), _lib.f64p), _p(dx, _lib.f64p))
        if rc == GOX_SINGULAR:
            return None
        check(rc, "gox_topo_emulate_step")
        return dx

    def factor_values(self, p_spec, q_spec, vm, va, precision=GOX_PRECISION_FP64):
        """The device's Jacobian (emission order) and factor (LU slot layout:
        per factor column its U entries, diagonal, L entries) at the given
        voltages, [B, nnzJ] and [B, slots]; see gox_topo_factor_values."""
        L = _lib.load()
        p_spec, q_spec = _f64(np.atleast_2d(p_spec)), _f64(np.atleast_2d(q_spec))
        vm, va = _f64(np.atleast_2d(vm)), _f64(np.atleast_2d(va))
        B = p_spec.shape[0]
        if not (q_spec.shape == vm.shape == va.shape == p_spec.shape and p_spec.shape[1] == self.n_bus):
            raise ValueError("factor_values: arrays must be [B, n_bus]")
        inf = self.info()
        jac = np.zeros((B, inf["nnz_j"]))
        lu = np.zeros((B, inf["lu_slots"]))
        check(L.gox_topo_factor_values(self._h, B, _p(p_spec, _lib.f64p), _p(q_spec, _lib.f64p),
                                       _p(vm, _lib.f64p), _p(va, _lib.f64p), int(precision),
                                       _p(jac, _lib.f64p), _p(lu, _lib.f64p)),
              "gox_topo_factor_values")
        return jac, lu

    def pivot_solve(self, jac_vals, rhs) -> Optional[np.ndarray]:
        """dx of J dx = rhs with J factored afresh with threshold partial
        pivoting on the GPU (the mixed path's repair of a poor static pivot
        order; gox_topo_pivot_solve); None when singular."""
        L = _lib.load()
        dx = np.zeros(len(rhs))
        rc = L.gox_topo_pivot_solve(self._h, _p(_f64(jac_vals), _lib.f64p),
                                    _p(_f64(rhs), _lib.f64p), _p(dx, _lib.f64p))
        if rc == GOX_SINGULAR:
            return None
        check(rc, "gox_topo_pivot_solve")
        return dx

    def stream_word(self, precision: int, warp: int, index: int, value: int) -> int:
        """Test hook: replace one word of the device refactor stream; returns the
        old word (gox_topo_stream_word)."""
        old = np.zeros(1, np.int32)
        check(_lib.load().gox_topo_stream_word(self._h, int(precision), int(warp), int(index),
                                               int(value), _p(old, _lib.i32p)),
              "gox_topo_stream_word")
        return int(old[0])

    def tuning(self, precision=GOX_PRECISION_MIXED) -> dict:
        """The refactor plan in `precision` and the autotuner's timed
        candidates (gox_topo_tuning)."""
        plan = np.zeros(9, np.int64)
        table = np.zeros((128, 7))
        rows = check(_lib.load().gox_topo_tuning(self._h, int(precision), _p(plan, _lib.i64p),
                                                 _p(table, _lib.f64p), 128), "gox_topo_tuning")
        return {"warps": int(plan[0]), "ring_rows": int(plan[1]), "big_rows": int(plan[2]),
                "chunk_words": int(plan[3]),
                "source": ("default", "measured", "cached")[int(plan[4])],
                "progress_flags": bool(plan[6]), "wide_levels": int(plan[7]),
                "wide_phases": int(plan[8]),
                "candidates": [dict(warps=int(r[0]), chunk_words=int(r[1]), ring_rows=int(r[2]),
                                    ms=float(r[3]), progress_flags=bool(r[4]),
                                    wide_levels=int(r[5]), wide_phases=int(r[6]))
                               for r in table[:rows]]}

    def info(self) -> dict:
        a = np.zeros(36, np.int64)
        check(_lib.load().gox_topo_info(self._h, _p(a, _lib.i64p)), "gox_topo_info")
        keys = ["n_u", "nnz_j", "nnz_l", "nnz_u", "nnz_off", "nblocks", "levels", "phases",
                "lu_slots", "max_collen", "rf32_warps", "rf32_ring_rows", "rf32_est_cycles",
                "rf32_rows_in_place", "rf32_rows_copied", "rf32_rows_ahead", "rf32_rows_at_start",
                "rf32_rows_just_in_time", "rf32_steps", "rf32_waits", "rf64_warps",
                "rf64_ring_rows", "rf64_est_cycles", "rf64_rows_in_place", "rf32_column_cmds",
                "rf32_stream_words", "rf32_with_bwd", "rf64_with_bwd", "rf32_pre_columns",
                "rf32_rows_by_helpers", "graph_solves", "rf32_progress_flags",
                "rf32_flag_waits", "rf32_flag_warps_waited", "rf32_wide_levels",
                "rf32_wide_phases"]
        return dict(zip(keys, [int(v) for v in a]))

    def structure(self) -> dict:
        inf = self.info()
        n = inf["n_u"]
        out = dict(P=np.zeros(n, np.int32), Q=np.zeros(n, np.int32),
                   R=np.zeros(inf["nblocks"] + 1, np.int32), Lp=np.zeros(n + 1, np.int32),
                   Li=np.zeros(max(inf["nnz_l"], 1), np.int32), Up=np.zeros(n + 1, np.int32),
                   Ui=np.zeros(max(inf["nnz_u"], 1), np.int32), flops=np.zeros(2))
        check(_lib.load().gox_topo_structure(
            self._h, *[_p(out[k], _lib.i32p) for k in ("P", "Q", "R", "Lp", "Li", "Up", "Ui")],
            _p(out["flops"], _lib.f64p)), "gox_topo_structure")
        out["Li"] = out["Li"][:inf["nnz_l"]]
        out["Ui"] = out["Ui"][:inf["nnz_u"]]
        return out

    def set_timing(self, on: bool):
        check(_lib.load().gox_set_timing(self._h, 1 if on else 0), "gox_set_timing")

    def last_timing(self) -> dict:
        a = np.zeros(6)
        check(_lib.load().gox_last_timing(self._h, _p(a, _lib.f64p)), "gox_last_timing")
        return dict(iterations=a[0], total_ms=a[1], mismatch_ms=a[2], fill_ms=a[3],
                    refactor_ms=a[4], solve_ms=a[5])

    def last_launches(self) -> int:
        return int(_lib.load().gox_last_launches(self._h))

    def repacks(self) -> int:
        """Re-packs of running scenarios into fewer groups so far (gox_topo_repacks)."""
        return int(_lib.load().gox_topo_repacks(self._h))

    def set_pivot_tolerance(self, tol: float) -> None:
        """Mixed path: scenarios whose FP32 refactor meets |u_kk| < tol *
        max|L(:, k)| are solved again in FP64 (default 1e-6; 0 disables)."""
        check(_lib.load().gox_set_pivot_tolerance(self._h, float(tol)), "gox_set_pivot_tolerance")

    def last_fallbacks(self) -> int:
        """Scenarios of the last solve that were solved again in FP64."""
        return int(_lib.load().gox_last_fallbacks(self._h))

    def set_zip(self, imp=None, cur=None) -> None:
        """ZIP terms of the effective injection (src/network.rs:600-611): per
        bus complex constant-impedance and constant-current injections (per
        unit at |V| = 1), added as imp |V|^2 + cur |V| to p_spec + j q_spec in
        every mismatch; None for both clears them."""
        L = _lib.load()
        if imp is None and cur is None:
            check(L.gox_topo_set_zip(self._h, None, None, None, None), "gox_topo_set_zip")
            return
        imp = np.zeros(self.n_bus, np.complex128) if imp is None else np.asarray(imp, np.complex128)
        cur = np.zeros(self.n_bus, np.complex128) if cur is None else np.asarray(cur, np.complex128)
        a = [_f64(imp.real), _f64(imp.imag), _f64(cur.real), _f64(cur.imag)]
        check(L.gox_topo_set_zip(self._h, *[_p(x, _lib.f64p) for x in a]), "gox_topo_set_zip")

    def set_split(self, parts: int) -> None:
        """Solve large batches as 1 to 8 concurrent parts, 0 by batch size (gox_topo_set_split)."""
        check(_lib.load().gox_topo_set_split(self._h, int(parts)), "gox_topo_set_split")

    def set_graph(self, on: bool) -> None:
        """Run the Newton loop as a captured CUDA graph (default) or host-driven."""
        check(_lib.load().gox_topo_set_graph(self._h, 1 if on else 0), "gox_topo_set_graph")

    def set_initial_guess(self, mode: str) -> None:
        """Start point of the batched solves: "given" (vm0/va0 as passed) or
        "linear" (the reference BatchSolver's linear initial guess from them,
        src/network.rs:627-678, on the GPU)."""
        code = {"given": _lib.GOX_GUESS_GIVEN, "linear": _lib.GOX_GUESS_LINEAR}[mode]
        check(_lib.load().gox_topo_set_initial_guess(self._h, code), "gox_topo_set_initial_guess")

    def initial_guess(self, p_spec, q_spec, vm0, va0):
        """The linear initial guess (src/network.rs:627-678) of each scenario,
        computed on the GPU: ([B, N] |V|, [B, N] theta); the given start where
        the guess system is singular."""
        p_spec = _f64(np.atleast_2d(p_spec))
        q_spec = _f64(np.atleast_2d(q_spec))
        B, n = p_spec.shape
        if n != self.n_bus or q_spec.shape != p_spec.shape:
            raise ValueError("p_spec/q_spec must be [B, n_bus]")
        vm0, va0 = _f64(vm0), _f64(va0)
        vm, va = np.empty((B, n)), np.empty((B, n))
        check(_lib.load().gox_topo_initial_guess(
            self._h, B, _p(p_spec, _lib.f64p), _p(q_spec, _lib.f64p), _p(vm0, _lib.f64p),
            _p(va0, _lib.f64p), n if vm0.ndim == 2 else 0, _p(vm, _lib.f64p), _p(va, _lib.f64p)),
            "gox_topo_initial_guess")
        return vm, va

    def __del__(self):
        try:
            if self._h:
                _lib.load().gox_topo_destroy(self._h)
                self._h = None
        except Exception:
            pass


# ---------------------------------------------------------------------------
# BatchSolver mirror

@dataclass
class BusOverride:
    """batch::BusOverride (src/batch.rs:40-68)."""

    bus: int
    p_spec: Optional[float] = None
    q_spec: Optional[float] = None
    voltage_mag: Optional[float] = None


@dataclass
class Scenario:
    """batch::Scenario (src/batch.rs:73-91).  ``branch_outages`` holds at most
    one branch index here: the N-1 outage keeps the branch's Y-bus entries in
    the pattern and zeroes its series admittance and charging."""

    bus_overrides: list = field(default_factory=list)
    branch_outages: list = field(default_factory=list)


class BatchError(Exception):
    """batch::BatchError (src/batch.rs:108-135)."""

    def __init__(self, kind: str, detail=None):
        self.kind = kind
        self.detail = detail
        super().__init__(f"{kind}: {detail}")


def uniform_load_scaling(p_spec, q_spec, factor: float) -> Scenario:
    """batch::uniform_load_scaling (src/batch.rs:98-106)."""
    ov = [BusOverride(i, float(p) * factor, float(q) * factor)
          for i, (p, q) in enumerate(zip(p_spec, q_spec)) if p != 0.0 or q != 0.0]
    return Scenario(ov)


@dataclass
class Buses:
    """The bus template: per-bus arrays of the reference's ``Bus`` fields the
    engine consumes (src/types.rs:26-42)."""

    bus_type: np.ndarray
    voltage_mag: np.ndarray
    voltage_ang: np.ndarray
    p_spec: np.ndarray
    q_spec: np.ndarray


@dataclass
class PowerFlowReport:
    voltage_mag: np.ndarray
    voltage_ang: np.ndarray
    status: int
    mismatch_history: np.ndarray

    @property
    def iterations(self) -> int:
        return len(self.mismatch_history)


class BatchSolver:
    """batch::BatchSolver with a GB300 backend.  Scenario validation, the
    linear initial guess before every scenario and result order follow
    src/batch.rs:198-289; the work runs as one GPU batch instead of a rayon
    work queue."""

    def __init__(self, backend=JacobianBackend.Gb300):
        self.backend = backend
        self._topos = {}

    def solve(self, buses: Buses, ybus, scenarios: Sequence[Scenario], tol: float,
              max_iter: int, branch_stamps=None) -> list:
        """``branch_stamps(branch) -> (slots[4], dre[4], dim[4])`` supplies the
        Y-bus deltas of an outage (see grids.outage_deltas)."""
        n = len(buses.bus_type)
        for i, sc in enumerate(scenarios):
            for ov in sc.bus_overrides:
                if ov.bus < 0 or ov.bus >= n:
                    raise BatchError("BusOutOfRange", dict(scenario=i, bus=ov.bus, n_buses=n))
            if len(sc.branch_outages) > 1 or (sc.branch_outages and branch_stamps is None):
                raise BatchError("OutagesUnsupported", dict(scenario=i))
        if len(scenarios) == 0:
            return []
        B = len(scenarios)
        p = np.tile(_f64(buses.p_spec), (B, 1))
        q = np.tile(_f64(buses.q_spec), (B, 1))
        vm = np.tile(_f64(buses.voltage_mag), (B, 1))
        va = np.tile(_f64(buses.voltage_ang), (B, 1))
        outage = None
        if any(sc.branch_outages for sc in scenarios):
            sl = np.full((B, 4), -1, np.int32)
            dr = np.zeros((B, 4))
            di = np.zeros((B, 4))
            for s, sc in enumerate(scenarios):
                if sc.branch_outages:
                    sl[s], dr[s], di[s] = branch_stamps(sc.branch_outages[0])
            outage = (sl, dr, di)
        for s, sc in enumerate(scenarios):
            for ov in sc.bus_overrides:
                if ov.p_spec is not None:
                    p[s, ov.bus] = ov.p_spec
                if ov.q_spec is not None:
                    q[s, ov.bus] = ov.q_spec
                if ov.voltage_mag is not None:
                    vm[s, ov.bus] = ov.voltage_mag
        key = id(ybus)
        topo = self._topos.get(key)
        if topo is None:
            topo = Topology(ybus, buses.bus_type)
            topo.set_initial_guess("linear")  # every scenario starts from it (src/batch.rs:268)
            self._topos[key] = topo
        res = topo.solve(p, q, vm, va, tol=tol, max_iter=max_iter, precision=self.backend,
                         outage=outage, history=True)
        return [PowerFlowReport(res.voltage_mag[s], res.voltage_ang[s], int(res.status[s]),
                                res.history[s, :res.iterations[s]]) for s in range(B)]


def analyze(n: int, Ap, Ai):
    """klu_analyze (BTF + AMD) through the library: (P, Q, R)."""
    L = _lib.load()
    P = np.zeros(n, np.int32)
    Q = np.zeros(n, np.int32)
    R = np.zeros(n + 1, np.int32)
    nb = check(L.gox_analyze(n, _p(_i32(Ap), _lib.i32p), _p(_i32(Ai), _lib.i32p),
                             _p(P, _lib.i32p), _p(Q, _lib.i32p), _p(R, _lib.i32p)), "gox_analyze")
    return P, Q, R[:nb + 1].copy()


def factor_host(n: int, rows, cols, vals) -> Optional[dict]:
    """The host partial-pivoting factorization (klu_extract layout), or None."""
    L = _lib.load()
    rows, cols, vals = _i32(rows), _i32(cols), _f64(vals)
    sz = np.zeros(4, np.int64)
    args = (n, len(rows), _p(rows, _lib.i32p), _p(cols, _lib.i32p), _p(vals, _lib.f64p),
            _p(sz, _lib.i64p))
    rc = L.gox_factor_host(*args, *([None] * 12))
    if rc == GOX_SINGULAR:
        return None
    check(rc, "gox_factor_host")
    lnz, unz, nzoff, nb = [int(v) for v in sz]
    out = dict(Lp=np.zeros(n + 1, np.int32), Li=np.zeros(lnz, np.int32), Lx=np.zeros(lnz),
               Up=np.zeros(n + 1, np.int32), Ui=np.zeros(unz, np.int32), Ux=np.zeros(unz),
               Fp=np.zeros(n + 1, np.int32), Fi=np.zeros(max(nzoff, 1), np.int32),
               Fx=np.zeros(max(nzoff, 1)), P=np.zeros(n, np.int32), Q=np.zeros(n, np.int32),
               R=np.zeros(nb + 1, np.int32))
    keys = ("Lp", "Li", "Lx", "Up", "Ui", "Ux", "Fp", "Fi", "Fx", "P", "Q", "R")
    check(L.gox_factor_host(*args, *[_p(out[k], _lib.i32p if out[k].dtype == np.int32
                                        else _lib.f64p) for k in keys]), "gox_factor_host")
    out["Fi"] = out["Fi"][:nzoff]
    out["Fx"] = out["Fx"][:nzoff]
    return out


class Server:
    """Continuous batching of single-scenario requests over registered
    topologies (gox_server_*): worker threads in the library batch the
    queued requests of a topology (one batch per topology at a time, or up
    to ``set_lanes`` on clones of it) and solve them on the GPU; ``poll``
    returns a request's report (with its latency) once solved.  A
    registered Topology is used by the server's threads only."""

    def __init__(self, max_batch: int = 1024, precision: int = GOX_PRECISION_MIXED,
                 tol: float = 1e-8, max_iter: int = 20):
        L = _lib.load()
        h = C.c_void_p()
        check(L.gox_server_create(int(max_batch), int(precision), float(tol), int(max_iter),
                                  C.byref(h)), "gox_server_create")
        self._h = h
        self._topos = []
        self._n = []

    def add_topology(self, topo: "Topology") -> int:
        tid = C.c_int32()
        check(_lib.load().gox_server_add_topology(self._h, topo._h, C.byref(tid)),
              "gox_server_add_topology")
        self._topos.append(topo)
        self._n.append(topo.n_bus)
        return int(tid.value)

    def submit(self, topo_id: int, p_spec, q_spec, vm0, va0, outage=None) -> int:
        n = self._n[topo_id]
        arrs = [_f64(a) for a in (p_spec, q_spec, vm0, va0)]
        if any(a.shape != (n,) for a in arrs):
            raise ValueError("p_spec, q_spec, vm0, va0 must be [n_bus]")
        if outage is not None:
            sl, dr, di = _i32(outage[0]), _f64(outage[1]), _f64(outage[2])
            op = (_p(sl, _lib.i32p), _p(dr, _lib.f64p), _p(di, _lib.f64p))
        else:
            op = (None, None, None)
        t = C.c_int64()
        check(_lib.load().gox_server_submit(self._h, int(topo_id), *[_p(a, _lib.f64p) for a in arrs],
                                            *op, C.byref(t)), "gox_server_submit")
        return int(t.value)

    def submit_many(self, topo_ids, p_ptrs, q_ptrs, vm_ptrs, va_ptrs, out_ptrs=None) -> np.ndarray:
        """Queues len(topo_ids) requests in one call (gox_server_submit_many),
        the inputs by address: uint64 arrays holding, per request, the
        address of its contiguous float64 [n_bus] p_spec, q_spec, vm0, va0;
        out_ptrs = (slot, dre, dim) uint64 address arrays (0: no outage) or
        None.  The caller keeps the addressed arrays alive during the call
        (the library copies them).  Returns the tickets."""
        ids = _i32(topo_ids)
        m = len(ids)
        cols = [np.ascontiguousarray(a, dtype=np.uint64) for a in (p_ptrs, q_ptrs, vm_ptrs, va_ptrs)]
        if any(c.shape != (m,) for c in cols) or m == 0 or any(np.any(c == 0) for c in cols):
            raise ValueError("one non-null address per request and array")
        if np.any(ids < 0) or np.any(ids >= len(self._n)):
            raise ValueError("unknown topology id")
        if out_ptrs is not None:
            outs = [np.ascontiguousarray(a, dtype=np.uint64) for a in out_ptrs]
            if len(outs) != 3 or any(o.shape != (m,) for o in outs):
                raise ValueError("out_ptrs: three address arrays, one entry per request")
        tickets = np.zeros(m, np.int64)
        vpp = _lib.vpp
        args = [c.ctypes.data_as(vpp) for c in cols]
        oargs = [o.ctypes.data_as(vpp) for o in outs] if out_ptrs is not None else [None] * 3
        check(_lib.load().gox_server_submit_many(self._h, m, _p(ids, _lib.i32p), *args, *oargs,
                                                 _p(tickets, _lib.i64p)), "gox_server_submit_many")
        return tickets

    def poll(self, ticket: int, n_bus: int) -> Optional[dict]:
        vm, va = np.zeros(n_bus), np.zeros(n_bus)
        it, st = C.c_int32(), C.c_int32()
        mm, lat = C.c_double(), C.c_double()
        rc = _lib.load().gox_server_poll(self._h, int(ticket), _p(vm, _lib.f64p), _p(va, _lib.f64p),
                                         C.byref(it), C.byref(st), C.byref(mm), C.byref(lat))
        if rc == _lib.GOX_PENDING:
            return None
        check(rc, "gox_server_poll")
        return dict(vm=vm, va=va, iterations=int(it.value), status=int(st.value),
                    max_mismatch=float(mm.value), latency_s=float(lat.value))

    def wait(self, ticket: int, n_bus: int, timeout: float = 120.0) -> dict:
        import time
        t0 = time.perf_counter()
        while True:
            r = self.poll(ticket, n_bus)
            if r is not None:
                return r
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError(f"request {ticket} not solved in {timeout} s")
            time.sleep(1e-4)

    def stats(self) -> dict:
        a = np.zeros(8, np.int64)
        check(_lib.load().gox_server_stats(self._h, _p(a, _lib.i64p)), "gox_server_stats")
        return dict(batches=int(a[0]), solved=int(a[1]), queued=int(a[2]),
                    reserved_bytes=int(a[3]), peak_reserved_bytes=int(a[4]),
                    queue_us=int(a[5]), solve_us=int(a[6]), clones=int(a[7]))

    def set_lanes(self, lanes: int) -> None:
        """Batches of one topology solved at the same time, 1..8 (gox_server_set_lanes)."""
        check(_lib.load().gox_server_set_lanes(self._h, int(lanes)), "gox_server_set_lanes")

    def set_budget(self, nbytes: int) -> None:
        """Admit batches by an HBM budget in bytes (0: none)."""
        check(_lib.load().gox_server_set_budget(self._h, int(nbytes)), "gox_server_set_budget")

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().gox_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
