"""The C-ABI library: loads, exports every symbol include/*.h declares, and
rejects bad input with the documented status codes -- without a GPU."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu
from gridoxide_gb300 import _lib
from gridoxide_gb300 import grids as G


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(gox_\w+)\s*\(", src)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(gox):
    L = _lib.load()
    names = _declared()
    assert set(names) == set(_lib.SIGNATURES)
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_version(gox):
    assert b"sm_103a" in _lib.load().gox_version()


def test_invalid_arguments(gox):
    L = _lib.load()
    Ap = np.array([0, 2, 1], np.int32)  # decreasing column pointers
    Ai = np.array([0, 1], np.int32)
    P = np.zeros(2, np.int32); Q = np.zeros(2, np.int32); R = np.zeros(3, np.int32)
    p = lambda a: a.ctypes.data_as(_lib.i32p)
    assert L.gox_analyze(2, p(Ap), p(Ai), p(P), p(Q), p(R)) == _lib.GOX_E_INVALID
    # unsorted Y-bus row
    h = C.c_void_p()
    yp = np.array([0, 2, 3], np.int32)
    yi = np.array([1, 0, 1], np.int32)
    yr = np.ones(3); yim = np.ones(3)
    bt = np.array([3, 1], np.int32)
    f = lambda a: a.ctypes.data_as(_lib.f64p)
    assert L.gox_topo_register(2, p(yp), p(yi), f(yr), f(yim), p(bt), C.byref(h)) == _lib.GOX_E_INVALID
    bt_bad = np.array([3, 7], np.int32)
    yi_ok = np.array([0, 1, 1], np.int32)
    assert L.gox_topo_register(2, p(yp), p(yi_ok), f(yr), f(yim), p(bt_bad), C.byref(h)) == _lib.GOX_E_INVALID


def test_topology_register_and_empty_batch_without_gpu(gox):
    g = G.config_grid("case118")
    topo = gox.Topology(G.build_ybus(g), g.bus_type)
    res = topo.solve(np.zeros((0, g.n_bus)), np.zeros((0, g.n_bus)), g.vm, g.va)
    assert res.voltage_mag.shape == (0, g.n_bus)
    with pytest.raises(gox.GoxError):
        topo.info()  # no pivot order fixed yet


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_no_device_is_reported(gox):
    g = G.config_grid("case118")
    topo = gox.Topology(G.build_ybus(g), g.bus_type)
    with pytest.raises(gox.GoxError) as ei:
        topo.solve(g.p_spec[None], g.q_spec[None], g.vm, g.va)
    assert ei.value.code == _lib.GOX_E_NO_DEVICE


def test_batch_solver_validation(gox):
    """BatchError cases of batch_solver_test.rs:188-217."""
    g = G.config_grid("case118")
    yb = G.build_ybus(g)
    buses = gox.Buses(g.bus_type, g.vm, g.va, g.p_spec, g.q_spec)
    bs = gox.BatchSolver(gox.JacobianBackend.Gb300)
    with pytest.raises(gox.BatchError) as ei:
        bs.solve(buses, yb, [gox.Scenario([gox.BusOverride(500, 1.0)])], 1e-8, 20)
    assert ei.value.kind == "BusOutOfRange"
    with pytest.raises(gox.BatchError) as ei:
        bs.solve(buses, yb, [gox.Scenario([], [3])], 1e-8, 20)
    assert ei.value.kind == "OutagesUnsupported"
    assert bs.solve(buses, yb, [], 1e-8, 20) == []
    sc = gox.uniform_load_scaling(g.p_spec, g.q_spec, 1.1)
    assert all(ov.p_spec == pytest.approx(g.p_spec[ov.bus] * 1.1) for ov in sc.bus_overrides)


def test_loop_settings_validate_without_gpu(gox):
    """Split parts (0 = by batch size, 1..8), re-packing and the other
    process-wide loop and plan switches take their documented values and
    reject the rest, without a GPU."""
    from gridoxide_gb300 import solver as S
    g = G.config_grid("case118")
    topo = gox.Topology(G.build_ybus(g), g.bus_type)
    for k in (0, 1, 2, 8):
        topo.set_split(k)
    for bad in (-1, 9):
        with pytest.raises(gox.GoxError):
            topo.set_split(bad)
    L = _lib.load()
    assert L.gox_topo_repacks(None) == -1
    assert topo.repacks() == 0
    for on in (False, True):  # True, the default, last
        S.set_repack(on)
    assert L.gox_topo_set_split(None, 2) == _lib.GOX_E_INVALID
    assert L.gox_server_submit_many(None, 0, None, None, None, None, None, None, None, None,
                                    None) == _lib.GOX_E_INVALID
