"""GPU: outage scenarios that split the grid.  A bridge outage leaves a
component without a slack bus; the batched solve pins it to V = 0 with no
injection (mark_unreferenced_islands, src/network.rs:196-223) and solves
the energized part, so every scenario converges.  FP64: same iterations and
status as the oracle on the marked network with the same outage, |V| and
theta within 1e-9; non-splitting scenarios of the same batch are unchanged
by the split (equal to solving them alone); mixed precision converges to
within 1e-7 of FP64.  Also through the device entry and with the linear
guess."""
import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, oracle_topology, ybus_from_fixture

pytestmark = pytest.mark.gpu


def _case(B, seed):
    fx = load_fixture("case118")
    g, yb = grid_from_fixture(fx), ybus_from_fixture(fx)
    rng = np.random.default_rng(seed)
    bridge = np.flatnonzero(G.bridges(g))
    other = np.flatnonzero(~G.bridges(g))
    br = np.where(rng.random(B) < 0.4, rng.choice(bridge, B), rng.choice(other, B))
    out = G.outage_deltas(g, yb, br)
    p, q = G.load_scenarios(g, B, 0.1, seed + 1)
    return g, yb, out, p, q


def _oracle(O, g, yb, out, p, q, ver, guess=False):
    B = p.shape[0]
    vm = np.zeros((B, g.n_bus)); va = np.zeros((B, g.n_bus))
    it = np.zeros(B, np.int32); st = np.zeros(B, np.int32)
    for s in range(B):
        pin = ver[s] == 1
        types = np.where(pin, G.BUS_SLACK, g.bus_type).astype(np.int32)
        ps, qs = np.where(pin, 0.0, p[s]), np.where(pin, 0.0, q[s])
        v0, a0 = np.where(pin, 0.0, g.vm), np.where(pin, 0.0, g.va)
        o1 = (out[0][s:s + 1], out[1][s:s + 1], out[2][s:s + 1])
        if guess:
            re, im = yb.re.copy(), yb.im.copy()
            for c in range(4):
                re[o1[0][0][c]] += o1[1][0][c]
                im[o1[0][0][c]] += o1[2][0][c]
            import dataclasses
            ys = dataclasses.replace(yb, re=re, im=im)
            v0, a0 = O.linear_initial_guess(ys, types, ps, qs, v0, a0)
        ot = oracle_topology(O, yb, types)
        r = ot.batch_solve(ps[None], qs[None], v0, a0, tol=1e-8, max_iter=20, outage=o1)
        vm[s], va[s], it[s], st[s] = r["vm"][0], r["va"][0], r["iters"][0], r["status"][0]
    return vm, va, it, st


def test_bridge_outages_fp64_matches_oracle(gox, oracle_mod):
    g, yb, out, p, q = _case(48, 11)
    topo = gox.Topology(yb, g.bus_type)
    nis, lab, ver = topo.outage_islands(out)
    split = nis > 1
    assert 8 < split.sum() < 40
    res = topo.solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_FP64, outage=out)
    vm, va, it, st = _oracle(oracle_mod, g, yb, out, p, q, ver)
    np.testing.assert_array_equal(res.status, st)
    assert np.all(res.status == gox.GOX_CONVERGED)
    np.testing.assert_array_equal(res.iterations, it)
    assert np.max(np.abs(res.voltage_mag - vm)) < 1e-9
    assert np.max(np.abs(res.voltage_ang - va)) < 1e-9
    assert np.all(res.voltage_mag[ver == 1] == 0.0)
    # the non-splitting scenarios alone give the same results
    keep = np.flatnonzero(~split)
    alone = gox.Topology(yb, g.bus_type).solve(
        p[keep], q[keep], g.vm, g.va, precision=gox.GOX_PRECISION_FP64,
        outage=(out[0][keep], out[1][keep], out[2][keep]))
    np.testing.assert_array_equal(alone.voltage_mag, res.voltage_mag[keep])
    mixed = gox.Topology(yb, g.bus_type).solve(p, q, g.vm, g.va, precision=gox.GOX_PRECISION_MIXED,
                                              outage=out)
    assert np.all(mixed.status == gox.GOX_CONVERGED)
    assert np.max(np.abs(mixed.voltage_mag - res.voltage_mag)) < 1e-7


def test_bridge_outages_device_entry_and_guess(gox, oracle_mod):
    torch = pytest.importorskip("torch")
    g, yb, out, p, q = _case(40, 21)
    topo = gox.Topology(yb, g.bus_type)
    topo.set_initial_guess("linear")
    _, _, ver = topo.outage_islands(out)
    d = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    B, n = p.shape
    vm_o = torch.empty((B, n), dtype=torch.float64, device="cuda")
    va_o = torch.empty_like(vm_o)
    it_o = torch.empty(B, dtype=torch.int32, device="cuda")
    st_o = torch.empty_like(it_o)
    mm_o = torch.empty(B, dtype=torch.float64, device="cuda")
    topo.solve_device(d(p), d(q), d(g.vm), d(g.va), vm_o, va_o, it_o, st_o, mm_o,
                      precision=gox.GOX_PRECISION_FP64,
                      outage=(d(out[0], torch.int32), d(out[1]), d(out[2])))
    torch.cuda.synchronize()
    vm, va, it, st = _oracle(oracle_mod, g, yb, out, p, q, ver, guess=True)
    np.testing.assert_array_equal(st_o.cpu().numpy(), st)
    np.testing.assert_array_equal(it_o.cpu().numpy(), it)
    assert np.max(np.abs(vm_o.cpu().numpy() - vm)) < 1e-9
    assert np.max(np.abs(va_o.cpu().numpy() - va)) < 1e-9
