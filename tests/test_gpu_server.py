"""GPU: the serving loop (gox_server_*).  Requests arrive one scenario at a
time (Poisson arrivals from a client thread) over three topologies, some
with an N-1 outage; the workers batch them per topology, with or without
an HBM budget (the buffers held then stay within it), with one or several
server lanes per topology (clones solving batches of one topology at the
same time).  Every report must equal, bit for bit, a direct batched solve
of the same scenario on the same topology (scenarios are independent, so
neither the batch nor the clone a request ran on changes its result), and
carry a positive latency."""
import threading
import time

import numpy as np
import pytest

from gridoxide_gb300 import grids as G
from helpers import grid_from_fixture, load_fixture, ybus_from_fixture

pytestmark = pytest.mark.gpu


def _grids():
    fx = load_fixture("case118")
    g1, y1 = grid_from_fixture(fx), ybus_from_fixture(fx)
    g2 = G.make_grid(300, 45, 420, seed=31)
    g3 = G.make_grid(600, 90, 840, seed=32, load_scale=0.5)
    return [(g1, y1), (g2, G.build_ybus(g2)), (g3, G.build_ybus(g3))]


# 2 MB is below one group of 32 scenarios of the two larger grids: such a
# batch waits until no other topology holds buffers, then runs alone
@pytest.mark.parametrize("precision,budget,lanes", [(0, 0, 2), (1, 0, 1), (1, 0, 4),
                                                    (1, 16 << 20, 2), (1, 2 << 20, 2)])
def test_server_reports_equal_direct_solves(gox, precision, budget, lanes):
    grids = _grids()
    topos = [gox.Topology(yb, g.bus_type) for g, yb in grids]
    rng = np.random.default_rng(40)
    reqs = []  # (topo id, p, q, outage or None)
    for i in range(150):
        t = int(rng.integers(0, 3))
        g, yb = grids[t]
        p, q = G.load_scenarios(g, 1, 0.1, 1000 + i)
        out = None
        if rng.random() < 0.1:
            br = rng.choice(np.flatnonzero(~G.bridges(g)), size=1)
            out = tuple(a[0] for a in G.outage_deltas(g, yb, br))
        reqs.append((t, p[0], q[0], out))
    # (batches of at most 8 with several lanes: a topology's queued requests
    # then take several batches, which run on its clones at the same time)
    srv = gox.Server(max_batch=64 if lanes == 1 or budget else 8, precision=precision)
    ids = [srv.add_topology(tp) for tp in topos]
    if budget:
        srv.set_budget(budget)
    srv.set_lanes(lanes)
    if lanes > 1:  # each topology's first batch fixes its pivot order and plan
        for t, (g, _) in enumerate(grids):
            srv.wait(srv.submit(ids[t], g.p_spec, g.q_spec, g.vm, g.va), g.n_bus)
    tickets = [None] * len(reqs)

    def client():
        for i, (t, p, q, out) in enumerate(reqs):
            g = grids[t][0]
            tickets[i] = srv.submit(ids[t], p, q, g.vm, g.va, outage=out)
            time.sleep(rng.exponential(2e-4))

    th = threading.Thread(target=client)
    th.start()
    th.join()
    reports = [srv.wait(tickets[i], grids[reqs[i][0]][0].n_bus) for i in range(len(reqs))]
    st = srv.stats()
    srv.close()
    warm = 3 if lanes > 1 else 0
    assert st["solved"] == len(reqs) + warm and st["queued"] == 0 and st["batches"] >= 3
    if budget >= 16 << 20:  # admitted batches kept the topologies' buffers within the budget
        assert 0 < st["peak_reserved_bytes"] <= budget
    if budget:  # one lane per topology under a budget
        assert st["clones"] == 0
    elif lanes == 1:
        assert st["clones"] == 0
    else:  # requests arriving while a topology's batch runs start on a clone
        assert 1 <= st["clones"] <= 3 * (lanes - 1)
    lat = np.array([r["latency_s"] for r in reports])
    assert np.all(lat > 0)
    # the same scenarios solved directly on the same topologies
    for t in range(3):
        idx = [i for i, r in enumerate(reqs) if r[0] == t]
        g = grids[t][0]
        p = np.stack([reqs[i][1] for i in idx])
        q = np.stack([reqs[i][2] for i in idx])
        has = [reqs[i][3] is not None for i in idx]
        out = None
        if any(has):
            sl = np.full((len(idx), 4), -1, np.int32)
            dr = np.zeros((len(idx), 4))
            di = np.zeros((len(idx), 4))
            for r, i in enumerate(idx):
                if reqs[i][3] is not None:
                    sl[r], dr[r], di[r] = reqs[i][3]
            out = (sl, dr, di)
        res = topos[t].solve(p, q, g.vm, g.va, precision=precision, outage=out)
        for r, i in enumerate(idx):
            np.testing.assert_array_equal(reports[i]["vm"], res.voltage_mag[r])
            np.testing.assert_array_equal(reports[i]["va"], res.voltage_ang[r])
            np.testing.assert_array_equal(
                [reports[i]["iterations"], reports[i]["status"], reports[i]["max_mismatch"]],
                [res.iterations[r], res.status[r], res.max_mismatch[r]])


def test_server_rejects_bad_requests(gox):
    g, yb = _grids()[0]
    srv = gox.Server(max_batch=8)
    tid = srv.add_topology(gox.Topology(yb, g.bus_type))
    with pytest.raises(ValueError):
        srv.submit(tid, g.p_spec[:-1], g.q_spec, g.vm, g.va)
    with pytest.raises(Exception):
        srv.submit(tid + 5, g.p_spec, g.q_spec, g.vm, g.va)
    t = srv.submit(tid, g.p_spec, g.q_spec, g.vm, g.va)
    r = srv.wait(t, g.n_bus)
    assert r["status"] == gox.GOX_CONVERGED
    with pytest.raises(Exception):
        srv.poll(t, g.n_bus)  # a retired ticket
    for bad in (0, 9):
        with pytest.raises(Exception):
            srv.set_lanes(bad)
    srv.close()


def test_submit_many_equals_single_submits(gox):
    """Requests queued in one call (gox_server_submit_many) report what the
    same requests queued one by one report, bit for bit; a batch with an
    unknown topology id queues nothing."""
    grids = _grids()
    topos = [gox.Topology(yb, g.bus_type) for g, yb in grids]
    rng = np.random.default_rng(41)
    reqs = []
    for i in range(40):
        t = int(rng.integers(0, 3))
        g, yb = grids[t]
        p, q = G.load_scenarios(g, 1, 0.1, 2000 + i)
        out = None
        if i % 5 == 0:
            br = rng.choice(np.flatnonzero(~G.bridges(g)), size=1)
            sl, dr, di = G.outage_deltas(g, yb, br)
            out = (np.ascontiguousarray(sl[0], np.int32), np.ascontiguousarray(dr[0]),
                   np.ascontiguousarray(di[0]))
        reqs.append((t, np.ascontiguousarray(p[0]), np.ascontiguousarray(q[0]), out))
    reports = {}
    for mode in ("single", "many"):
        srv = gox.Server(max_batch=16)
        ids = [srv.add_topology(tp) for tp in topos]
        if mode == "single":
            tk = [srv.submit(ids[t], p, q, grids[t][0].vm, grids[t][0].va, outage=o)
                  for t, p, q, o in reqs]
        else:
            vms = [np.ascontiguousarray(g.vm) for g, _ in grids]
            vas = [np.ascontiguousarray(g.va) for g, _ in grids]
            addr = lambda a: a.ctypes.data
            with pytest.raises(ValueError):
                srv.submit_many([0, 7], [addr(reqs[0][1])] * 2, [addr(reqs[0][2])] * 2,
                                [addr(vms[0])] * 2, [addr(vas[0])] * 2)
            assert srv.stats()["queued"] == 0
            tk = srv.submit_many(
                [ids[t] for t, _, _, _ in reqs], [addr(p) for _, p, _, _ in reqs],
                [addr(q) for _, _, q, _ in reqs], [addr(vms[t]) for t, _, _, _ in reqs],
                [addr(vas[t]) for t, _, _, _ in reqs],
                out_ptrs=[[addr(o[c]) if o is not None else 0 for _, _, _, o in reqs]
                          for c in range(3)])
        reports[mode] = [srv.wait(int(k), grids[reqs[i][0]][0].n_bus) for i, k in enumerate(tk)]
        srv.close()
    for a, b in zip(reports["single"], reports["many"]):
        np.testing.assert_array_equal(a["vm"], b["vm"])
        np.testing.assert_array_equal(a["va"], b["va"])
        assert (a["iterations"], a["status"], a["max_mismatch"]) == \
            (b["iterations"], b["status"], b["max_mismatch"])
    assert any(b["status"] == gox.GOX_CONVERGED for b in reports["many"])
