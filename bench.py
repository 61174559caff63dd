"""Benchmark: batched Newton-Raphson power flow on one GB300.

Workload (one "step" = one batched solve): the 2,000-bus synthetic meshed
grid (1 slack, 300 PV, 1,699 PQ, 2,799 branches), 4,096 scenarios with
every bus load x lognormal(0, 0.15) and PV generation rebalanced, flat
start, tol 1e-8 pu, <= 20 iterations.  Headline = the mixed-precision path
(FP32 refactor/solve, FP64 mismatch/update); the plain FP64 GPU path is
timed in the same run.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value` = solves/s with inputs resident in
HBM; `e2e` = the same through the host-buffer C-ABI call (host<->device
copies inside the timed region).  The working set (>1 GB of factors) is far
larger than L2, and L2 is also flushed (256 MB write) between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

# more hardware work queues than the 8 by default, for the legs that solve
# from several host threads at once (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(grid="case2000", scenarios=4096, sigma=0.15, seed=2024, tol=1e-8, max_iter=20)
METRIC = "PF solves/s on 1 GB300 at <=1e-8 pu mismatch, mixed vs FP64; p50/p99 latency"


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        """Starts the sampler and returns once it has printed its first
        sample (its NVML start-up, which can hold the driver for a moment,
        is then over before the timed region begins; at most 10 s)."""
        import select
        self.first = ""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            ready, _, _ = select.select([self.proc.stdout], [], [], 10.0)
            if ready:
                self.first = self.proc.stdout.readline()
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        out = self.first + (out or "")
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(world: int = 1, rank: int = 0):
    """The workload grid and this rank's scenarios.  With `world` ranks the
    job is `world` x the single-GPU batch (weak scaling), drawn as one
    global batch and cut into contiguous shards (replicas.shard_bounds)."""
    from gridoxide_gb300 import grids as G
    from gridoxide_gb300 import replicas
    if WORKLOAD["grid"].startswith("fam"):  # profiling: a family grid of that many buses
        g = G.family_grid(int(WORKLOAD["grid"][3:]), 77)
    else:
        g = G.config_grid(WORKLOAD["grid"])
    yb = G.build_ybus(g)
    total = WORKLOAD["scenarios"] * world
    p, q = G.load_scenarios(g, total, WORKLOAD["sigma"], WORKLOAD["seed"])
    if world == 1:
        return g, yb, p, q
    lo, hi = replicas.shard_bounds(total, world, rank)
    make_inputs.global_batch = (p, q)
    return g, yb, p[lo:hi].copy(), q[lo:hi].copy()


def workload_config(world: int = 1) -> dict:
    """The `config` of both arms' JSON lines: the workload and the two value
    scales of the generated grid (its loads and resistances; the pattern is
    the literal one)."""
    from gridoxide_gb300 import grids as G
    n, npv, nbr, gseed, ls, rs = G.CONFIGS[WORKLOAD["grid"]]
    return {"workload": f"{WORKLOAD['grid']} x {WORKLOAD['scenarios']} scenarios per GPU, "
                        f"lognormal(0,{WORKLOAD['sigma']}) loads, flat start, tol "
                        f"{WORKLOAD['tol']:g} pu, mixed precision (FP64 timed beside it)",
            "buses": n, "pv": npv, "branches": nbr, "grid_seed": gseed,
            "load_scale": ls, "r_scale": rs,
            "l2": "inputs > L2 and 256 MB flush per step",
            "parallelism": f"replicas x{world} (scenario shards)", **WORKLOAD}


def physical_cores() -> int:
    """Physical cores (not SMT siblings), counted as the reference's
    scripts/bench/bench_batch.py:37-59 does, from the sysfs topology first
    (Arm hosts list no `core id` in /proc/cpuinfo)."""
    ids = set()
    base = "/sys/devices/system/cpu"
    try:
        for d in os.listdir(base):
            if not (d.startswith("cpu") and d[3:].isdigit()):
                continue
            t = os.path.join(base, d, "topology")
            with open(os.path.join(t, "core_id")) as fh:
                core = fh.read().strip()
            with open(os.path.join(t, "physical_package_id")) as fh:
                pkg = fh.read().strip()
            ids.add((pkg, core))
    except OSError:
        ids = set()
    if ids:
        return len(ids)
    try:
        core, pkg = None, None
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.startswith("core id"):
                    core = line.split(":")[1].strip()
                elif line.startswith("physical id"):
                    pkg = line.split(":")[1].strip()
                elif not line.strip() and core is not None:
                    ids.add((pkg, core))
                    core, pkg = None, None
        if core is not None:
            ids.add((pkg, core))
    except OSError:
        pass
    return len(ids) or (os.cpu_count() or 1)


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def algorithmic_bytes(info: dict, n_bus: int, w: int) -> dict:
    """Compulsory HBM bytes per scenario-iteration for each kernel."""
    N, nU, nJ = n_bus, info["n_u"], info["nnz_j"]
    nLU = info["nnz_l"] + info["nnz_u"] + info["n_u"]
    return {
        "mismatch": 16 * N + 16 * N + 8 * nU,
        "fill": 16 * N + 16 * N + w * nJ,
        "refactor": w * nJ + w * nLU,
        "solve": w * nLU + 8 * nU + w * nU,
    }


def read_traffic(kernel: str):
    """DRAM bytes per scenario of one launch of `kernel`, from the committed
    ncu summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_per_scenario.txt")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        for line in fh:
            f = line.split()
            if len(f) >= 2 and f[0] == kernel:
                try:
                    return float(f[1])
                except ValueError:
                    return None
    return None


def serve(gox, rates, seconds: float) -> dict:
    """Serving leg: single-scenario requests arrive as a Poisson process at
    each rate of `rates` per second for `seconds` over 16 family grids of
    100-50,000 buses (log-uniform sizes, each request's grid uniform at
    random), loads x lognormal(0, 0.1), 10 % of the requests with one
    non-bridge branch out, warm started from the grid's base-case solution,
    queued by one front-end thread that submits every due request in one
    gox_server_submit_many call, through the library's serving loop
    (continuous batching on worker threads, mixed precision, host buffers).
    Latency = the request's due time to its completion (the front end's
    delay included; `*_from_submit` without it).  The rates run in increasing order until one
    saturates: fewer than 0.95 x offered requests per second completed while
    requests were arriving (`completed_in_window_rps`; a server that keeps up
    leaves only the requests of its last latency in flight, one that does not
    a growing queue), or the front end could not submit 0.95 x offered
    (`client_limited`: the server kept up with what arrived, and the sweep
    cannot offer more).  `completed_rps` divides by the time until the last
    completion instead (the window plus `drain_ms`, which is the latency of
    the slowest grids' last batches); `submitted_rps` is the rate the client
    thread actually reached.  That rate and every one before it are in
    `sweep`, with p50 and p99 latency by grid size; `saturation_rps` is the
    highest offered rate the server kept up with, `max_completed_in_window_rps`
    the most requests per second it completed in a window.  Each grid's requests draw their load vectors
    from 32 seeded samples of the grid's distribution (the per-request host
    copies are the grid's size whatever the sample)."""
    from gridoxide_gb300 import grids as G
    import gc
    # the earlier legs' pinned host buffers are freed now, not by a later
    # collection inside a window (freeing pinned memory synchronizes the GPU)
    gc.collect()
    spec = G.many_topologies(count=16, n_min=100, n_max=50000, seed=5)
    grids, topos, cand, v0 = [], [], [], []
    for (n, gs, _b, _ss) in spec:
        g = G.family_grid(n, gs)
        yb = G.build_ybus(g)
        grids.append((g, yb))
        topo = gox.Topology(yb, g.bus_type)
        base = topo.solve(g.p_spec[None, :], g.q_spec[None, :], g.vm, g.va,
                          precision=gox.GOX_PRECISION_FP64)
        v0.append((base.voltage_mag[0].copy(), base.voltage_ang[0].copy()))
        topos.append(topo)
        cand.append(np.flatnonzero(~G.bridges(g)))
    sizes = np.array([x[0] for x in spec])
    bins = [("<1k", sizes < 1000), ("1k-10k", (sizes >= 1000) & (sizes < 10000)),
            (">=10k", sizes >= 10000)]
    loads = [G.load_scenarios(g, 32, 0.1, 5000 + t) for t, (g, _) in enumerate(grids)]
    sweep = []
    saturation = None
    for k, rate in enumerate(rates):
        srv = gox.Server(max_batch=1024, precision=gox.GOX_PRECISION_MIXED,
                         tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"])
        ids = [srv.add_topology(t) for t in topos]
        rng = np.random.default_rng(7 + k)
        n_req = max(1, int(rate * seconds))
        gaps = rng.exponential(1.0 / rate, size=n_req)
        which = rng.integers(0, len(spec), size=n_req)
        pick = rng.integers(0, 32, size=n_req)
        reqs = []
        for i in range(n_req):
            t = int(which[i])
            g, yb = grids[t]
            p, q = loads[t][0][pick[i]], loads[t][1][pick[i]]
            out = None
            if rng.random() < 0.1:
                br = rng.choice(cand[t], size=1)
                out = tuple(a[0] for a in G.outage_deltas(g, yb, br))
            reqs.append((t, p, q, out))
        # warm-up: one request per grid (first-use allocations, pivot orders)
        for t in range(len(spec)):
            g = grids[t][0]
            srv.wait(srv.submit(ids[t], g.p_spec, g.q_spec, *v0[t]), g.n_bus)
        st0 = srv.stats()
        # the arrival schedule, drained by one front-end thread: it queues
        # every request that is due in one gox_server_submit_many call (up to
        # 512), and a request's latency counts from its due time, so the
        # front end's delay is included
        due_at = np.cumsum(gaps)

        def addr(a):
            return a.ctypes.data
        tid = np.array([ids[r[0]] for r in reqs], np.int32)
        pa = np.array([addr(r[1]) for r in reqs], np.uint64)
        qa = np.array([addr(r[2]) for r in reqs], np.uint64)
        vma = np.array([addr(v0[r[0]][0]) for r in reqs], np.uint64)
        vaa = np.array([addr(v0[r[0]][1]) for r in reqs], np.uint64)
        oa = [np.array([addr(r[3][c]) if r[3] is not None else 0 for r in reqs], np.uint64)
              for c in range(3)]
        tickets = np.zeros(n_req, np.int64)
        call_t = np.zeros(n_req)
        t0 = time.perf_counter()
        due = t0 + due_at
        k = 0
        while k < n_req:
            e = min(int(np.searchsorted(due, time.perf_counter(), side="right")), k + 512)
            if e <= k:
                continue
            tc = time.perf_counter()
            tickets[k:e] = srv.submit_many(tid[k:e], pa[k:e], qa[k:e], vma[k:e], vaa[k:e],
                                           out_ptrs=[o[k:e] for o in oa])
            call_t[k:e] = tc
            k = e
        t_last = float(call_t.max())
        lat_sub, conv = [], 0
        for (t, _, _, _), tk in zip(reqs, tickets):
            r = srv.wait(int(tk), grids[t][0].n_bus)
            lat_sub.append(r["latency_s"])
            conv += int(r["status"] == 0 and r["max_mismatch"] < WORKLOAD["tol"])
        t1 = time.perf_counter()
        st = srv.stats()
        srv.close()
        lat_sub = np.array(lat_sub) * 1000.0
        lag = (call_t - due) * 1000.0
        lat = lag + lat_sub  # from the request's due time
        nb = st["batches"] - st0["batches"]
        grid_of = np.array([r[0] for r in reqs])
        by_size, by_size99 = {}, {}
        for name, sel in bins:
            m = np.isin(grid_of, np.flatnonzero(sel))
            if m.any():
                by_size[name] = round(float(np.percentile(lat[m], 50)), 3)
                by_size99[name] = round(float(np.percentile(lat[m], 99)), 3)
        dq = (st["queue_us"] - st0["queue_us"]) / 1000.0 / n_req
        ds = (st["solve_us"] - st0["solve_us"]) / 1000.0 / n_req
        done_rps = n_req / (t1 - t0)
        # completions while requests were arriving, per second of arrivals
        finished = call_t + lat_sub / 1000.0
        steady_rps = float(np.sum(finished <= t_last)) / max(t_last - t0, 1e-9)
        sweep.append({"offered_rps": rate, "requests": n_req,
                      "submitted_rps": round(n_req / max(t_last - t0, 1e-9), 1),
                      "mean_queued_ms": round(dq, 3), "mean_in_solve_ms": round(ds, 3),
                      "completed_rps": round(done_rps, 1),
                      "completed_in_window_rps": round(steady_rps, 1),
                      "drain_ms": round(1000.0 * (t1 - t_last), 1),
                      "p50_ms": round(float(np.percentile(lat, 50)), 3),
                      "p99_ms": round(float(np.percentile(lat, 99)), 3),
                      "p50_ms_from_submit": round(float(np.percentile(lat_sub, 50)), 3),
                      "p99_ms_from_submit": round(float(np.percentile(lat_sub, 99)), 3),
                      "mean_front_end_delay_ms": round(float(lag.mean()), 3), "batches": nb,
                      "mean_batch": round(n_req / max(nb, 1), 1), "converged": conv,
                      "p50_ms_by_buses": by_size, "p99_ms_by_buses": by_size99})
        # the server kept up when it completed 0.95 of what arrived; the
        # rate counts only when the client also offered 0.95 of it
        submitted = n_req / max(t_last - t0, 1e-9)
        client_limited = submitted < 0.95 * rate
        sweep[-1]["client_limited"] = client_limited
        if steady_rps < 0.95 * submitted:
            break
        if client_limited:
            break
        saturation = rate
    out = dict(sweep[-1])
    out.update({"sweep": sweep, "grids": len(spec), "saturation_rps": saturation,
                "max_completed_in_window_rps": max(w["completed_in_window_rps"] for w in sweep),
                "buses": [int(sizes.min()), int(sizes.max())],
                "note": "Poisson arrivals of single scenarios over 16 grids (100-50,000 buses), 10 % "
                        "with an N-1 outage, queued by one front-end thread (every due request "
                        "in one gox_server_submit_many call; latency from the due time), "
                        "gox_server_* continuous batching on 16 workers, mixed precision, host "
                        "buffers, warm start from each grid's base case"})
    return out


def n1_case10000(gox, rounds: int, batch: int = 8192) -> dict:
    """N-1 leg: the 10,000-bus grid, `batch` scenarios, each with one
    non-bridge branch out (4-slot Y delta) and loads x lognormal(0, 0.15),
    warm started from the base case's solution, mixed precision with the
    pivot-ratio check (a trip re-solves that scenario in FP64); host buffers,
    inputs and results in pinned memory allocated once and reused every
    round (as the e2e leg and a serving caller do), so the time holds the
    copies but not the host's page faults on fresh result arrays.  Beside
    it (`device`) the same batch with inputs and results in device memory:
    the round trip of 2.6 GB through the host follows the shared host's
    memory traffic, this one does not; its results must equal the
    host-buffer ones bit for bit.  Both re-pack the stragglers."""
    import torch
    from gridoxide_gb300 import grids as G
    g = G.config_grid("case10000")
    yb = G.build_ybus(g)
    topo = gox.Topology(yb, g.bus_type)
    base = topo.solve(g.p_spec[None, :], g.q_spec[None, :], g.vm, g.va,
                      precision=gox.GOX_PRECISION_FP64)
    vm0, va0 = base.voltage_mag[0], base.voltage_ang[0]
    p, q = G.load_scenarios(g, batch, 0.15, 2025)
    p = torch.from_numpy(p).pin_memory().numpy()
    q = torch.from_numpy(q).pin_memory().numpy()
    rng = np.random.default_rng(2026)
    br = rng.choice(np.flatnonzero(~G.bridges(g)), size=batch, replace=True)
    out = G.outage_deltas(g, yb, br)
    n = g.n_bus

    def _pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()
    res_buf = gox.BatchResult(_pinned((batch, n), torch.float64),
                              _pinned((batch, n), torch.float64),
                              _pinned((batch,), torch.int32), _pinned((batch,), torch.int32),
                              _pinned((batch,), torch.float64))

    def one():
        return topo.solve(p, q, vm0, va0, tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"],
                          precision=gox.GOX_PRECISION_MIXED, outage=out, out=res_buf)

    res = one()  # warm-up
    times = []
    for _ in range(rounds):
        t0 = time.perf_counter()
        res = one()
        times.append(time.perf_counter() - t0)
    t = float(np.median(times))
    # the same batch device-resident
    dev = torch.device("cuda", torch.cuda.current_device())

    def _dev(a, dt=torch.float64):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    tp, tq, tvm0, tva0 = _dev(p), _dev(q), _dev(vm0), _dev(va0)
    tout = (_dev(out[0], torch.int32), _dev(out[1]), _dev(out[2]))
    ovm = torch.empty((batch, n), dtype=torch.float64, device=dev)
    ova = torch.empty_like(ovm)
    oit = torch.empty(batch, dtype=torch.int32, device=dev)
    ost = torch.empty_like(oit)
    omm = torch.empty(batch, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def dev_step():
        topo.solve_device(tp, tq, tvm0, tva0, ovm, ova, oit, ost, omm, tol=WORKLOAD["tol"],
                          max_iter=WORKLOAD["max_iter"], precision=gox.GOX_PRECISION_MIXED,
                          outage=tout, stream=stream)
    dev_step()
    torch.cuda.synchronize()
    dms = []
    for _ in range(rounds):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dev_step()
        e1.record(stream)
        e1.synchronize()
        dms.append(e0.elapsed_time(e1))
    same = bool(np.array_equal(ovm.cpu().numpy(), res.voltage_mag) and
                np.array_equal(oit.cpu().numpy(), res.iterations))
    td = float(np.median(dms)) / 1000.0
    del tp, tq, tout, ovm, ova
    return {"value": round(batch / t, 1), "unit": "solves/s", "scenarios": batch,
            "ms_per_step": round(1000 * t, 2),
            "device": {"value": round(batch / td, 1), "unit": "solves/s",
                       "ms_per_step": round(1000 * td, 2), "equal_to_host_buffers_bitwise": same,
                       "repacks": int(topo.repacks())},
            "converged": int(np.sum(res.status == 0)),
            "max_mismatch_converged": float(np.max(res.max_mismatch[res.status == 0])),
            "iterations_hist": np.bincount(res.iterations).tolist(),
            "fp64_fallbacks": int(topo.last_fallbacks()), "rounds": rounds,
            "note": "case10000, one non-bridge branch out per scenario, warm start from the base "
                    "case, mixed precision, host buffers (H2D/D2H inside the time; inputs and "
                    "results in pinned memory reused every round)"}


def many_topologies(gox, rounds: int) -> dict:
    """Many-topology leg: 48 family grids (log-uniform 30-20,000 buses), a
    batch of 8-1,024 scenarios each (loads x lognormal(0, 0.15), flat
    start); a round solves every grid's batch once; host buffers, mixed
    precision.  `value`: the round as one gox_multi_solve call in its
    default form (one Newton loop, each phase one launch over every grid
    still running); beside it the same round in the call's other form
    (`one_launch`: one persistent launch whose CTAs run whole Newton loops of
    (grid, group of 32) items from a device queue) and as 48 independent
    solves issued from 8 host threads (`threads`: each its own Newton loop
    and stream).  Every form
    reads its inputs from, and writes its results to, pinned host memory
    allocated once and reused every round (as a serving caller would), each
    form its own result buffers; the one-call forms' results must equal the
    threads' bit for bit."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    from gridoxide_gb300 import grids as G

    def _pin(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    def _pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    def _results():
        return [gox.BatchResult(_pinned(p.shape, torch.float64), _pinned(p.shape, torch.float64),
                                _pinned((p.shape[0],), torch.int32),
                                _pinned((p.shape[0],), torch.int32),
                                _pinned((p.shape[0],), torch.float64))
                for (_t, _g, p, _q) in jobs]
    spec = G.many_topologies()
    jobs = []
    for (n, gs, b, ss) in spec:
        g = G.family_grid(n, gs)
        topo = gox.Topology(G.build_ybus(g), g.bus_type)
        p, q = G.load_scenarios(g, b, 0.15, ss)
        jobs.append((topo, g, _pin(p), _pin(q)))
    res_t = _results()

    def one(k):
        topo, g, p, q = jobs[k]
        return topo.solve(p, q, g.vm, g.va, tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"],
                          precision=gox.GOX_PRECISION_MIXED, out=res_t[k])

    # warm-up: each grid alone first (pivot orders, allocations, and the
    # autotuner timing its candidates on an otherwise idle GPU), then once
    # from the 8 threads
    ks = range(len(jobs))
    res = [one(k) for k in ks]
    ex = ThreadPoolExecutor(max_workers=8)
    res = list(ex.map(one, ks))
    times = []
    for _ in range(rounds):
        t0 = time.perf_counter()
        res = list(ex.map(one, ks))
        times.append(time.perf_counter() - t0)
    ex.shutdown()
    total = sum(x[2] for x in spec)
    conv = sum(int(np.sum(r.status == 0)) for r in res)
    t = float(np.median(times))
    # the same round in one call (gox_multi_solve), in both forms: one Newton
    # loop with one launch per phase over every grid still running, and one
    # persistent launch whose CTAs run whole Newton loops of (grid, group)
    # items from a queue
    from gridoxide_gb300 import solver as S
    mj = [(topo, p, q, g.vm, g.va) for (topo, g, p, q) in jobs]
    kw = dict(tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"], precision=gox.GOX_PRECISION_MIXED)
    forms = {}
    res_m = _results()
    for persistent in (False, True):
        S.set_multi_persistent(persistent)
        mres = gox.multi_solve(mj, out=res_m, **kw)  # warm-up
        mtimes = []
        for _ in range(rounds):
            t0 = time.perf_counter()
            mres = gox.multi_solve(mj, out=res_m, **kw)
            mtimes.append(time.perf_counter() - t0)
        same = all(np.array_equal(a.voltage_mag, b.voltage_mag) and
                   np.array_equal(a.iterations, b.iterations) for a, b in zip(res, mres))
        forms[persistent] = (float(np.median(mtimes)), same)
    S.set_multi_persistent(False)  # the default
    tm = forms[False][0]
    return {"value": round(total / tm, 1), "unit": "solves/s", "grids": len(spec),
            "scenarios_per_round": total, "ms_per_round": round(1000 * tm, 2),
            "buses": [int(min(x[0] for x in spec)), int(max(x[0] for x in spec))],
            "converged": conv, "rounds": rounds,
            "equal_to_threads_bitwise": forms[False][1],
            "threads": {"value": round(total / t, 1), "unit": "solves/s",
                        "ms_per_round": round(1000 * t, 2),
                        "note": "the 48 grids' batches as independent solves issued from 8 host "
                                "threads, each its own Newton loop and stream"},
            "one_launch": {"value": round(total / forms[True][0], 1), "unit": "solves/s",
                           "ms_per_round": round(1000 * forms[True][0], 2),
                           "equal_to_threads_bitwise": forms[True][1],
                           "note": "gox_multi_solve's persistent form: one launch whose CTAs run "
                                   "whole Newton loops of (grid, group of 32) items from a device "
                                   "queue, largest grid first"},
            "note": "one gox_multi_solve call per round, default form: one Newton loop, each "
                    "phase one launch over every grid still running; host buffers (pinned, "
                    "allocated once), mixed precision, flat start"}


def pgm_batch(gox, rounds: int, batch: int = 4096) -> dict:
    """PGM leg, the reference's scripts/bench/bench_batch.py workflow: the
    2,000-bus grid written as a power-grid-model JSON file, loaded with
    PowerFlowModel.from_pgm_json and solved as `batch` uniform load scalings
    U[0.8, 1.2] (solve_batch_scaled: linear guess per scenario, tol 1e-6, 20
    iterations); one warm-up call, then min over `rounds` calls, as that
    script times; per backend ("klu_native" = FP64, "gb300" = mixed)."""
    import random
    import tempfile
    from gridoxide_gb300 import grids as G, pgm
    g = G.config_grid("case2000")
    out = {"grid": "case2000 as PGM JSON (its slack a 10 GVA source)", "scenarios": batch,
           "rounds": rounds}
    rng = random.Random(20260726)
    scales = [rng.uniform(0.8, 1.2) for _ in range(batch)]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "case2000_pgm.json")
        with open(path, "w") as fh:
            json.dump(pgm.from_grid(g), fh)
        for backend in ("klu_native", "gb300"):
            t0 = time.perf_counter()
            m = gox.PowerFlowModel.from_pgm_json(path, backend=backend)
            t_load = time.perf_counter() - t0
            res = m.solve_batch_scaled(scales)  # warm-up: analysis, pivot order, buffers
            times = []
            for _ in range(rounds):
                t0 = time.perf_counter()
                res = m.solve_batch_scaled(scales)
                times.append(time.perf_counter() - t0)
            t = min(times)
            out[backend] = {"value": round(batch / t, 1), "unit": "solves/s",
                            "ms_per_batch": round(1000 * t, 2),
                            "model_load_ms": round(1000 * t_load, 1),
                            "converged": sum(int(r.converged) for r in res),
                            "iterations_hist": np.bincount([r.iterations for r in res]).tolist()}
        out["nodes"] = m.n_nodes
    return out


def qlim_case2000(gox, rounds: int, batch: int = 4096) -> dict:
    """Q-limit leg: case2000 x `batch` (loads x lognormal(0, 0.15), flat
    start), reactive limits on the six PV buses with the largest |Q| at the
    25 % / 75 % quantiles of their unconstrained Q over the batch (floor for
    the three most negative, ceiling for the three most positive), so each
    scenario trips its own subset; gox_batch_solve_qlim, mixed precision,
    host buffers.  The first call builds a topology variant per switched set;
    the timed calls reuse them."""
    from gridoxide_gb300 import grids as G
    g = G.config_grid("case2000")
    yb = G.build_ybus(g)
    p, q = G.load_scenarios(g, batch, WORKLOAD["sigma"], 2031)
    plain = gox.Topology(yb, g.bus_type).solve(p, q, g.vm, g.va, tol=WORKLOAD["tol"],
                                               max_iter=WORKLOAD["max_iter"],
                                               precision=gox.GOX_PRECISION_MIXED)
    # unconstrained Q of the PV buses: Im(V conj(Y V)) per scenario
    n = g.n_bus
    rows = np.repeat(np.arange(n), np.diff(yb.indptr))
    pv = np.flatnonzero(g.bus_type == G.BUS_PV)
    sel = np.isin(rows, pv)
    v = plain.voltage_mag * np.exp(1j * plain.voltage_ang)
    col = {b: k for k, b in enumerate(pv)}
    cur = np.zeros((batch, pv.size), np.complex128)
    yv = (yb.re + 1j * yb.im)[sel]
    for r_, c_, yy in zip(rows[sel], yb.indices[sel], yv):
        cur[:, col[r_]] += yy * v[:, c_]
    qpv = (v[:, pv] * np.conj(cur)).imag
    med = np.median(qpv, axis=0)
    lo, hi = np.argsort(med)[:3], np.argsort(med)[-3:]
    q_min = np.full(n, -np.inf)
    q_max = np.full(n, np.inf)
    q_min[pv[lo]] = np.quantile(qpv[:, lo], 0.25, axis=0)
    q_max[pv[hi]] = np.quantile(qpv[:, hi], 0.75, axis=0)
    topo = gox.Topology(yb, g.bus_type)

    def one():
        return topo.solve_qlim(p, q, g.vm, g.va, q_min, q_max, tol=WORKLOAD["tol"],
                               max_iter=WORKLOAD["max_iter"], max_outer=10,
                               precision=gox.GOX_PRECISION_MIXED)

    t0 = time.perf_counter()
    res, sw, stab = one()  # builds the variants
    t_first = time.perf_counter() - t0
    times = []
    for _ in range(rounds):
        t0 = time.perf_counter()
        res, sw, stab = one()
        times.append(time.perf_counter() - t0)
    t = float(np.median(times))
    return {"value": round(batch / t, 1), "unit": "solves/s", "scenarios": batch,
            "ms_per_step": round(1000 * t, 2), "first_call_ms": round(1000 * t_first, 1),
            "switched_sets": len({tuple(np.flatnonzero(r)) for r in sw}),
            "scenarios_switching": int(sw.any(axis=1).sum()),
            "converged": int(np.sum(res.status == 0)), "stabilized": int(stab.sum()),
            "rounds": rounds,
            "note": "case2000, six PV buses with reactive limits at quantiles of their Q, "
                    "PV->PQ switching per scenario, mixed precision, host buffers"}


_ORACLE_TOPO = {}


def _oracle_topology(g, yb):
    """The oracle port's topology for the workload grid (built once).  Its
    symbolic ordering is the reference's own klu_analyze output for this
    grid, committed as a fixture (tests/golden/); nothing of the product
    library is loaded on this path."""
    key = id(yb)
    if key not in _ORACLE_TOPO:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build(ref=False) if not os.path.exists(O.LIB) else None
        order = O.fixture_ordering(WORKLOAD["grid"], yb, g.bus_type)
        _ORACLE_TOPO[key] = O.Topology(yb, g.bus_type, *order)
    return _ORACLE_TOPO[key]


def cpu_pass(g, yb, p, q, threads: int):
    """One pass of the oracle port (C restatement of BatchSolver + KLU, one
    persistent solver per worker thread) over every scenario of p, q;
    returns (solves/s, seconds, reports)."""
    topo = _oracle_topology(g, yb)
    t0 = time.perf_counter()
    res = topo.batch_solve(p, q, g.vm, g.va, tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"],
                           threads=threads)
    dt = time.perf_counter() - t0
    return p.shape[0] / dt, dt, res


def thread_sweep(g, yb, p, q, per_thread: int = 32, repeats: int = 3) -> dict:
    """The reference's scripts/bench/bench_batch.py method on the oracle
    port: thread counts 1, 2, 4, ... up to the logical cores, each on a
    sample of `per_thread` x threads scenarios (bounded time): one warm-up
    call, then the minimum of `repeats` timed calls; every thread count's
    voltages must equal the 1-thread run's on the shared scenarios."""
    logical = os.cpu_count() or 1
    counts = [t for t in (1, 2, 4, 8, 16, 32, 64, 128) if t <= logical]
    if logical not in counts:
        counts.append(logical)
    out, first = {}, None
    for t in counts:
        n = min(p.shape[0], per_thread * t)
        _, _, res = cpu_pass(g, yb, p[:n], q[:n], t)
        m = per_thread if first is None else min(first.shape[0], n)
        if first is None:
            first = res["vm"][:m].copy()
        else:
            worst = float(np.max(np.abs(res["vm"][:m] - first[:m])))
            assert worst < 1e-12, f"threads={t} disagrees with threads=1 by {worst:.3e}"
        best = min(cpu_pass(g, yb, p[:n], q[:n], t)[1] for _ in range(repeats))
        out[str(t)] = round(n / best, 1)
    return out


def cpu_baseline(g, yb, p, q, threads: int, min_seconds: float = 10.0):
    """The oracle port on the host's cores: passes over the whole workload
    until at least `min_seconds` have run (after one warm-up pass over a
    slice).  Returns (solves/s, seconds, passes, reports of the last pass)."""
    cpu_pass(g, yb, p[:threads * 4], q[:threads * 4], threads)  # warm-up
    n, t, passes, res = 0, 0.0, 0, None
    while t < min_seconds:
        v, dt, res = cpu_pass(g, yb, p, q, threads)
        n += p.shape[0]
        t += dt
        passes += 1
    return n / t, t, passes, res


def error_vs_oracle(vm, va, iters, status, ref) -> dict:
    """max |dV| (pu) and |dtheta| (rad) of a GPU result against the oracle's
    reports of the same scenarios, and how many iteration counts / statuses
    agree."""
    return {"max_abs_dvm": float(np.max(np.abs(vm - ref["vm"]))),
            "max_abs_dva": float(np.max(np.abs(va - ref["va"]))),
            "iterations_equal": int(np.sum(iters == ref["iters"])),
            "status_equal": int(np.sum(status == ref["status"])),
            "scenarios": int(vm.shape[0])}


def run_reference_arm(args):
    """The reference's CPU implementation of the path (the oracle port, all
    host threads): each step is one pass over the whole workload."""
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    g, yb, p, q = make_inputs()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_pass(g, yb, p[:threads * 4], q[:threads * 4], threads)
    vals, secs = [], []
    for _ in range(args.steps):
        v, dt, _ = cpu_pass(g, yb, p, q, threads)
        vals.append(v)
        secs.append(dt)
    value = float(np.median(vals))
    B = p.shape[0]
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000.0 * float(np.median(secs)), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.gpus),
        "cpu_baseline": {"value": round(value, 1), "unit": "solves/s", "cores": threads,
                         "kind": "port", "cpu": cpu_model(), "physical_cores": physical_cores(),
                         "ordering": "the reference's compiled klu_analyze (committed fixture)",
                         "sample": f"the whole {B}-scenario workload per step (one GPU's share), "
                                   f"{threads} threads"},
        "e2e": {"value": round(value, 1), "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-rate", type=float, default=30000.0,
                    help="serving leg: highest Poisson arrival rate of the sweep (0 = skip)")
    ap.add_argument("--many-rounds", type=int, default=3,
                    help="N-1 10,000-bus and many-topology legs: timed rounds (0 = skip)")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--grid", default=WORKLOAD["grid"], help="profiling: another grid")
    ap.add_argument("--scenarios", type=int, default=WORKLOAD["scenarios"],
                    help="profiling: a smaller batch")
    ap.add_argument("--quick", action="store_true",
                    help="profiling: mixed-precision steps only (no FP64, e2e, CPU legs)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="profiling: the default refactor plan, no candidate timing")
    ap.add_argument("--wide", type=int, default=0,
                    help="profiling: the default plan's wide split (narrowest wide level)")
    ap.add_argument("--host-loop", action="store_true",
                    help="profiling: host-driven Newton loop on one host thread (no graph, no "
                         "split parts)")
    args = ap.parse_args()
    WORKLOAD["grid"] = args.grid
    WORKLOAD["scenarios"] = args.scenarios
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch
    import gridoxide_gb300 as gox

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    gox.build.build()
    if args.no_autotune:
        from gridoxide_gb300 import solver as S
        S.set_autotune(False)
        S.set_refactor_wide(args.wide)

    g, yb, p, q = make_inputs(world, rank)
    B, N = p.shape
    topo = gox.Topology(yb, g.bus_type)
    if args.host_loop:
        topo.set_graph(False)
        topo.set_split(1)
    stream = torch.cuda.Stream(device=dev)
    tp = torch.from_numpy(p).to(dev)
    tq = torch.from_numpy(q).to(dev)
    tvm0 = torch.from_numpy(g.vm).to(dev)
    tva0 = torch.from_numpy(g.va).to(dev)
    ovm = torch.empty((B, N), dtype=torch.float64, device=dev)
    ova = torch.empty_like(ovm)
    oit = torch.empty(B, dtype=torch.int32, device=dev)
    ost = torch.empty(B, dtype=torch.int32, device=dev)
    omm = torch.empty(B, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def step(precision):
        topo.solve_device(tp, tq, tvm0, tva0, ovm, ova, oit, ost, omm, tol=WORKLOAD["tol"],
                          max_iter=WORKLOAD["max_iter"], precision=precision, stream=stream)

    def timed(precision, steps, clocks=None, kernel_timing=False):
        """`steps` timed steps.  Without kernel_timing the library runs each
        solve's Newton loop as its captured CUDA graph; with it, the
        host-driven loop records CUDA events around every phase."""
        topo.set_timing(kernel_timing)
        ms, kern, launches = [], {"mismatch": 0.0, "fill": 0.0, "refactor": 0.0, "solve": 0.0}, 0
        iters_run = []
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(precision)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            if kernel_timing:
                t = topo.last_timing()
                kern["mismatch"] += t["mismatch_ms"]
                kern["fill"] += t["fill_ms"]
                kern["refactor"] += t["refactor_ms"]
                kern["solve"] += t["solve_ms"]
                iters_run.append(int(t["iterations"]))
            else:
                iters_run.append(int(oit.max().item()))
            launches += topo.last_launches()
        torch.cuda.synchronize()
        cl = clocks.stop() if clocks else None
        if world > 1:
            torch.distributed.barrier()
        return np.array(ms), kern, launches, iters_run, cl

    # warm-up (pivot orders, plan timing, captured loops), each step after an
    # L2 flush as in the timed loop: FP64 first, so the timed mixed steps
    # follow mixed ones
    if not args.quick:
        for _ in range(args.warmup):
            flush.zero_()
            step(gox.GOX_PRECISION_FP64)
    for _ in range(args.warmup):
        flush.zero_()
        step(gox.GOX_PRECISION_MIXED)
    torch.cuda.synchronize()
    # correctness of the timed configuration
    its = oit.cpu().numpy()
    sts = ost.cpu().numpy()
    mm = omm.cpu().numpy()

    clocks = ClockSampler(local)
    ms_mx, _, launches_mx, iters_mx, cl = timed(gox.GOX_PRECISION_MIXED, args.steps, clocks)
    st_mx = ost.cpu().numpy().copy()
    mm_mx = omm.cpu().numpy().copy()
    it_mx = oit.cpu().numpy().copy()
    vm_mx = ovm.cpu().numpy().copy()
    va_mx = ova.cpu().numpy().copy()
    # the same steps again with CUDA events around every phase (host-driven
    # loop): the per-kernel times and the roofline
    ms_k, kern_mx, _, iters_k, _ = timed(gox.GOX_PRECISION_MIXED, args.steps, kernel_timing=True)
    if args.quick:
        print(json.dumps({"quick": True, "ms_per_step": float(np.mean(ms_mx)),
                          "ms_per_step_events": float(np.mean(ms_k)), "kernels_ms": kern_mx,
                          "iterations": iters_mx, "graph_solves": topo.info()["graph_solves"]}),
              flush=True)
        return
    step(gox.GOX_PRECISION_FP64)  # untimed: the switch back to the FP64 loop
    ms_64, kern_64, launches_64, iters_64, _ = timed(gox.GOX_PRECISION_FP64,
                                                     max(3, args.steps // 2))
    it_64 = oit.cpu().numpy().copy()
    st_64 = ost.cpu().numpy().copy()
    vm_64 = ovm.cpu().numpy().copy()
    va_64 = ova.cpu().numpy().copy()

    from gridoxide_gb300 import replicas
    total_ms = replicas.max_over_ranks(float(ms_mx.sum()))
    value = world * B * args.steps / (total_ms / 1000.0)
    fp64_value = B * len(ms_64) / (ms_64.sum() / 1000.0)

    # e2e through the host-buffer C-ABI call: inputs and result arrays in
    # pinned host memory (allocated once, reused every step, as a serving
    # caller would); H2D of the inputs and D2H of the results every step
    hp = torch.from_numpy(p).pin_memory().numpy()
    hq = torch.from_numpy(q).pin_memory().numpy()

    def _pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()
    res_buf = gox.BatchResult(_pinned((B, N), torch.float64), _pinned((B, N), torch.float64),
                              _pinned((B,), torch.int32), _pinned((B,), torch.int32),
                              _pinned((B,), torch.float64))
    e2e_ms = []
    for k in range(max(3, args.steps // 2)):
        if world > 1:
            # the replicas path: every rank solves its shard of the global
            # batch and the reports are gathered on the host
            pg, qg = make_inputs.global_batch
            torch.distributed.barrier()
            t0 = time.perf_counter()
            rep = replicas.solve_replicas(
                replicas.topology_solver(topo, gox.GOX_PRECISION_MIXED), pg, qg, g.vm, g.va,
                tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"])
            e2e_ms.append(replicas.max_over_ranks(1000.0 * (time.perf_counter() - t0)))
            assert int(np.sum(rep["status"] == 0)) == world * B
            continue
        t0 = time.perf_counter()
        topo.solve(hp, hq, g.vm, g.va, tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"],
                   precision=gox.GOX_PRECISION_MIXED, out=res_buf)
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    if world == 1:
        assert int(np.sum(res_buf.status == 0)) == B
    e2e_value = world * B / (np.median(e2e_ms) / 1000.0)
    h2d = 2 * B * N * 8 + 2 * N * 8
    d2h = 2 * B * N * 8 + B * (4 + 4 + 8)

    # roofline of the dominant kernel (mixed path).  When the refactor's
    # command streams also run the backward substitution there is no solve
    # launch: the refactor kernel does both, and its bytes are both kernels'.
    info = topo.info()
    abytes = algorithmic_bytes(info, N, 4)
    if info.get("rf32_with_bwd"):
        abytes["refactor"] += abytes.pop("solve")
        kern_mx["refactor"] += kern_mx.pop("solve")
    dom = max(kern_mx, key=lambda k: kern_mx[k])
    n_launch = sum(iters_k) if dom != "mismatch" else sum(iters_k) + args.steps
    per_launch_bytes = abytes[dom] * B
    avg_launch_ms = kern_mx[dom] / max(n_launch, 1)
    achieved = per_launch_bytes / (avg_launch_ms / 1000.0) / 1e9
    peak, peak_kind = _peaks()
    traffic = read_traffic(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
            "traffic": None if traffic is None else traffic * B,
            "algorithmic_bytes_per_launch": per_launch_bytes,
            "avg_launch_ms": round(avg_launch_ms, 4)}
    kernels = {}
    for k in kern_mx:
        nl = sum(iters_k) + (args.steps if k == "mismatch" else 0)
        t_ms = kern_mx[k] / max(nl, 1)
        kernels[k] = {"ms_per_launch": round(t_ms, 4),
                      "GB/s": round(abytes[k] * B / (t_ms / 1000.0) / 1e9, 1) if t_ms > 0 else None,
                      "share": round(kern_mx[k] / max(sum(kern_mx.values()), 1e-9), 3)}

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(float(np.mean(ms_mx)), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 LU/solve + f64 mismatch",
        "data": "synthetic",
        "config": workload_config(world),
        "latency_ms": {"p50": round(float(np.percentile(ms_mx, 50)), 4),
                       "p99": round(float(np.percentile(ms_mx, 99)), 4)},
        "fp64": {"value": round(fp64_value, 1), "unit": "solves/s",
                 "ms_per_step": round(float(np.mean(ms_64)), 4),
                 "iterations_hist": np.bincount(it_64).tolist()},
        "mixed_over_fp64": round(value / world / fp64_value, 3),
        "iterations_hist": np.bincount(it_mx).tolist(),
        "converged": int(np.sum(st_mx == 0)), "max_mismatch": float(mm_mx.max()),
        "e2e": {"value": round(e2e_value, 1), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches_mx),
        "newton_loop": {"graph_solves": int(topo.info()["graph_solves"]),
                        "kernel_timing": "kernels and roofline from a second pass of the same "
                                         "steps with CUDA events around every phase (host-driven "
                                         "loop); the timed steps run each solve's loop as its "
                                         "captured CUDA graph",
                        "ms_per_step_with_events": round(float(np.mean(ms_k)), 4)},
        "roofline": roof,
        "kernels": kernels,
        "clocks": cl,
    }
    if rank == 0 and args.many_rounds > 0 and not args.quick:
        line["n1_case10000"] = n1_case10000(gox, args.many_rounds)
        line["many_topologies"] = many_topologies(gox, args.many_rounds)
        line["pgm_batch"] = pgm_batch(gox, args.many_rounds)
        line["qlim_case2000"] = qlim_case2000(gox, args.many_rounds)
    # serving last: its 16 grids' refactor plans (tuned on one-group batches)
    # enter the process's plan cache, where later topologies of the same
    # size, fill and batch bucket would take them untimed
    if rank == 0 and args.serve_rate > 0 and not args.quick:
        rates = sorted({r for r in (1000.0, 3000.0, 10000.0, 30000.0, args.serve_rate)
                        if r <= args.serve_rate})
        line["serving"] = serve(gox, rates, args.serve_seconds)
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, dt, passes, ref = cpu_baseline(g, yb, p, q, threads)
        line["cpu_baseline"] = {"value": round(v, 1), "unit": "solves/s", "cores": threads,
                                "kind": "port", "cpu": cpu_model(),
                                "physical_cores": physical_cores(),
                                "threads_sweep_solves_per_s": thread_sweep(g, yb, p, q),
                                "ordering": "the reference's compiled klu_analyze (committed "
                                            "fixture)",
                                "sample": f"{passes} passes over the {p.shape[0]}-scenario "
                                          f"workload ({dt:.1f} s)"}
        # every result states its error against the FP64 oracle: the timed
        # steps' results (the last step of each precision) against the
        # oracle's reports of the same scenarios
        line["err_vs_oracle"] = {
            "fp64": error_vs_oracle(vm_64, va_64, it_64, st_64, ref),
            "mixed": error_vs_oracle(vm_mx, va_mx, it_mx, st_mx, ref),
            "note": "max over all scenarios of the timed configuration; the FP64 path must match "
                    "the oracle's iteration counts and |V|, theta within 1e-9"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
