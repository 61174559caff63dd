"""Seeded synthetic meshed transmission grids and their Y-bus.

The generator builds the grid family the batched power-flow workloads are
quoted on: a random spanning tree in which every bus ``i > 0`` hangs off a
uniformly chosen bus among its 8 predecessors, plus chords between buses at
most 12 indices apart; ``r ~ U[0.002, 0.03]``, ``x = r * U[4, 10]``,
``b ~ U[0, 0.06]``; 10 % of the branches are transformers with a real tap
``~ U[0.95, 1.05]``; PQ loads ``P ~ U[0.05, 0.6]``, ``Q = P * U[0.1, 0.5]``;
PV generation equal to 1.03 x the total load, split by ``U[0.5, 1.5]``
weights, with set-points ``~ U[0.98, 1.06]``; bus 0 is the slack at
``1.04 /_ 0``.

Y-bus stamping follows the reference's pi-model:
  * lines: ``build_ybus`` (gridoxide src/network.rs:225-247): series
    ``y = 1/(r + jx)``, half the charging at each end;
  * transformers: ``branch_calc_param`` with both ends closed
    (src/network.rs:339-360): ``yff = (y_s + y_sh/2)/k^2``,
    ``yft = -y_s/conj(t)``, ``ytf = -y_s/t``, ``ytt = y_s + y_sh/2``;
  * duplicates are summed in insertion order (lines first, then
    transformers), as ``YBus::finish`` does (src/network.rs:52-71).
Complex division uses num-complex's formula
``(a.re*b.re + a.im*b.im, a.im*b.re - a.re*b.im) / |b|^2`` so the admittances
match the reference bit for bit.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BUS_PQ = 1
BUS_PV = 2
BUS_SLACK = 3


def _cdiv(ar, ai, br, bi):
    n = br * br + bi * bi
    return (ar * br + ai * bi) / n, (ai * br - ar * bi) / n


@dataclass
class Grid:
    """One topology plus its base-case bus data (per-unit)."""

    n_bus: int
    bus_type: np.ndarray          # int32 [N]: BUS_PQ / BUS_PV / BUS_SLACK
    vm: np.ndarray                # float64 [N]: slack/PV set-point, 1.0 for PQ (flat start)
    va: np.ndarray                # float64 [N]: 0 (flat start)
    p_spec: np.ndarray            # float64 [N]: net injection (generation - load)
    q_spec: np.ndarray            # float64 [N]
    br_from: np.ndarray           # int32 [M]
    br_to: np.ndarray             # int32 [M]
    br_r: np.ndarray              # float64 [M]
    br_x: np.ndarray              # float64 [M]
    br_b: np.ndarray              # float64 [M] total line charging
    br_tap: np.ndarray            # float64 [M] off-nominal ratio (1.0 for lines)
    br_is_trafo: np.ndarray       # bool [M]
    load_p: np.ndarray = field(default=None)   # float64 [N] base load P (PQ buses)
    load_q: np.ndarray = field(default=None)
    pv_weight: np.ndarray = field(default=None)  # float64 [N], zero off PV buses
    seed: int = 0

    @property
    def n_branch(self) -> int:
        return int(self.br_from.shape[0])


def make_grid(n_bus: int, n_pv: int, n_branch: int, seed: int,
              slack_vm: float = 1.04, load_scale: float = 1.0,
              r_scale: float = 1.0) -> Grid:
    """Builds one seeded grid of the synthetic meshed family (see module doc).

    ``load_scale`` multiplies every drawn load (and so the PV generation that
    balances it); ``r_scale`` multiplies every drawn resistance after the
    reactance ``x = r * U[4, 10]`` was drawn from the unscaled ``r``.  Both
    default to 1 (the literal distributions).  Neither touches the graph or
    the bus types, so the sparsity pattern -- and with it every symbolic and
    kernel cost -- is that of the literal grid."""
    if n_bus < 2:
        raise ValueError("need at least 2 buses")
    if n_pv > n_bus - 1:
        raise ValueError("too many PV buses")
    n_chord = n_branch - (n_bus - 1)
    if n_chord < 0:
        raise ValueError("n_branch must be >= n_bus - 1 (spanning tree)")
    rng = np.random.default_rng(seed)

    # spanning tree: bus i attaches to a uniform bus among the 8 preceding
    edges = []
    have = set()
    for i in range(1, n_bus):
        lo = max(0, i - 8)
        j = int(rng.integers(lo, i))
        edges.append((j, i))
        have.add((j, i))
    # chords between distinct buses |i - j| <= 12 that are not yet connected
    tries = 0
    while len(edges) < n_branch:
        tries += 1
        if tries > 1000 * n_branch + 10000:
            raise RuntimeError("could not place the requested chords")
        i = int(rng.integers(0, n_bus))
        d = int(rng.integers(1, 13))
        j = i + d
        if j >= n_bus:
            continue
        if (i, j) in have:
            continue
        have.add((i, j))
        edges.append((i, j))
    m = len(edges)
    br_from = np.array([e[0] for e in edges], dtype=np.int32)
    br_to = np.array([e[1] for e in edges], dtype=np.int32)
    br_r = rng.uniform(0.002, 0.03, m)
    br_x = br_r * rng.uniform(4.0, 10.0, m)
    br_b = rng.uniform(0.0, 0.06, m)
    br_r = br_r * r_scale
    n_tr = int(round(0.10 * m))
    is_tr = np.zeros(m, dtype=bool)
    is_tr[rng.choice(m, n_tr, replace=False)] = True
    br_tap = np.ones(m)
    br_tap[is_tr] = rng.uniform(0.95, 1.05, n_tr)

    bus_type = np.full(n_bus, BUS_PQ, dtype=np.int32)
    bus_type[0] = BUS_SLACK
    pv = np.sort(rng.choice(np.arange(1, n_bus), n_pv, replace=False))
    bus_type[pv] = BUS_PV

    vm = np.ones(n_bus)
    vm[0] = slack_vm
    vm[pv] = rng.uniform(0.98, 1.06, n_pv)
    va = np.zeros(n_bus)

    pq = np.flatnonzero(bus_type == BUS_PQ)
    load_p = np.zeros(n_bus)
    load_q = np.zeros(n_bus)
    load_p[pq] = rng.uniform(0.05, 0.6, pq.size)
    load_q[pq] = load_p[pq] * rng.uniform(0.1, 0.5, pq.size)
    w = np.zeros(n_bus)
    w[pv] = rng.uniform(0.5, 1.5, n_pv)
    load_p *= load_scale
    load_q *= load_scale

    g = Grid(n_bus=n_bus, bus_type=bus_type, vm=vm, va=va,
             p_spec=np.zeros(n_bus), q_spec=np.zeros(n_bus),
             br_from=br_from, br_to=br_to, br_r=br_r, br_x=br_x, br_b=br_b,
             br_tap=br_tap, br_is_trafo=is_tr, load_p=load_p, load_q=load_q,
             pv_weight=w, seed=seed)
    g.p_spec, g.q_spec = injections_for_loads(g, load_p, load_q)
    return g


def injections_for_loads(g: Grid, load_p: np.ndarray, load_q: np.ndarray):
    """Net injections for given PQ loads; PV generation = 1.03 x total load
    split by the grid's PV weights.  Works on [N] or [B, N] load arrays."""
    load_p = np.asarray(load_p, dtype=np.float64)
    load_q = np.asarray(load_q, dtype=np.float64)
    total = load_p.sum(axis=-1, keepdims=True)
    wsum = g.pv_weight.sum()
    gen = 1.03 * total * (g.pv_weight / wsum if wsum > 0 else g.pv_weight)
    p = gen - load_p
    q = -load_q
    return p, q


def load_scenarios(g: Grid, n_scen: int, sigma: float, seed: int):
    """[B, N] injections: every bus load x lognormal(0, sigma) (same factor for
    P and Q of a bus), PV generation rescaled to 1.03 x the scenario's load."""
    rng = np.random.default_rng(seed)
    mult = rng.lognormal(0.0, sigma, size=(n_scen, g.n_bus))
    lp = g.load_p[None, :] * mult
    lq = g.load_q[None, :] * mult
    return injections_for_loads(g, lp, lq)


# ---------------------------------------------------------------------------
# Y-bus

def branch_admittances(g: Grid):
    """Per-branch (yff, yft, ytf, ytt) as (re, im) arrays, reference formulas."""
    one_re, one_im = 1.0, 0.0
    ys_re, ys_im = _cdiv(one_re, one_im, g.br_r, g.br_x)
    # lines: diag = y_line + (g/2, b/2), off = -y_line (src/network.rs:231-245)
    sh_re = np.zeros_like(g.br_b)
    sh_im = g.br_b / 2.0
    line_d_re = ys_re + sh_re
    line_d_im = ys_im + sh_im
    # transformers (src/network.rs:339-360, tap real, clock 0)
    k = np.abs(g.br_tap)
    yd_re = ys_re + 0.0 * 0.5
    yd_im = ys_im + g.br_b * 0.5
    yff_t_re = yd_re / (k * k)
    yff_t_im = yd_im / (k * k)
    # -y_s / conj(t) with t = (k, 0): conj(t) = (k, -0.0)
    yft_t_re, yft_t_im = _cdiv(-ys_re, -ys_im, k, -0.0 * k)
    ytf_t_re, ytf_t_im = _cdiv(-ys_re, -ys_im, k, 0.0 * k)
    tr = g.br_is_trafo
    yff = (np.where(tr, yff_t_re, line_d_re), np.where(tr, yff_t_im, line_d_im))
    yft = (np.where(tr, yft_t_re, -ys_re), np.where(tr, yft_t_im, -ys_im))
    ytf = (np.where(tr, ytf_t_re, -ys_re), np.where(tr, ytf_t_im, -ys_im))
    ytt = (np.where(tr, yd_re, line_d_re), np.where(tr, yd_im, line_d_im))
    return yff, yft, ytf, ytt


@dataclass
class YBus:
    """CSR Y-bus, each row's columns ascending, duplicates summed."""

    n: int
    indptr: np.ndarray   # int32 [N+1]
    indices: np.ndarray  # int32 [nnz]
    re: np.ndarray       # float64 [nnz]
    im: np.ndarray       # float64 [nnz]

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])

    def slot(self, i: int, j: int) -> int:
        s, e = self.indptr[i], self.indptr[i + 1]
        pos = s + int(np.searchsorted(self.indices[s:e], j))
        if pos >= e or self.indices[pos] != j:
            raise KeyError((i, j))
        return pos

    def dense(self) -> np.ndarray:
        a = np.zeros((self.n, self.n), dtype=np.complex128)
        for i in range(self.n):
            for p in range(self.indptr[i], self.indptr[i + 1]):
                a[i, self.indices[p]] += self.re[p] + 1j * self.im[p]
        return a


def build_ybus(g: Grid) -> YBus:
    yff, yft, ytf, ytt = branch_admittances(g)
    rows, cols, vre, vim = [], [], [], []

    def add(sel):
        f, t = g.br_from[sel], g.br_to[sel]
        # per branch, the reference adds ff, tt, ft, tf for lines and
        # ff, ft, tf, tt for transformers; summation order per (i, j) only
        # depends on branch order, which both respect.
        for (rr, cc, y) in ((f, f, yff), (t, t, ytt), (f, t, yft), (t, f, ytf)):
            rows.append(rr)
            cols.append(cc)
            vre.append(y[0][sel])
            vim.append(y[1][sel])

    lines = np.flatnonzero(~g.br_is_trafo)
    trafos = np.flatnonzero(g.br_is_trafo)
    # interleave per branch to keep the reference's insertion order
    order_r, order_c, order_re, order_im = [], [], [], []
    for sel_all in (lines, trafos):
        if sel_all.size == 0:
            continue
        rows.clear(); cols.clear(); vre.clear(); vim.clear()
        add(sel_all)
        # stack as [4, m] then transpose to per-branch order
        r4 = np.stack(rows); c4 = np.stack(cols); re4 = np.stack(vre); im4 = np.stack(vim)
        order_r.append(r4.T.ravel()); order_c.append(c4.T.ravel())
        order_re.append(re4.T.ravel()); order_im.append(im4.T.ravel())
    r = np.concatenate(order_r).astype(np.int64)
    c = np.concatenate(order_c).astype(np.int64)
    vr = np.concatenate(order_re)
    vi = np.concatenate(order_im)
    return ybus_from_triplets(g.n_bus, r, c, vr, vi)


def ybus_from_triplets(n, r, c, vr, vi) -> YBus:
    """Sums duplicates in insertion order and sorts each row by column."""
    r = np.asarray(r, dtype=np.int64)
    c = np.asarray(c, dtype=np.int64)
    key = r * n + c
    # stable sort keeps insertion order within a key -> sequential summation
    order = np.argsort(key, kind="stable")
    ks = key[order]
    uniq, start = np.unique(ks, return_index=True)
    nnz = uniq.size
    re = np.zeros(nnz)
    im = np.zeros(nnz)
    # sequential (insertion-order) sums
    bounds = np.append(start, ks.size)
    vr_o = np.asarray(vr, dtype=np.float64)[order]
    vi_o = np.asarray(vi, dtype=np.float64)[order]
    maxdup = int(np.max(np.diff(bounds))) if nnz else 0
    for d in range(maxdup):
        idx = start + d
        ok = idx < bounds[1:]
        re[ok] = re[ok] + vr_o[idx[ok]]
        im[ok] = im[ok] + vi_o[idx[ok]]
    rows = (uniq // n).astype(np.int64)
    cols = (uniq % n).astype(np.int32)
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    indptr = np.cumsum(indptr).astype(np.int32)
    return YBus(n=n, indptr=indptr, indices=cols, re=re, im=im)


def ybus_from_lines(n, lines) -> YBus:
    """Y-bus from reference-style line records (from, to, r, x, b_shunt[, g_shunt]),
    build_ybus order (src/network.rs:225-247), self-loops as pure shunts."""
    rows, cols, vr, vi = [], [], [], []
    for ln in lines:
        f, t, r, x, b = ln[:5]
        gsh = ln[5] if len(ln) > 5 else 0.0
        if f == t:
            rows.append(f); cols.append(f); vr.append(gsh); vi.append(b)
            continue
        yr, yi = _cdiv(1.0, 0.0, r, x)
        hr, hi = gsh / 2.0, b / 2.0
        for (a, bb, er, ei) in ((f, f, yr + hr, yi + hi), (t, t, yr + hr, yi + hi),
                                (f, t, -yr, -yi), (t, f, -yr, -yi)):
            rows.append(a); cols.append(bb); vr.append(er); vi.append(ei)
    return ybus_from_triplets(n, rows, cols, vr, vi)


# ---------------------------------------------------------------------------
# N-1 outages

def bridges(g: Grid) -> np.ndarray:
    """Boolean [M]: branch is a bridge (its removal disconnects the grid).
    Iterative Tarjan low-link over the branch multigraph."""
    n = g.n_bus
    adj = [[] for _ in range(n)]
    for e in range(g.n_branch):
        a, b = int(g.br_from[e]), int(g.br_to[e])
        adj[a].append((b, e))
        adj[b].append((a, e))
    disc = [-1] * n
    low = [0] * n
    is_bridge = np.zeros(g.n_branch, dtype=bool)
    timer = 0
    for root in range(n):
        if disc[root] != -1:
            continue
        stack = [(root, -1, 0)]
        disc[root] = low[root] = timer
        timer += 1
        while stack:
            u, pe, it = stack[-1]
            if it < len(adj[u]):
                stack[-1] = (u, pe, it + 1)
                v, e = adj[u][it]
                if e == pe:
                    continue
                if disc[v] == -1:
                    disc[v] = low[v] = timer
                    timer += 1
                    stack.append((v, e, 0))
                else:
                    low[u] = min(low[u], disc[v])
            else:
                stack.pop()
                if stack:
                    p = stack[-1][0]
                    low[p] = min(low[p], low[u])
                    if low[u] > disc[p]:
                        is_bridge[pe] = True
    return is_bridge


def outage_deltas(g: Grid, yb: YBus, branches: np.ndarray):
    """Per outage, the 4 Y-bus slots (ff, ft, tf, tt) and the values to ADD to
    them (the negated branch stamp).  Returns (slots [S,4] int32,
    dre [S,4], dim [S,4])."""
    yff, yft, ytf, ytt = branch_admittances(g)
    branches = np.asarray(branches, dtype=np.int64)
    S = branches.size
    slots = np.zeros((S, 4), dtype=np.int32)
    dre = np.zeros((S, 4))
    dim = np.zeros((S, 4))
    for s, e in enumerate(branches):
        f, t = int(g.br_from[e]), int(g.br_to[e])
        slots[s] = (yb.slot(f, f), yb.slot(f, t), yb.slot(t, f), yb.slot(t, t))
        dre[s] = (-yff[0][e], -yft[0][e], -ytf[0][e], -ytt[0][e])
        dim[s] = (-yff[1][e], -yft[1][e], -ytf[1][e], -ytt[1][e])
    return slots, dre, dim


# ---------------------------------------------------------------------------
# Named workloads

# Grid-size dependent value scaling.  The literal distributions are only
# solvable on small grids: the generator's graph is a band (tree edges reach
# back <= 8 buses, chords <= 12), so a 2,000-bus grid is ~450 hops deep and
# every loss or local imbalance must cross it to reach the single slack at
# bus 0.  Newton-Raphson (the reference's own algorithm, run by the oracle)
# diverges from flat start on the literal 2,000-bus grid at >= 25 % load and
# on the 10,000-bus grid even at zero load.  The scales below are the
# smallest changes that give flat-start convergence in 5-6 iterations.
CONFIGS = {
    # name: (n_bus, n_pv, n_branch, seed, load_scale, r_scale)
    "case118": (118, 53, 186, 1, 1.0, 1.0),
    "case2000": (2000, 300, 2799, 2, 0.1, 0.2),
    "case10000": (10000, 1500, 13499, 3, 0.01, 0.05),
}


def config_grid(name: str) -> Grid:
    """The grids the batched workloads are quoted on (seed = 1 + index)."""
    n, npv, nbr, seed, ls, rs = CONFIGS[name]
    return make_grid(n, npv, nbr, seed=seed, load_scale=ls, r_scale=rs)


# ---------------------------------------------------------------------------
# Multi-topology workloads: grids of any size from the same family.  The
# value scales follow the log-linear trend between the 2,000- and 10,000-bus
# configs (capped for small grids) and are halved; every one of the 48
# many-topology grids below then converges from flat start (checked against
# the oracle when the list was fixed).

def family_scales(n_bus: int) -> tuple[float, float]:
    """(load_scale, r_scale) for a family grid of n_bus buses."""
    lg = np.log10(max(n_bus, 2))
    ls = min(0.3, 10.0 ** (3.72 - 1.43 * lg)) * 0.5
    rs = min(0.5, 10.0 ** (2.143 - 0.861 * lg)) * 0.5
    return float(ls), float(rs)


def family_grid(n_bus: int, seed: int, pv_frac: float = 0.15) -> Grid:
    """A family grid: pv_frac PV buses, 40 chords per 100 buses."""
    ls, rs = family_scales(n_bus)
    n_pv = max(1, int(round(pv_frac * n_bus)))
    n_branch = (n_bus - 1) + int(round(0.4 * n_bus))
    return make_grid(int(n_bus), n_pv, n_branch, seed=seed, load_scale=ls, r_scale=rs)


def many_topologies(count: int = 48, n_min: int = 30, n_max: int = 20000, b_min: int = 8,
                    b_max: int = 1024, seed: int = 4):
    """The many-topology workload: `count` grids with bus counts log-uniform
    in [n_min, n_max] and batch sizes uniform in [b_min, b_max]; returns
    [(n_bus, grid seed, batch, scenario seed)]."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count)).astype(int)
    bs = rng.integers(b_min, b_max + 1, size=count)
    return [(int(n), 1000 + t, int(b), 40 + t) for t, (n, b) in enumerate(zip(ns, bs))]
