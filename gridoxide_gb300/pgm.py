"""power-grid-model (PGM) JSON input to the batched solver's network.

A restatement of the reference's symmetric PGM conversion
(`pgm_to_buses_and_branches`, src/pgm.rs:347-595, with `node_id_to_idx`
:261-268 and `pgm_shunts_1ph` :270-288), its Y-bus stamping (`build_ybus`,
`stamp_transformers`, `stamp_shunts`, src/network.rs:225-247, 339-378,
473-478), and the island handling its solver applies before Newton
(`connected_components`, `classify`, `mark_unreferenced_islands`,
src/network.rs:121-223): nodes become PQ buses, every active source a
virtual slack bus behind its source impedance, constant-impedance /
constant-current loads and generators ZIP terms, an active voltage regulator
makes its generator's node PV, and the buses of a component without a slack
become slack buses at V = 0.  A three-winding transformer becomes three
two-winding legs to an internal star bus (src/pgm.rs:461-532, with
`three_winding_star_params`, src/network.rs:572-594).  Asymmetric branches
and the 3-phase model are not converted.

`solve` runs a converted network on the GPU the way the reference's PGM tests
do (src/tests klu_native_jacobian_test.rs:18-24): linear initial guess, then
Newton-Raphson with tol 1e-6, at most 20 iterations, FP64.
"""
from __future__ import annotations

import copy
import json
import math
from dataclasses import dataclass

import numpy as np

from . import grids as G

S_BASE_VA = 1e6
FREQ_HZ = 50.0


@dataclass
class Network:
    """A converted PGM input: buses (physical nodes in id order, then the
    sources' virtual slack buses), Y-bus, ZIP terms, node id -> bus index."""

    n_bus: int
    bus_type: np.ndarray   # int32
    vm: np.ndarray
    va: np.ndarray
    p_spec: np.ndarray
    q_spec: np.ndarray
    zip_imp: np.ndarray    # complex, constant impedance (per unit at |V| = 1)
    zip_cur: np.ndarray    # complex, constant current
    ybus: G.YBus
    id_to_idx: dict
    u_rated: np.ndarray    # V, per bus (a source's slack bus: its node's; a star bus: winding 1's)
    zip_terms: np.ndarray  # int32, ZIP terms per bus (loads and generators of type 1 or 2)
    islands: list          # components without a slack bus, pinned to V = 0
    guess_singular: bool   # the reference's linear guess would meet a singular system
    q_min: np.ndarray      # per unit, the voltage regulators' reactive limits (-inf: none)
    q_max: np.ndarray      # per unit (+inf: none)


def load(path: str) -> dict:
    with open(path) as fh:
        return json.load(fh)


def node_id_to_idx(data: dict) -> dict:
    """src/pgm.rs:261-268: node ids in ascending order."""
    return {nid: k for k, nid in enumerate(sorted(int(n["id"]) for n in data.get("node", [])))}


def _polar(mag, ang):
    return complex(mag * math.cos(ang), mag * math.sin(ang))


def transformer_tap(u1, u2, tap_side, tap_pos, tap_min, tap_max, tap_nom, tap_size, clock):
    """src/network.rs:519-540 (with tap_ratio_from_voltages :305-307)."""
    tap_pos = min(max(tap_pos, min(tap_min, tap_max)), max(tap_min, tap_max))
    delta = (tap_pos - tap_nom) * tap_size
    if tap_side == 0:
        return _polar((u1 + delta) / u1, clock * math.pi / 6.0)
    return _polar(u2 / (u2 + delta), clock * math.pi / 6.0)


def transformer_admittances(u_field, u_base, sn, uk, pk, i0, p0, s_base):
    """src/network.rs:542-564: series and shunt admittance in per unit of the
    to-side base u_base, scaled by the nameplate voltage u_field."""
    base_y_to = s_base / (u_base * u_base)
    uk_sign = 1.0 if uk >= 0.0 else -1.0
    z_abs = abs(uk) * u_field * u_field / sn
    r_ohm = pk * u_field * u_field / (sn * sn)
    x_sq = z_abs * z_abs - r_ohm * r_ohm
    x_ohm = uk_sign * (math.sqrt(x_sq) if x_sq > 0.0 else 0.0)
    y_series = (1.0 / complex(r_ohm, x_ohm)) / base_y_to
    g_fe = p0 / (u_field * u_field)
    y_sh_abs = i0 * sn / (u_field * u_field)
    b_sq = y_sh_abs * y_sh_abs - g_fe * g_fe
    b_m = -math.sqrt(b_sq) if b_sq > 0.0 else 0.0
    return y_series, complex(g_fe, b_m) / base_y_to


def _half_open_branch_shunt(y_series, y_shunt):
    """src/network.rs:320-327."""
    if y_shunt == 0:
        return 0j
    return y_shunt * 0.5 + 1.0 / (1.0 / y_series + 2.0 / y_shunt)


def branch_calc_param(y_series, y_shunt, tap, from_status, to_status):
    """src/network.rs:339-362: [yff, yft, ytf, ytt]."""
    k = abs(tap)
    if from_status == 1 and to_status == 1:
        y_diag = y_series + y_shunt * 0.5
        return [y_diag / (k * k), -y_series / tap.conjugate(), -y_series / tap, y_diag]
    if from_status == 1 and to_status == 0:
        return [_half_open_branch_shunt(y_series, y_shunt) / (k * k), 0j, 0j, 0j]
    if from_status == 0 and to_status == 1:
        return [0j, 0j, 0j, _half_open_branch_shunt(y_series, y_shunt)]
    return [0j, 0j, 0j, 0j]


def three_winding_star_params(sn_1, sn_2, sn_3, uk_12, uk_13, uk_23, pk_12, pk_13, pk_23):
    """src/network.rs:572-594: star-equivalent uk and pk on side 1's power base."""
    uk_12r = uk_12 * sn_1 / min(sn_1, sn_2)
    uk_13r = uk_13 * sn_1 / min(sn_1, sn_3)
    uk_23r = uk_23 * sn_1 / min(sn_2, sn_3)
    uk = (0.5 * (uk_12r + uk_13r - uk_23r),
          0.5 * (uk_12r + uk_23r - uk_13r) * (sn_2 / sn_1),
          0.5 * (uk_13r + uk_23r - uk_12r) * (sn_3 / sn_1))
    pk_12r = pk_12 * (sn_1 / min(sn_1, sn_2)) ** 2
    pk_13r = pk_13 * (sn_1 / min(sn_1, sn_3)) ** 2
    pk_23r = pk_23 * (sn_1 / min(sn_2, sn_3)) ** 2
    pk = (0.5 * (pk_12r + pk_13r - pk_23r),
          0.5 * (pk_12r + pk_23r - pk_13r) * (sn_2 / sn_1) ** 2,
          0.5 * (pk_13r + pk_23r - pk_12r) * (sn_3 / sn_1) ** 2)
    return uk, pk


def source_impedance_pu(sk, rx_ratio, s_base):
    """src/network.rs:495-499."""
    z = s_base / sk
    x = z / math.sqrt(rx_ratio * rx_ratio + 1.0)
    return rx_ratio * x, x


def convert(doc: dict, s_base: float = S_BASE_VA, freq_hz: float = FREQ_HZ,
            mark_islands: bool = True) -> Network:
    """pgm_to_buses_and_branches + pgm_shunts_1ph + build_ybus + stamp_shunts;
    with `mark_islands`, then mark_unreferenced_islands (the start of every
    solve in the reference)."""
    data = doc["data"]
    id_to_idx = node_id_to_idx(data)
    u_rated = {int(n["id"]): float(n["u_rated"]) for n in data.get("node", [])}
    n_nodes = len(id_to_idx)
    p_inj = np.zeros(n_nodes)
    q_inj = np.zeros(n_nodes)
    zimp = np.zeros(n_nodes, np.complex128)
    zcur = np.zeros(n_nodes, np.complex128)
    nzip = np.zeros(n_nodes, np.int32)

    def accumulate(node, load_type, p, q, sign):
        s = complex(p, q) * sign / s_base
        k = id_to_idx[int(node)]
        if load_type == 1:
            zimp[k] += s
            nzip[k] += 1
        elif load_type == 2:
            zcur[k] += s
            nzip[k] += 1
        else:
            p_inj[k] += s.real
            q_inj[k] += s.imag

    for ld in data.get("sym_load", []):
        if ld["status"] != 0:
            accumulate(ld["node"], ld.get("type", 0), ld["p_specified"], ld["q_specified"], -1.0)
    for gn in data.get("sym_gen", []):
        if gn["status"] != 0:
            accumulate(gn["node"], gn.get("type", 0), gn["p_specified"], gn["q_specified"], 1.0)
    for ld in data.get("asym_load", []):
        if ld["status"] != 0:
            accumulate(ld["node"], ld.get("type", 0), sum(ld["p_specified"]), sum(ld["q_specified"]), -1.0)
    for gn in data.get("asym_gen", []):
        if gn["status"] != 0:
            accumulate(gn["node"], gn.get("type", 0), sum(gn["p_specified"]), sum(gn["q_specified"]), 1.0)

    sources = [s for s in data.get("source", []) if s["status"] != 0]
    trafo3 = data.get("three_winding_transformer", [])
    n_star = len(trafo3)
    n = n_nodes + n_star + len(sources)
    bus_type = np.full(n, G.BUS_PQ, np.int32)
    vm = np.ones(n)
    va = np.zeros(n)
    p_spec = np.zeros(n)
    q_spec = np.zeros(n)
    p_spec[:n_nodes] = p_inj
    q_spec[:n_nodes] = q_inj
    zip_imp = np.zeros(n, np.complex128)
    zip_cur = np.zeros(n, np.complex128)
    zip_imp[:n_nodes] = zimp
    zip_cur[:n_nodes] = zcur
    zip_terms = np.zeros(n, np.int32)
    zip_terms[:n_nodes] = nzip
    u_rated_bus = np.zeros(n)
    for nid, k in id_to_idx.items():
        u_rated_bus[k] = u_rated[nid]

    # voltage regulators: their generator's node becomes PV at u_ref, with
    # the regulator's reactive limits (NaN or absent: none)
    q_min = np.full(n, -np.inf)
    q_max = np.full(n, np.inf)
    gen_node = {int(g["id"]): int(g["node"]) for g in data.get("sym_gen", [])}
    for vr in data.get("voltage_regulator", []):
        if vr["status"] == 0 or int(vr["regulated_object"]) not in gen_node:
            continue
        k = id_to_idx[gen_node[int(vr["regulated_object"])]]
        if bus_type[k] == G.BUS_PQ:
            bus_type[k] = G.BUS_PV
            vm[k] = vr["u_ref"]
            lo, hi = vr.get("q_min", math.nan), vr.get("q_max", math.nan)
            q_min[k] = -np.inf if lo is None or math.isnan(lo) else lo / s_base
            q_max[k] = np.inf if hi is None or math.isnan(hi) else hi / s_base

    rows, cols, vals = [], [], []

    def add(i, j, y):
        rows.append(i)
        cols.append(j)
        vals.append(y)

    omega = 2.0 * math.pi * freq_hz
    lines = []  # (from, to, r, x, b_shunt)
    for ln in data.get("line", []):
        fs, ts = ln["from_status"], ln["to_status"]
        if fs == 1 and ts == 1:
            zb = u_rated[int(ln["from_node"])] ** 2 / s_base
            lines.append((id_to_idx[int(ln["from_node"])], id_to_idx[int(ln["to_node"])],
                          ln["r1"] / zb, ln["x1"] / zb, omega * ln["c1"] * zb))
        elif fs == 1 and ts == 0:
            zb = u_rated[int(ln["from_node"])] ** 2 / s_base
            k = id_to_idx[int(ln["from_node"])]
            lines.append((k, k, 0.0, 0.0, omega * ln["c1"] * zb))
        elif fs == 0 and ts == 1:
            zb = u_rated[int(ln["to_node"])] ** 2 / s_base
            k = id_to_idx[int(ln["to_node"])]
            lines.append((k, k, 0.0, 0.0, omega * ln["c1"] * zb))
    for i, src in enumerate(sources):
        v = n_nodes + n_star + i
        bus_type[v] = G.BUS_SLACK
        vm[v] = src["u_ref"]
        u_rated_bus[v] = u_rated[int(src["node"])]
        r_s, x_s = source_impedance_pu(src["sk"], src["rx_ratio"], s_base)
        lines.append((v, id_to_idx[int(src["node"])], r_s, x_s, 0.0))
    # build_ybus: lines (self-loops as shunts, series branches), then transformers
    for (f, t, r, x, b) in lines:
        if f == t:
            add(f, f, complex(0.0, b))
            continue
        y_line = 1.0 / complex(r, x)
        y_half = complex(0.0, b / 2.0)
        add(f, f, y_line + y_half)
        add(t, t, y_line + y_half)
        add(f, t, -y_line)
        add(t, f, -y_line)
    trafos = []  # (from, to, from_status, to_status, y_series, y_shunt, tap)
    for tr in data.get("transformer", []):
        tap = transformer_tap(tr["u1"], tr["u2"], tr["tap_side"], tr["tap_pos"], tr["tap_min"],
                              tr["tap_max"], tr["tap_nom"], tr["tap_size"], tr["clock"])
        ys, ysh = transformer_admittances(tr["u2"], tr["u2"], tr["sn"], tr["uk"], tr["pk"], tr["i0"],
                                          tr["p0"], s_base)
        trafos.append((id_to_idx[int(tr["from_node"])], id_to_idx[int(tr["to_node"])],
                       tr["from_status"], tr["to_status"], ys, ysh, tap))
    for i, t3 in enumerate(trafo3):
        star = n_nodes + i
        u1r, u2r, u3r = (u_rated[int(t3[k])] for k in ("node_1", "node_2", "node_3"))
        u_rated_bus[star] = u1r
        direction = 1.0 if t3["tap_max"] > t3["tap_min"] else -1.0
        delta = direction * (t3["tap_pos"] - t3["tap_nom"]) * t3["tap_size"]
        u1, u2, u3 = t3["u1"], t3["u2"], t3["u3"]
        if t3["tap_side"] == 0:
            u1 += delta
        elif t3["tap_side"] == 1:
            u2 += delta
        else:
            u3 += delta
        uk, pk = three_winding_star_params(t3["sn_1"], t3["sn_2"], t3["sn_3"], t3["uk_12"], t3["uk_13"],
                                           t3["uk_23"], t3["pk_12"], t3["pk_13"], t3["pk_23"])
        legs = ((t3["node_1"], t3["status_1"], t3["sn_1"], 0, t3["i0"], t3["p0"],
                 _polar(1.0, 0.0)),
                (t3["node_2"], t3["status_2"], t3["sn_2"], 1, 0.0, 0.0,
                 _polar((u2 * u1r) / (u1 * u2r), (12 - t3["clock_12"]) * math.pi / 6.0)),
                (t3["node_3"], t3["status_3"], t3["sn_3"], 2, 0.0, 0.0,
                 _polar((u3 * u1r) / (u1 * u3r), (12 - t3["clock_13"]) * math.pi / 6.0)))
        for node, status, sn, w, i0, p0, tap in legs:
            ys, ysh = transformer_admittances(u1, u1r, sn, uk[w], pk[w], i0, p0, s_base)
            trafos.append((id_to_idx[int(node)], star, status, 1, ys, ysh, tap))
    for (f, t, fs, ts, ys, ysh, tap) in trafos:
        yff, yft, ytf, ytt = branch_calc_param(ys, ysh, tap, fs, ts)
        add(f, f, yff)
        add(f, t, yft)
        add(t, f, ytf)
        add(t, t, ytt)
    for sh in data.get("shunt", []):
        if sh["status"] == 0:
            continue
        ur = u_rated[int(sh["node"])]
        base_y = s_base / (ur * ur)
        k = id_to_idx[int(sh["node"])]
        add(k, k, complex(sh["g1"], sh["b1"]) / base_y)
    yb = G.ybus_from_triplets(n, rows, cols, [v.real for v in vals], [v.imag for v in vals])
    net = Network(n_bus=n, bus_type=bus_type, vm=vm, va=va, p_spec=p_spec, q_spec=q_spec,
                  zip_imp=zip_imp, zip_cur=zip_cur, ybus=yb, id_to_idx=id_to_idx,
                  u_rated=u_rated_bus, zip_terms=zip_terms, islands=[], guess_singular=False,
                  q_min=q_min, q_max=q_max)
    if mark_islands:
        mark_unreferenced_islands(net)
    return net


def connected_components(yb: G.YBus):
    """src/network.rs:121-140: components of the Y-bus pattern."""
    n = yb.n
    seen = np.zeros(n, bool)
    comps = []
    for start in range(n):
        if seen[start]:
            continue
        members, stack = [], [start]
        seen[start] = True
        while stack:
            i = stack.pop()
            members.append(i)
            for p in range(int(yb.indptr[i]), int(yb.indptr[i + 1])):
                j = int(yb.indices[p])
                if j != i and not seen[j]:
                    seen[j] = True
                    stack.append(j)
        comps.append(sorted(members))
    return comps


def _guess_block_singular(net: Network, comp) -> bool:
    """Whether the linear-guess rows of one slack-free component (its PQ
    buses, Y + the constant-admittance load on the diagonal, as in
    src/network.rs:627-671) form a singular system.  The reference builds its
    guess before it marks islands, so such a component makes its whole guess
    fail (src/sparse.rs:48-63 returns None) and every bus keeps its start."""
    from . import solver as S
    yb = net.ybus
    pq = [i for i in comp if net.bus_type[i] == G.BUS_PQ]
    if not pq:
        return False
    pos = {b: r for r, b in enumerate(pq)}
    rows, cols, vals = [], [], []

    def block(r, c, y):
        rows.extend((2 * r, 2 * r, 2 * r + 1, 2 * r + 1))
        cols.extend((2 * c, 2 * c + 1, 2 * c, 2 * c + 1))
        vals.extend((y.real, -y.imag, y.imag, y.real))

    for r, i in enumerate(pq):
        v = net.vm[i]
        s_eff = complex(net.p_spec[i], net.q_spec[i]) + net.zip_imp[i] * v * v + net.zip_cur[i] * v
        y_load = -s_eff.conjugate()
        diag = False
        for e in range(int(yb.indptr[i]), int(yb.indptr[i + 1])):
            j = int(yb.indices[e])
            y = complex(yb.re[e], yb.im[e])
            if j == i:
                diag = True
                block(r, r, y + y_load)
            elif j in pos:
                block(r, pos[j], y)
        if not diag:
            block(r, r, y_load)
    return S.factor_host(2 * len(pq), rows, cols, vals) is None


def mark_unreferenced_islands(net: Network) -> None:
    """src/network.rs:142-223: a component without a slack bus is pinned to
    V = 0 as slack buses with no injection.  The reference does this at the
    start of Newton, after its linear guess; here it happens first (the GPU
    guess then covers the energized part only, which is the same system as
    long as the island rows are regular) and `guess_singular` records when
    they are not, so the solve starts from the given voltages instead, as
    the reference's does."""
    for comp in connected_components(net.ybus):
        if not np.any(net.bus_type[comp] == G.BUS_SLACK):
            net.islands.append(comp)
            if not net.guess_singular and _guess_block_singular(net, comp):
                net.guess_singular = True
            net.bus_type[comp] = G.BUS_SLACK
            net.vm[comp] = 0.0
            net.va[comp] = 0.0
            net.p_spec[comp] = 0.0
            net.q_spec[comp] = 0.0
            net.zip_imp[comp] = 0.0
            net.zip_cur[comp] = 0.0


def apply_batch_scenario(base: dict, scenario: dict) -> dict:
    """The reference tests' apply_batch_scenario (tests/common): every
    component listed in a scenario update overrides the base component of the
    same id, field by field."""
    doc = copy.deepcopy(base)
    for comp, updates in scenario.items():
        items = {int(x["id"]): x for x in doc["data"].get(comp, [])}
        for up in updates:
            if int(up["id"]) in items:
                items[int(up["id"])].update(up)
    return doc


def topology(gox, net: Network):
    """The network registered on the GPU: Y-bus, bus types, ZIP terms and the
    start-point rule (the linear guess unless the reference's would fail)."""
    topo = gox.Topology(net.ybus, net.bus_type)
    if np.any(net.zip_imp != 0) or np.any(net.zip_cur != 0):
        topo.set_zip(net.zip_imp, net.zip_cur)
    topo.set_initial_guess("given" if net.guess_singular else "linear")
    return topo


def solve(gox, net: Network, tol: float = 1e-6, max_iter: int = 20,
          precision: int | None = None):
    """One scenario of a converted network on the GPU: linear initial guess,
    then Newton-Raphson (FP64 unless `precision` says otherwise)."""
    topo = topology(gox, net)
    prec = gox.GOX_PRECISION_FP64 if precision is None else precision
    return topo.solve(net.p_spec[None], net.q_spec[None], net.vm, net.va, tol=tol,
                      max_iter=max_iter, precision=prec)


def from_grid(g: G.Grid, u_rated: float = 110e3, sk: float = 1e10, rx_ratio: float = 0.1,
              s_base: float = S_BASE_VA, freq_hz: float = FREQ_HZ) -> dict:
    """A generated grid as a power-grid-model input document, so that the
    PGM path (`PowerFlowModel.from_pgm_json`, the reference's
    scripts/bench/bench_batch.py workflow) can load it.  Every node is rated
    `u_rated`; lines keep r, x and charging; a transformer becomes a PGM
    transformer with the same series impedance (uk = |z|, pk = r s_base,
    sn = s_base) and its off-nominal ratio as one tap step, its charging as
    two shunts (b/2k^2 at the tapped end, b/2 at the other); PQ buses carry
    their net injection as a constant-power load, PV buses as a generator
    under a voltage regulator at their set-point; the slack bus becomes the
    node of a source at its set-point with short-circuit power `sk` (its
    virtual bus is the slack, so the grid's slack bus turns PQ)."""
    zb = u_rated * u_rated / s_base
    omega = 2.0 * math.pi * freq_hz
    next_id = [g.n_bus]

    def new_id():
        next_id[0] += 1
        return next_id[0]

    node = [{"id": i + 1, "u_rated": u_rated} for i in range(g.n_bus)]
    line, transformer, shunt, sym_load, sym_gen, source, regulator = [], [], [], [], [], [], []
    for b in range(g.n_branch):
        f, t = int(g.br_from[b]) + 1, int(g.br_to[b]) + 1
        r, x, bc = float(g.br_r[b]), float(g.br_x[b]), float(g.br_b[b])
        if not g.br_is_trafo[b]:
            line.append({"id": new_id(), "from_node": f, "to_node": t, "from_status": 1,
                         "to_status": 1, "r1": r * zb, "x1": x * zb, "c1": bc / (omega * zb),
                         "tan1": 0.0, "r0": r * zb, "x0": x * zb, "c0": bc / (omega * zb),
                         "tan0": 0.0})
            continue
        k = float(g.br_tap[b])
        transformer.append({"id": new_id(), "from_node": f, "to_node": t, "from_status": 1,
                            "to_status": 1, "u1": u_rated, "u2": u_rated, "sn": s_base,
                            "uk": math.hypot(r, x), "pk": r * s_base, "i0": 0.0, "p0": 0.0,
                            "winding_from": 0, "winding_to": 0, "clock": 0, "tap_side": 0,
                            "tap_pos": 1, "tap_min": 0, "tap_max": 1, "tap_nom": 0,
                            "tap_size": (k - 1.0) * u_rated})
        if bc != 0.0:
            base_y = s_base / (u_rated * u_rated)
            for nd, y in ((f, bc / 2.0 / (k * k)), (t, bc / 2.0)):
                shunt.append({"id": new_id(), "node": nd, "status": 1, "g1": 0.0, "b1": y * base_y,
                              "g0": 0.0, "b0": 0.0})
    for i in range(g.n_bus):
        bt = int(g.bus_type[i])
        if bt == G.BUS_PQ:
            sym_load.append({"id": new_id(), "node": i + 1, "status": 1, "type": 0,
                             "p_specified": -float(g.p_spec[i]) * s_base,
                             "q_specified": -float(g.q_spec[i]) * s_base})
        elif bt == G.BUS_PV:
            gid = new_id()
            sym_gen.append({"id": gid, "node": i + 1, "status": 1, "type": 0,
                            "p_specified": float(g.p_spec[i]) * s_base, "q_specified": 0.0})
            regulator.append({"id": new_id(), "regulated_object": gid, "status": 1,
                              "u_ref": float(g.vm[i])})
        else:
            source.append({"id": new_id(), "node": i + 1, "status": 1, "u_ref": float(g.vm[i]),
                           "sk": sk, "rx_ratio": rx_ratio, "z01_ratio": 1.0})
    data = {"node": node, "line": line, "transformer": transformer, "shunt": shunt,
            "sym_load": sym_load, "sym_gen": sym_gen, "source": source,
            "voltage_regulator": regulator}
    return {"version": "1.0", "type": "input", "is_batch": False, "attributes": {}, "data": data}
