"""Islands of outage scenarios on the host (gox_outage_islands, after
network::connected_components / classify, src/network.rs:121-194): an
outage splits the grid exactly when its branch is a bridge; the components
and their verdicts equal a plain graph search on the Y-bus pattern without
that branch."""
import numpy as np
from scipy.sparse import csr_matrix
from scipy.sparse.csgraph import connected_components

import gridoxide_gb300 as gox
from gridoxide_gb300 import grids as G


def test_outage_islands_match_graph_search():
    g = G.config_grid("case118")
    yb = G.build_ybus(g)
    topo = gox.Topology(yb, g.bus_type)
    br = np.arange(g.n_branch)
    out = G.outage_deltas(g, yb, br)
    nis, lab, ver = topo.outage_islands(out)
    bridge = G.bridges(g)
    assert bridge.any() and not bridge.all()
    np.testing.assert_array_equal(nis == 2, bridge)
    assert np.all(nis[~bridge] == 1) and np.all(lab[~bridge] == 0) and np.all(ver[~bridge] == 0)
    rows = np.repeat(np.arange(yb.n), np.diff(yb.indptr))
    for b in np.flatnonzero(bridge):
        f, t = int(g.br_from[b]), int(g.br_to[b])
        keep = ~(((rows == f) & (yb.indices == t)) | ((rows == t) & (yb.indices == f)))
        a = csr_matrix((np.ones(keep.sum()), (rows[keep], yb.indices[keep])), shape=(yb.n, yb.n))
        nc, ref = connected_components(a, directed=False)
        assert nc == 2
        # same partition, labelled in order of each component's smallest bus
        first = {c: np.flatnonzero(ref == c)[0] for c in range(nc)}
        order = sorted(range(nc), key=lambda c: first[c])
        np.testing.assert_array_equal(lab[b], np.array([order.index(c) for c in ref]))
        slack_comp = lab[b][np.flatnonzero(g.bus_type == G.BUS_SLACK)[0]]
        np.testing.assert_array_equal(ver[b], np.where(lab[b] == slack_comp, 0, 1))
