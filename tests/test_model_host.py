"""PowerFlowModel (src/python.rs:99-478) on the host side: loading a PGM
file, the inspection methods that need no solve, and argument errors."""
import os

import numpy as np
import pytest

import gridoxide_gb300 as gox
from gridoxide_gb300 import pgm
from helpers import GOLDEN


def _path(case):
    return os.path.join(GOLDEN, "pgm", case, "input.json")


def test_model_inspection():
    m = gox.PowerFlowModel.from_pgm_json(_path("transmission-case"))
    doc = pgm.load(_path("transmission-case"))
    net = pgm.convert(doc)
    assert m.n_nodes == len(doc["data"]["node"]) + len(doc["data"]["source"]) == net.n_bus
    rows, cols, g, b = m.ybus_triplets()
    assert rows == np.repeat(np.arange(net.n_bus), np.diff(net.ybus.indptr)).tolist()
    assert cols == net.ybus.indices.tolist() and g == net.ybus.re.tolist() and b == net.ybus.im.tolist()
    kinds, p, q = m.bus_spec()
    assert kinds[-1] == 0 and set(kinds[:-1]) <= {1, 2}
    assert p == net.p_spec.tolist() and q == net.q_spec.tolist()
    assert m.zip_term_counts() == [0] * m.n_nodes
    assert m.voltage_mag() == net.vm.tolist()      # before the first solve: the template
    assert gox.PowerFlowModel.default_threads() >= 1
    assert m.solve_batch([]) == [] and m.solve_batch_scaled([]) == []


def test_model_bus_spec_keeps_islands_unmarked():
    m = gox.PowerFlowModel.from_pgm_json(_path("basic-node"))
    kinds, _, _ = m.bus_spec()
    assert kinds == [2, 2, 0]      # node_2 has no source but stays PQ in the template


def test_model_zip_counts_and_kv():
    m = gox.PowerFlowModel.from_pgm_json(_path("sym_load"))
    doc = pgm.load(_path("sym_load"))
    assert sum(m.zip_term_counts()) == sum(1 for ld in doc["data"]["sym_load"]
                                           if ld["status"] and ld.get("type", 0) in (1, 2))
    u = {n["id"]: n["u_rated"] for n in doc["data"]["node"]}
    kv = m.voltage_kv()
    for nid, k in pgm.node_id_to_idx(doc["data"]).items():
        assert kv[k] == pytest.approx(u[nid] / 1e3)


def test_model_errors(tmp_path):
    with pytest.raises(ValueError):
        gox.PowerFlowModel.from_pgm_json(_path("line"), backend="cuda")
    with pytest.raises(RuntimeError):
        gox.PowerFlowModel.from_pgm_json(str(tmp_path / "missing.json"))
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    with pytest.raises(ValueError):
        gox.PowerFlowModel.from_pgm_json(str(bad))
    m = gox.PowerFlowModel.from_pgm_json(_path("line"))
    with pytest.raises(RuntimeError):
        m.solve_batch([[(m.n_nodes, 0.1, 0.0)]])
