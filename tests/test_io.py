"""The .in reader/writer (io.cu:24-108 dialect) and its error behaviour."""
import numpy as np
import pytest

from clustersm_gb300.native import HostGraph, Query, SmgError


def test_example_graph(example):
    g, q = example
    assert (g.n, g.m) == (11, 13)
    assert q.k == 5 and len(q.edges) == 10
    # neighbour lists keep file order (io.cu:86-93)
    off = g.offsets()
    assert g.neighbors()[off[1]:off[2]].tolist() == [0, 2, 4]
    assert q.labels.tolist() == [0, 0, 0, 1, 2]


def test_roundtrip(tmp_path):
    g = HostGraph.er(200, 600, 5, seed=3)
    p = tmp_path / "g.in"
    g.write(p)
    h = HostGraph.read(p).sorted_copy()
    assert np.array_equal(h.offsets(), g.offsets())
    assert np.array_equal(h.neighbors(), g.neighbors())
    assert np.array_equal(h.labels(), g.labels())
    q = Query.generate(g, 6, "sparse", seed=9)
    qp = tmp_path / "q.in"
    q.write(qp)
    r = Query.read(qp)
    assert r.edges.tolist() == q.edges.tolist() and r.labels.tolist() == q.labels.tolist()


@pytest.mark.parametrize("text,status", [
    ("x 2 1\n", 3),                                  # no 't' header
    ("t 2 1\nv 0 0 1\nv 1 0 1\ne 0 5\n", 3),         # endpoint out of range
    ("t 2 1\nv 0 0 2\nv 1 0 1\ne 0 1\n", 3),         # declared degree differs
    ("t 2 1\nv 0 0 0\nv 1 0 0\ne 1 1\n", 3),         # self-loop
    ("t 2 2\nv 0 0 2\nv 1 0 2\ne 0 1\ne 1 0\n", 3),  # repeated edge
    ("t 3 1\nv 0 0 1\nv 1 0 1\ne 0 1\n", 3),         # missing 'v' line
    ("t 2 2\nv 0 0 1\nv 1 0 1\ne 0 1\n", 3),         # edge count differs
])
def test_malformed(tmp_path, text, status):
    p = tmp_path / "bad.in"
    p.write_text(text)
    with pytest.raises(SmgError) as e:
        HostGraph.read(p)
    assert e.value.status == status


def test_missing_file(tmp_path):
    with pytest.raises(SmgError) as e:
        HostGraph.read(tmp_path / "nope.in")
    assert e.value.status == 2


def test_from_arrays_rejects_asymmetric():
    with pytest.raises(SmgError):
        HostGraph.from_arrays([0, 1, 1], [1], [0, 0])
