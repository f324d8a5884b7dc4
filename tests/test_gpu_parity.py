"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bit-exact: initial candidate masks, the cluster bitmap and final candidate
masks against the oracle's restatement of filter.cu; uint64 counts and sorted
embedding sets against the backtracking oracle.  Plain and batched paths must
agree.
"""
import numpy as np
import pytest

import oracle
from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, HostGraph, Plan, Query

pytestmark = pytest.mark.gpu

EXAMPLE_EMBEDDINGS = [(0, 1, 4, 2, 3), (4, 1, 0, 2, 3), (5, 8, 7, 9, 10), (7, 8, 5, 9, 10)]
BUDGET = 3_000_000  # oracle partial matches per query (keeps the CPU side short)


@pytest.fixture(scope="module")
def er(ctx):
    g = HostGraph.er(1000, 4000, 4, seed=1)
    return g, DeviceGraph(ctx, g)


@pytest.fixture(scope="module")
def rmat(ctx):
    g = HostGraph.rmat(12, 16, 8, seed=7)
    return g, DeviceGraph(ctx, g)


ER_SHAPES = ("tree", "sparse", "induced")          # ER 1k/4k has (almost) no dense walks
RMAT_SHAPES = ("tree", "sparse", "dense", "induced")


def small_queries(g, shapes=ER_SHAPES, ks=(4, 5, 6, 7, 8), seeds=range(4)):
    out = []
    for shape in shapes:
        for k in ks:
            for s in seeds:
                try:
                    out.append(Query.generate(g, k, shape, seed=1000 * k + s))
                except native.SmgError:  # no walk of that shape exists (dense on sparse graphs)
                    pass
    return out


def test_example(ctx, example):
    g, q = example
    dg = DeviceGraph(ctx, g)
    plan = Plan(q)
    res, emb = native.match(ctx, dg, plan, emit=16)
    assert res.count == 4
    assert res.embeddings_written == 4 and res.overflow == 0
    rows = sorted(tuple(r) for r in emb.tolist())
    assert rows == EXAMPLE_EMBEDDINGS


def check_filter(ctx, host, dev, q):
    plan = Plan(q)
    vm, enc, cm = native.filter_inspect(ctx, dev, plan)
    ovm = oracle.nlc_filter(host, plan)
    oenc, ocm = oracle.encode(host, plan, ovm)
    assert np.array_equal(vm, ovm), "initial candidate masks differ"
    assert np.array_equal(enc, oenc), "cluster bitmaps differ"
    assert np.array_equal(cm, ocm), "final candidate masks differ"
    return plan, ocm


@pytest.mark.parametrize("shape", ["tree", "sparse", "induced"])
def test_filter_bit_exact_er(ctx, er, shape):
    host, dev = er
    for q in small_queries(host, shapes=(shape,), ks=(4,), seeds=range(12)):
        check_filter(ctx, host, dev, q)


@pytest.mark.parametrize("shape", ["tree", "sparse", "dense"])
def test_filter_bit_exact_rmat(ctx, rmat, shape):
    host, dev = rmat
    for q in small_queries(host, shapes=(shape,), ks=(4, 6, 8, 10, 12, 16), seeds=range(3)):
        check_filter(ctx, host, dev, q)


def budgeted(host, q):
    c, used = oracle.count_budget(host, q, BUDGET)
    return None if used is None else c


@pytest.mark.parametrize("which", ["er", "rmat"])
def test_counts_match_oracle(ctx, er, rmat, which):
    host, dev = er if which == "er" else rmat
    checked = 0
    shapes = RMAT_SHAPES if which == "rmat" else ER_SHAPES
    for q in small_queries(host, shapes=shapes, ks=(4, 5, 6) if which == "rmat" else (4, 5, 6, 8), seeds=range(3)):
        want = budgeted(host, q)
        if want is None:
            continue
        res, _ = native.match(ctx, dev, Plan(q))
        assert res.count == want, (q.to_dict(), res.count, want)
        checked += 1
    assert checked >= 10


def test_batch_equals_plain(ctx, er):
    host, dev = er
    qs = small_queries(host, ks=(4, 6, 8), seeds=range(3))
    plans = [Plan(q) for q in qs]
    counts, st = native.match_batch(ctx, dev, plans)
    for p, c in zip(plans, counts):
        res, _ = native.match(ctx, dev, p)
        assert res.count == int(c)
    assert st.total_embeddings == int(counts.sum())


def test_embeddings_equal_oracle(ctx, er):
    host, dev = er
    for q in small_queries(host, ks=(4, 5), seeds=range(2)):
        want = budgeted(host, q)
        if want is None or want > 200000:
            continue
        cnt, rows = oracle.embeddings(host, q, max_rows=want + 1)
        res, emb = native.match(ctx, dev, Plan(q), emit=want + 1)
        assert res.count == cnt and res.embeddings_written == cnt and not res.overflow
        got = emb[np.lexsort(emb.T[::-1])]
        assert np.array_equal(got, rows)


def test_emit_overflow_keeps_exact_count(ctx, er):
    host, dev = er
    q = Query.generate(host, 4, "tree", seed=3)
    full, _ = native.match(ctx, dev, Plan(q))
    assert full.count > 8
    res, emb = native.match(ctx, dev, Plan(q), emit=8)
    assert res.count == full.count and res.overflow == 1 and res.embeddings_written == 8


def test_edge_cases(ctx, er):
    host, dev = er
    # a label absent from the data graph: no candidate, count 0
    res, _ = native.match(ctx, dev, Plan(Query([0, 7], [0, 1])))
    assert res.count == 0
    # a single edge: ordered pairs of adjacent vertices with those labels
    lab = host.labels()
    off, adj = host.offsets().astype(np.int64), host.neighbors()
    want = sum(1 for v in range(host.n) for w in adj[off[v]:off[v + 1]] if lab[v] == 0 and lab[w] == 1)
    res, _ = native.match(ctx, dev, Plan(Query([0, 1], [0, 1])))
    assert res.count == want
    # triangle of one label
    q = Query([2, 2, 2], [0, 1, 1, 2, 2, 0])
    res, _ = native.match(ctx, dev, Plan(q))
    assert res.count == oracle.count(host, q)


def test_graph_with_isolated_vertices(ctx):
    g = HostGraph.from_arrays([0, 1, 2, 2, 2], [1, 0], [0, 0, 0, 0])
    dev = DeviceGraph(ctx, g)
    res, emb = native.match(ctx, dev, Plan(Query([0, 0], [0, 1])), emit=4)
    assert res.count == 2
    assert sorted(tuple(r) for r in emb.tolist()) == [(0, 1), (1, 0)]


def test_batch_graph_replay(ctx, er):
    host, dev = er
    plans = [Plan(q) for q in small_queries(host, ks=(4, 6), seeds=range(3))]
    first, _ = native.match_batch(ctx, dev, plans)             # captured
    again, _ = native.match_batch(ctx, dev, plans)             # replayed
    profiled, st = native.match_batch(ctx, dev, plans, profile=True)
    native.match(ctx, dev, plans[0])                           # invalidates the graph
    after, _ = native.match_batch(ctx, dev, plans)             # re-staged and recaptured
    direct, _ = native.match_batch(ctx, dev, plans, use_graph=False)
    assert first.tolist() == again.tolist() == profiled.tolist() == after.tolist() == direct.tolist()
    assert st.join_ms > 0 and st.kernel_launches > 0


PLAN_ORDER_SCRIPT = r"""
import sys
sys.path.insert(0, sys.argv[1])
from clustersm_gb300 import native
from clustersm_gb300.native import Context, DeviceGraph, Plan
from clustersm_gb300.workloads import load
wl = load("er1k")
qs, want, _ = wl.queries()
ctx = Context(0)
dev = DeviceGraph(ctx, wl.graph())
counts, _ = native.match_batch(ctx, dev, [Plan(q) for q in qs])
bad = [i for i, (c, w) in enumerate(zip(counts.tolist(), want)) if int(c) != int(w)]
print("mismatches", bad)
sys.exit(1 if bad else 0)
"""


@pytest.mark.parametrize("mode", ["plan", "greedy"])
def test_other_join_orders_give_same_counts(ctx, mode):
    """SMG_JOIN_ORDER=plan matches vertices in the order the reference's edge
    order (order.cpp getBFSEdgeOrder) reaches them, =greedy in the cost-based
    order without the counted ending; the counts are the same (the setting is
    read once per process)."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, SMG_JOIN_ORDER=mode)
    r = subprocess.run([sys.executable, "-c", PLAN_ORDER_SCRIPT, str(root)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.parametrize("min_degree,enabled,rank_rows", [("1", "1", "1"), ("1", "1", "0"), ("64", "0", "1")])
def test_label_index_every_vertex_or_none(ctx, monkeypatch, min_degree, enabled, rank_rows):
    """The label index (neighbour lists ordered by label, with per-label run
    tables) given to every vertex, and left out; with every vertex indexed,
    the candidate tests of label-run entries by rank (the default) and by id:
    cluster bitmaps stay bit-exact and counts equal the oracle's either way.
    The settings are read when a graph is uploaded."""
    monkeypatch.setenv("SMG_LABEL_INDEX_MIN_DEGREE", min_degree)
    monkeypatch.setenv("SMG_LABEL_INDEX", enabled)
    monkeypatch.setenv("SMG_RANK_ROWS", rank_rows)
    host = HostGraph.rmat(12, 16, 8, seed=7)
    dev = DeviceGraph(ctx, host)
    checked = 0
    for q in small_queries(host, shapes=RMAT_SHAPES, ks=(4, 5, 6, 8), seeds=range(2)):
        plan, _ = check_filter(ctx, host, dev, q)
        want = budgeted(host, q)
        if want is None:
            continue
        res, _ = native.match(ctx, dev, plan)
        assert res.count == want, (q.to_dict(), res.count, want)
        checked += 1
    assert checked >= 8
    dev.free()


@pytest.mark.parametrize("layout", ["label", "id"])
def test_hub_bitmap_layouts(ctx, monkeypatch, layout):
    """Hub neighbour bitmaps laid out by (label, rank) and by id, with every
    vertex of degree >= 16 a hub: counts equal the oracle's either way (the
    settings are read when a graph is uploaded)."""
    monkeypatch.setenv("SMG_HUB_MIN_DEGREE", "16")
    monkeypatch.setenv("SMG_HUB_LAYOUT", layout)
    host = HostGraph.rmat(12, 16, 8, seed=7)
    dev = DeviceGraph(ctx, host)
    checked = 0
    for q in small_queries(host, shapes=RMAT_SHAPES, ks=(4, 5, 6), seeds=range(3)):
        want = budgeted(host, q)
        if want is None:
            continue
        res, _ = native.match(ctx, dev, Plan(q))
        assert res.count == want, (layout, q.to_dict(), res.count, want)
        checked += 1
    assert checked >= 10
    dev.free()


def test_memory_bounded_chunks(ctx, monkeypatch):
    """A batch whose state does not fit the memory cap runs as several
    chunks (each its own filter pass and join launch) with the same counts."""
    host = HostGraph.rmat(12, 16, 8, seed=7)
    dev = DeviceGraph(ctx, host)
    plans = [Plan(q) for q in small_queries(host, shapes=RMAT_SHAPES, ks=(4, 5), seeds=range(3))]
    whole, st1 = native.match_batch(ctx, dev, plans, use_graph=False)
    assert st1.chunks == 1
    # below a chunk's fixed part (queue bound and join buffers): one query per chunk
    monkeypatch.setenv("SMG_MAX_BATCH_BYTES", str(256 << 20))
    parts, st2 = native.match_batch(ctx, dev, plans, use_graph=False)
    assert st2.chunks > 1
    assert parts.tolist() == whole.tolist()
    dev.free()


def test_model_counter_leaves_counts(ctx):
    """SMG_FLAG_MODEL counts the breadth-first byte model and changes no count;
    without the flag the model reads 0.  For a 2-vertex query (one edge u-w)
    the model is exact by hand: every root v is a row of one vertex, written
    (4 B) and expanded along its own list (4 B read + 8 B offsets + 8 B per
    entry), with no complete row written."""
    from clustersm_gb300.native import HostGraph
    host = HostGraph.er(1000, 4000, 4, seed=1)
    dev = DeviceGraph(ctx, host)
    qs = []
    for k in (3, 4, 5):
        for sh in ("tree", "sparse"):
            try:
                qs.append(Query.generate(host, k, sh, seed=40 + k))
            except native.SmgError:
                pass  # no walk of that shape from this seed
    assert len(qs) >= 3
    plans = [Plan(q) for q in qs]
    c0, s0 = native.match_batch(ctx, dev, plans)
    c1, s1 = native.match_batch(ctx, dev, plans, model=True)
    assert c0.tolist() == c1.tolist() and s0.model_bytes == 0 and s1.model_bytes > 0
    edge = Plan(Query([1, 1], [0, 1]))  # both ends alike: either may be the join's first vertex
    _, se = native.match_batch(ctx, dev, [edge], model=True)
    roots = np.nonzero(native.filter_inspect(ctx, dev, edge)[2] & 1)[0]
    deg = np.diff(host.offsets().astype(np.int64))
    assert se.model_bytes == sum(4 + 4 + 8 + 8 * int(deg[v]) for v in roots)
