"""Breadth-first levels before the depth-first join (smg_match_opts.bfs_depth):
a warp queues every partial match of the first levels as a task instead of
descending into it.  The reference joins every level breadth-first
(join.cu:290-435); the set of embeddings does not depend on where the join
turns depth-first, so every count must equal the oracle's (exact, integers)
and the embedding sets must be the same rows."""
import numpy as np
import pytest

import oracle
from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, HostGraph, Plan, Query
from clustersm_gb300.workloads import load

pytestmark = pytest.mark.gpu

BUDGET = 3_000_000  # oracle partial matches per query


def drawn(host, shapes, ks, seeds):
    out = []
    for shape in shapes:
        for k in ks:
            for s in seeds:
                try:
                    out.append(Query.generate(host, k, shape, seed=7000 + 100 * k + s))
                except native.SmgError:
                    pass
    return out


@pytest.mark.parametrize("which", ["er", "rmat"])
def test_bfs_depths_match_oracle(ctx, which):
    """Queries of 4..8 vertices, batched at depths 0..5 (depths past the last
    two levels are clamped): every count equals the oracle's."""
    if which == "er":
        host = HostGraph.er(1000, 4000, 4, seed=1)
        shapes = ("tree", "sparse", "induced")
    else:
        host = HostGraph.rmat(12, 16, 8, seed=7)
        shapes = ("tree", "sparse", "dense")
    dev = DeviceGraph(ctx, host)
    qs, want = [], []
    for q in drawn(host, shapes, (4, 5, 6, 8), range(3)):
        c, used = oracle.count_budget(host, q, BUDGET)
        if used is not None:
            qs.append(q)
            want.append(c)
    assert len(qs) >= 12
    plans = [Plan(q) for q in qs]
    queued = []
    for depth in range(6):
        counts, st = native.match_batch(ctx, dev, plans, bfs_depth=depth)
        assert counts.tolist() == want, (which, depth)
        queued.append(st.bfs_tasks)
    assert queued[0] == 0
    assert all(b > 0 for b in queued[1:]), queued


def test_bfs_embeddings_equal_oracle(ctx):
    """Plain path with embeddings at depth 2: the same sorted rows as the
    oracle's."""
    host = HostGraph.er(1000, 4000, 4, seed=1)
    dev = DeviceGraph(ctx, host)
    checked = 0
    for q in drawn(host, ("sparse", "induced"), (4, 5, 6), range(2)):
        want, rows = oracle.embeddings(host, q, max_rows=1 << 16)
        if want > (1 << 16):
            continue
        res, emb = native.match(ctx, dev, Plan(q), emit=1 << 16, bfs_depth=2)
        assert res.count == want
        got = sorted(tuple(r) for r in emb.tolist())
        assert got == [tuple(r) for r in rows.tolist()]
        checked += 1
    assert checked >= 4


@pytest.mark.parametrize("depth", [2, 3])
def test_bfs_workload_rmat20(ctx, depth):
    """The 2^20-vertex workload's committed (oracle-verified) counts at
    breadth-first depths 2 and 3, batched and on the plain path."""
    wl = load("rmat20")
    qs, want, _ = wl.queries()
    dev = DeviceGraph(ctx, wl.graph())
    plans = [Plan(q) for q in qs]
    counts, st = native.match_batch(ctx, dev, plans, bfs_depth=depth)
    assert counts.tolist() == want
    assert st.bfs_tasks > 0
    idx = np.linspace(0, len(plans) - 1, num=8).astype(int)
    for i in idx:
        assert native.match(ctx, dev, plans[i], bfs_depth=depth)[0].count == want[i]
