"""Full-size parity: the benchmark workloads' committed counts (recomputed by
the CPU oracle when the fixtures were made, tests/golden/make_workloads.py)
against the CUDA path, batched and plain, at the benchmark graph sizes."""
import json
from pathlib import Path

import numpy as np
import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, Plan
from clustersm_gb300.workloads import load

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"


def available(name):
    return (GOLD / f"workload_{name}.json").exists()


@pytest.mark.parametrize("name", ["er1k", "rmat20", "rmat22"])
def test_workload_counts(ctx, name):
    if not available(name):
        pytest.skip(f"workload_{name}.json not generated")
    wl = load(name)
    queries, want, meta = wl.queries()
    assert all(w is not None for w in want)
    host = wl.graph()
    dev = DeviceGraph(ctx, host)
    plans = [Plan(q) for q in queries]
    counts, st = native.match_batch(ctx, dev, plans)
    assert counts.tolist() == want
    assert st.total_embeddings == sum(want)
    # plain path on a spread sample
    idx = np.linspace(0, len(plans) - 1, num=min(24, len(plans))).astype(int)
    for i in idx:
        res, _ = native.match(ctx, dev, plans[i])
        assert res.count == want[i], (name, i)
    # split the batch in two: counts do not depend on what else is in the batch
    half = len(plans) // 2
    c1, _ = native.match_batch(ctx, dev, plans[:half])
    c2, _ = native.match_batch(ctx, dev, plans[half:])
    assert c1.tolist() + c2.tolist() == want


def test_wide_workload_counts(ctx):
    """The 4..7-vertex queries of the 2^22 graph (up to 10^9 embeddings each,
    every count recomputed by the CPU oracle): batched, batched at a
    breadth-first depth of 2, and plain on a spread sample."""
    if not available("rmat22_k4to7"):
        pytest.skip("workload_rmat22_k4to7.json not generated")
    wl = load("rmat22_k4to7")
    queries, want, meta = wl.queries()
    assert sorted({q["k"] for q in meta["queries"]}) == [4, 5, 6, 7]
    dev = DeviceGraph(ctx, wl.graph())
    plans = [Plan(q) for q in queries]
    counts, st = native.match_batch(ctx, dev, plans)
    assert counts.tolist() == want
    counts2, _ = native.match_batch(ctx, dev, plans, bfs_depth=2)
    assert counts2.tolist() == want
    for i in np.linspace(0, len(plans) - 1, num=8).astype(int):
        assert native.match(ctx, dev, plans[i])[0].count == want[i], i


def test_workload_fixture_meta():
    for name in ["er1k", "rmat20", "rmat22", "rmat22_k4to7", "rmat24_k4to7"]:
        if not available(name):
            continue
        meta = json.loads((GOLD / f"workload_{name}.json").read_text())
        assert meta["queries"], name
        assert all("count" in q for q in meta["queries"])
        assert "oracle" in meta.get("verified_by", "")
