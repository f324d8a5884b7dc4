"""Failure paths without a GPU fault: the join's device-side time limit
(SMG_TIME_LIMIT_S, read on every call) runs out on heavy queries, every wait
in the persistent kernel gives up, and the call returns SMG_ERR_TIMEOUT for
smg_match, smg_match_batch and the server's requests.  The context stays
usable: with the limit lifted, the same context counts the same queries
exactly.  The reference instead exits the process on any CUDA error
(cuda_helpers.h:27-32)."""
import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, Plan, Server, SmgError
from clustersm_gb300.workloads import load

pytestmark = pytest.mark.gpu

TIMEOUT = 8  # SMG_ERR_TIMEOUT


@pytest.fixture(scope="module")
def heavy(ctx):
    wl = load("rmat20")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    idx = sorted(range(len(qs)), key=lambda i: -counts[i])[:8]
    return DeviceGraph(ctx, host), [Plan(qs[i]) for i in idx], [counts[i] for i in idx]


def test_match_time_limit(ctx, heavy, monkeypatch):
    dev, plans, want = heavy
    monkeypatch.setenv("SMG_TIME_LIMIT_S", "0.000001")
    with pytest.raises(SmgError) as e:
        native.match(ctx, dev, plans[0])
    assert e.value.status == TIMEOUT
    monkeypatch.delenv("SMG_TIME_LIMIT_S")
    assert native.match(ctx, dev, plans[0])[0].count == want[0]


def test_batch_time_limit(ctx, heavy, monkeypatch):
    dev, plans, want = heavy
    monkeypatch.setenv("SMG_TIME_LIMIT_S", "0.000001")
    for use_graph in (True, False):
        with pytest.raises(SmgError) as e:
            native.match_batch(ctx, dev, plans, use_graph=use_graph)
        assert e.value.status == TIMEOUT
    monkeypatch.delenv("SMG_TIME_LIMIT_S")
    counts, _ = native.match_batch(ctx, dev, plans)
    assert [int(c) for c in counts] == want


def test_server_time_limit(ctx, heavy, monkeypatch):
    dev, plans, want = heavy
    srv = Server(ctx, dev, max_inflight=16, memory_budget_bytes=8 << 30)
    monkeypatch.setenv("SMG_TIME_LIMIT_S", "0.000001")
    tickets = [srv.submit(p) for p in plans]
    srv.drain()
    res = [srv.poll(t) for t in tickets]
    assert all(r.status == TIMEOUT for r in res), [r.status for r in res]
    monkeypatch.delenv("SMG_TIME_LIMIT_S")
    tickets = [srv.submit(p) for p in plans]
    srv.drain()
    res = [srv.poll(t) for t in tickets]
    assert [r.status for r in res] == [0] * len(plans)
    assert [int(r.count) for r in res] == want
    srv.close()


def test_work_limit(ctx, heavy):
    """A per-query work limit (smg_match_opts.max_work) stops a heavy query
    without failing the call: the plain path reports limit_hit, the batch
    UINT64_MAX for that query, and the other queries of the batch stay exact."""
    dev, plans, want = heavy
    r, _ = native.match(ctx, dev, plans[0], max_work=1024)
    assert r.limit_hit == 1
    counts, _ = native.match_batch(ctx, dev, plans[:2], max_work=1024)
    assert [int(c) for c in counts] == [2**64 - 1] * 2
    counts, _ = native.match_batch(ctx, dev, plans[:2], max_work=1 << 40)
    assert [int(c) for c in counts] == want[:2]
