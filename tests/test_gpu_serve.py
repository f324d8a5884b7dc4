"""Serving: continuous batching over one resident graph.  Every response's
count equals the query's count alone (plain path) and the committed oracle
count, whether it ran alone or in a mix, and requests submitted while others
are on the device join the running work."""
import time

import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, Plan, Server
from clustersm_gb300.workloads import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def er(ctx):
    wl = load("er1k")
    qs, want, _ = wl.queries()
    host = wl.graph()
    return DeviceGraph(ctx, host), [Plan(q) for q in qs], want


def test_alone_equals_in_mix(ctx, er):
    dev, plans, want = er
    srv = Server(ctx, dev, max_inflight=16)
    t = srv.submit(plans[0])
    srv.drain()
    alone = srv.poll(t)
    assert alone.status == 0 and alone.count == want[0]
    tickets = [srv.submit(p) for p in plans]
    srv.drain()
    for tk, w in zip(tickets, want):
        r = srv.poll(tk)
        assert r.status == 0 and r.count == w
        assert r.finish_s >= r.start_s >= r.submit_s
    srv.close()


@pytest.fixture(scope="module")
def rmat22(ctx):
    wl = load("rmat22")
    try:
        qs, want, _ = wl.queries()
    except FileNotFoundError:
        pytest.skip("rmat22 workload not generated")
    return DeviceGraph(ctx, wl.graph()), [Plan(q) for q in qs[:96]], want[:96]


@pytest.mark.parametrize("live", ["1", "0"])
def test_arrivals_while_running(ctx, rmat22, monkeypatch, live):
    """Requests submitted while others run: admitted into the running slice
    (default), or between slices (SMG_SERVE_LIVE=0); counts exact either way."""
    dev, plans, want = rmat22
    monkeypatch.setenv("SMG_SERVE_LIVE", live)
    srv = Server(ctx, dev, max_inflight=32)
    tickets = []
    for i, p in enumerate(plans):
        tickets.append(srv.submit(p))
        if i % 8 == 7:
            srv.step()  # non-blocking: admits, launches or retires
    srv.drain()
    results = [srv.poll(tk) for tk in tickets]
    ss = srv.stats()
    srv.close()
    for r, w in zip(results, want):
        assert r.status == 0 and r.count == w
    if live == "0":
        assert ss.admitted_live == 0
    for p, w in list(zip(plans, want))[:8]:
        res, _ = native.match(ctx, dev, p)
        assert res.count == w


@pytest.mark.parametrize("slice_ms,min_ms,live", [("0.3", "0.1", "1"), ("0.3", "0.1", "0"), ("250", "0.2", "0"),
                                                  ("250", "0.2", "1")])
def test_preempted_slices_keep_counts(ctx, rmat22, monkeypatch, slice_ms, min_ms, live):
    """Sub-millisecond slices (every warp's stack is handed over to the next
    queue hundreds of times), doorbell-driven closings (arrivals while slots
    are free) and admission into running slices leave every count exact."""
    dev, plans, want = rmat22
    monkeypatch.setenv("SMG_SLICE_MS", slice_ms)
    monkeypatch.setenv("SMG_SLICE_MIN_MS", min_ms)
    monkeypatch.setenv("SMG_SERVE_LIVE", live)
    srv = Server(ctx, dev, max_inflight=24)
    tickets = []
    for i, p in enumerate(plans):
        tickets.append(srv.submit(p))
        for _ in range(4):
            srv.step()
        if i % 16 == 15:
            time.sleep(0.002)
    srv.drain()
    results = [srv.poll(tk) for tk in tickets]
    ss = srv.stats()
    srv.close()
    assert ss.admitted == len(plans) and ss.slices >= 1
    if live == "0":
        assert ss.admitted_live == 0
    assert [r.status for r in results] == [0] * len(plans)
    assert [int(r.count) for r in results] == [int(w) for w in want]


def test_cancel_and_budget(ctx, er):
    dev, plans, want = er
    srv = Server(ctx, dev, max_inflight=2)
    ts = [srv.submit(p) for p in plans[:6]]
    srv.cancel(ts[-1])
    srv.drain()
    assert srv.poll(ts[-1]).status == 11  # SMG_ERR_CANCELLED
    assert all(srv.poll(t).count == w for t, w in zip(ts[:-1], want[:5]))
    small = Server(ctx, dev, memory_budget_bytes=1024)
    with pytest.raises(native.SmgError) as e:
        small.submit(plans[0])
    assert e.value.status == 10  # SMG_ERR_BUDGET


def test_query_size_limit(ctx, er):
    """A server built for queries of at most 4 vertices (smaller task records,
    more resident warps) serves them exactly and rejects larger ones."""
    dev, plans, want = er
    srv = Server(ctx, dev, max_inflight=16, max_query_vertices=4)
    tickets = [srv.submit(p) for p in plans[:12]]
    big = Plan(native.Query([0, 1, 2, 3, 0], [0, 1, 1, 2, 2, 3, 3, 4]))
    with pytest.raises(native.SmgError) as e:
        srv.submit(big)
    assert e.value.status == 5  # SMG_ERR_LIMIT
    srv.drain()
    assert [int(srv.poll(t).count) for t in tickets] == [int(w) for w in want[:12]]
    with pytest.raises(native.SmgError) as e:  # a result is collected once
        srv.poll(tickets[0])
    assert e.value.status == 1  # SMG_ERR_INVALID
    srv.close()
