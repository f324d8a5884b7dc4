"""smg_join_noalloc: the allocation-free join for callers that cannot call
cudaMalloc while matching (code between another application's graph capture
and replay, framework-owned allocators, real-time loops).  Its counts must
equal the CPU oracle's (exact: the counts are integers) on two calls in a
row, with the inputs in device memory the caller owns (torch tensors here);
free device memory must not move across calls; a query that spends the
queue's slots must still count exactly; the time limit must come back as
SMG_ERR_TIMEOUT with the next call exact again.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import oracle
from clustersm_gb300 import native
from clustersm_gb300.native import Context, DeviceGraph, HostGraph, Plan, Query, check, lib
from clustersm_gb300.workloads import load

pytestmark = pytest.mark.gpu

MAX_TASKS = 65536  # SMG_NOALLOC_MAX_TASKS


def noalloc_status(ctx, dev, plan, cm_dev, roots_dev, n_roots):
    out = C.c_uint64()
    st = lib.smg_join_noalloc(ctx.handle, dev.handle, plan.handle, C.c_void_p(cm_dev.data_ptr()),
                              C.c_void_p(roots_dev.data_ptr()), n_roots, C.byref(out))
    return st, out.value


def noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n_roots):
    st, val = noalloc_status(ctx, dev, plan, cm_dev, roots_dev, n_roots)
    check(st, "smg_join_noalloc")
    return val


def inputs(torch, ctx, dev, plan):
    """Final candidate masks and root candidates in caller-owned device memory."""
    _, _, cm = native.filter_inspect(ctx, dev, plan)
    roots = np.nonzero((cm >> plan.view.root) & 1)[0].astype(np.int32)
    cm_dev = torch.from_numpy(cm.view(np.int32)).cuda()
    roots_dev = torch.from_numpy(roots if len(roots) else np.zeros(1, np.int32)).cuda()
    torch.cuda.synchronize()
    return cm_dev, roots_dev, len(roots)


def queue_use(device=0):
    out = (C.c_ulonglong * 3)()
    assert lib.smg_debug_noalloc_queue(device, out) == 0
    return out[0], out[1], out[2]


@pytest.mark.parametrize("graph", ["er", "rmat"])
def test_noalloc_matches_oracle(graph):
    torch = pytest.importorskip("torch")
    ctx = Context(0)
    if graph == "er":
        host = HostGraph.er(1000, 4000, 4, seed=1)
        shapes = ("tree", "sparse", "induced")
    else:
        host = HostGraph.rmat(12, 16, 8, seed=7)
        shapes = ("tree", "sparse", "dense")
    dev = DeviceGraph(ctx, host)
    checked = 0
    for shape in shapes:
        for s in range(3):
            q = Query.generate(host, 4 + s, shape, seed=500 + s)
            want, used = oracle.count_budget(host, q, 10**9)
            if used is None:
                continue
            plan = Plan(q)
            cm_dev, roots_dev, n = inputs(torch, ctx, dev, plan)
            first = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n)
            second = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n)
            assert first == second == want, (graph, shape, s)
            checked += 1
    assert checked >= 4
    ctx.close()


def test_noalloc_frees_nothing_and_takes_nothing():
    """Free device memory is the same before and after a run of calls whose
    inputs already exist (the first call on the device may load the image)."""
    torch = pytest.importorskip("torch")
    ctx = Context(0)
    host = HostGraph.er(1000, 4000, 4, seed=1)
    dev = DeviceGraph(ctx, host)
    plan = Plan(Query.generate(host, 5, "sparse", seed=3))
    cm_dev, roots_dev, n = inputs(torch, ctx, dev, plan)
    want = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        assert noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n) == want
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == before
    ctx.close()


def test_noalloc_spends_its_slots():
    """The heaviest queries of the 2^20-vertex workload split work until the
    queue's slots are spent; the counts stay equal to the committed
    oracle-verified ones, on two calls in a row."""
    torch = pytest.importorskip("torch")
    wl = load("rmat20")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    ctx = Context(0)
    dev = DeviceGraph(ctx, host)
    heavy = sorted(range(len(qs)), key=lambda i: -counts[i])[:4]
    spent = 0
    for i in heavy:
        plan = Plan(qs[i])
        cm_dev, roots_dev, n = inputs(torch, ctx, dev, plan)
        first = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n)
        taken, split, full = queue_use()
        second = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n)
        assert first == second == counts[i], (i, first, second, counts[i])
        # a split that finds the slots spent still advances the tail, so a
        # spent queue reads at or past MAX_TASKS
        spent += int(full != 0 or taken >= MAX_TASKS)
    assert spent >= 1, "no query spent the queue's slots"
    ctx.close()


def test_noalloc_time_limit(monkeypatch):
    """A time limit that has run out comes back as SMG_ERR_TIMEOUT; the next
    call on the same context, with the limit lifted, is exact."""
    torch = pytest.importorskip("torch")
    wl = load("rmat20")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    ctx = Context(0)
    dev = DeviceGraph(ctx, host)
    i = max(range(len(qs)), key=lambda j: counts[j])
    plan = Plan(qs[i])
    cm_dev, roots_dev, n = inputs(torch, ctx, dev, plan)
    monkeypatch.setenv("SMG_TIME_LIMIT_S", "0.000001")
    st, _ = noalloc_status(ctx, dev, plan, cm_dev, roots_dev, n)
    assert st == 8  # SMG_ERR_TIMEOUT
    monkeypatch.delenv("SMG_TIME_LIMIT_S")
    assert noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n) == counts[i]
    ctx.close()


def test_noalloc_rejects_too_many_roots():
    torch = pytest.importorskip("torch")
    ctx = Context(0)
    host = HostGraph.er(100, 300, 2, seed=3)
    dev = DeviceGraph(ctx, host)
    plan = Plan(Query([0, 1], [0, 1]))
    cm = torch.zeros(100, dtype=torch.int32, device="cuda")
    out = C.c_uint64()
    st = lib.smg_join_noalloc(ctx.handle, dev.handle, plan.handle, C.c_void_p(cm.data_ptr()),
                              C.c_void_p(cm.data_ptr()), 101, C.byref(out))
    assert st == 5  # SMG_ERR_LIMIT
    ctx.close()
