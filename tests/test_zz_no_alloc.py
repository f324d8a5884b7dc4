"""smg_join_noalloc: the allocation-free join for callers that cannot call
cudaMalloc while matching.  Its counts must equal smg_match's (exact: the
counts are integers) on two calls in a row, with the inputs in device memory
the caller owns (torch tensors here).  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import Context, DeviceGraph, HostGraph, Plan, Query, check, lib

pytestmark = pytest.mark.gpu


def noalloc_count(ctx, dev, plan, cm_dev, roots_dev, n_roots):
    out = C.c_uint64()
    check(lib.smg_join_noalloc(ctx.handle, dev.handle, plan.handle, C.c_void_p(cm_dev.data_ptr()),
                               C.c_void_p(roots_dev.data_ptr()), n_roots, C.byref(out)), "smg_join_noalloc")
    return out.value


@pytest.mark.parametrize("graph", ["er", "rmat"])
def test_noalloc_matches_plain(graph):
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
            plan = Plan(q)
            want, _ = native.match(ctx, dev, plan, max_count=10**9)
            if want.limit_hit:
                continue
            _, _, cm = native.filter_inspect(ctx, dev, plan)
            roots = np.nonzero((cm >> plan.view.root) & 1)[0].astype(np.int32)
            cm_dev = torch.from_numpy(cm.view(np.int32)).cuda()
            roots_dev = torch.from_numpy(roots if len(roots) else np.zeros(1, np.int32)).cuda()
            torch.cuda.synchronize()
            first = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, len(roots))
            second = noalloc_count(ctx, dev, plan, cm_dev, roots_dev, len(roots))
            assert first == second == want.count, (graph, shape, s)
            checked += 1
    assert checked >= 4
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
