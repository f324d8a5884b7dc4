"""Every C-ABI entry point answers bad arguments with a status instead of
exit() or a crash (the reference exits on bad input: io.cu:32,41,
cuda_helpers.h:27-32).  These calls return before any CUDA call, so they run
without a GPU."""
import ctypes as C

import numpy as np
import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import Query, QueryDesc, SmgError

lib = native.lib
INVALID, QUERY = 1, 4
vp = C.c_void_p


def test_null_arguments_give_invalid():
    out = vp()
    assert lib.smg_read_graph(None, C.byref(out)) == INVALID
    assert lib.smg_read_graph(b"x.in", None) == INVALID
    assert lib.smg_read_query(b"x.in", None) == INVALID
    assert lib.smg_plan_create(None, C.byref(out)) == INVALID
    assert lib.smg_plan_create_batch(None, 1, None) == INVALID
    assert lib.smg_plan_create_batch(None, 0, None) == 0  # nothing to plan
    assert lib.smg_plan_get(None, None) == INVALID
    assert lib.smg_graph_upload(None, None, C.byref(out)) == INVALID
    assert lib.smg_match(None, None, None, None, None) == INVALID
    assert lib.smg_match_batch(None, None, None, 0, None, None, None) == INVALID
    assert lib.smg_filter_inspect(None, None, None, None, None, None) == INVALID
    assert lib.smg_join_noalloc(None, None, None, None, None, 0, None) == INVALID
    assert lib.smg_autotune(None, None, None, 0, None) == INVALID
    assert lib.smg_set_tuning(None, None, 0) == INVALID
    assert lib.smg_graph_get_stats(None, None) == INVALID
    assert lib.smg_server_create(None, None, None, C.byref(out)) == INVALID
    assert lib.smg_server_submit(None, None, None) == INVALID
    assert lib.smg_server_step(None) == INVALID
    assert lib.smg_server_poll(None, 0, None) == INVALID
    assert lib.smg_server_drain(None) == INVALID
    assert lib.smg_server_cancel(None, 0) == INVALID
    assert lib.smg_server_get_stats(None, None) == INVALID
    assert lib.smg_host_graph_view(None, None) == INVALID
    assert lib.smg_host_query_view(None, None) == INVALID
    assert lib.smg_host_graph_from_csr(None, C.byref(out)) == INVALID
    assert lib.smg_write_graph(None, None) == INVALID
    assert lib.smg_write_query(None, None) == INVALID
    assert lib.smg_plan_class(None) == 0
    assert lib.smg_ctx_stream(None) is None
    # the error detail is recorded for the calling thread
    assert lib.smg_last_error()


def test_null_frees_are_no_ops():
    lib.smg_close(None)
    lib.smg_graph_free(None)
    lib.smg_plan_free(None)
    lib.smg_server_destroy(None)
    lib.smg_host_graph_free(None)
    lib.smg_host_query_free(None)


@pytest.mark.parametrize("labels,edges,status", [
    ([0], [], QUERY),                                   # fewer than 2 vertices
    ([0] * 33, [(i, i + 1) for i in range(32)], QUERY),  # more than 32
    ([0, 0], [], QUERY),                                # no edge
    ([0, 0], [(0, 2)], QUERY),                          # endpoint out of range
    ([0, 0], [(0, 0)], QUERY),                          # self-loop
    ([0, 0], [(0, 1), (1, 0)], QUERY),                  # repeated edge
    ([0, 0, 0, 0], [(0, 1), (2, 3)], QUERY),            # disconnected
])
def test_bad_queries(labels, edges, status):
    q = Query(labels, np.asarray(edges, dtype=np.uint32).reshape(-1, 2) if edges else np.zeros(0, np.uint32))
    with pytest.raises(SmgError) as e:
        native.Plan(q)
    assert e.value.status == status


def test_null_query_arrays():
    d = QueryDesc(3, 2, None, None)
    out = vp()
    assert lib.smg_plan_create(C.byref(d), C.byref(out)) == INVALID
