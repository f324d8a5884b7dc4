"""Python binding of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the checker or the timed CPU
baseline, never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB = Path(os.environ.get("SMG_ORACLE_PATH", _HERE / "lib" / "liboracle.so"))

u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)


def _load():
    if not _LIB.exists():
        raise ImportError(f"{_LIB} missing: run `python -m clustersm_gb300.build`")
    from clustersm_gb300.native import Csr, PlanView, QueryDesc
    lib = C.CDLL(str(_LIB))
    lib.oracle_count.argtypes = [C.POINTER(Csr), C.POINTER(QueryDesc), u32p, C.c_int, u64p]
    lib.oracle_embeddings.argtypes = [C.POINTER(Csr), C.POINTER(QueryDesc), C.c_uint64, u32p, u64p, u64p]
    lib.oracle_count_roots.argtypes = [C.POINTER(Csr), C.POINTER(QueryDesc), C.c_int, C.c_uint64, C.c_uint64,
                                       u64p, u64p]
    lib.oracle_nlc_filter.argtypes = [C.POINTER(Csr), C.POINTER(PlanView), u32p]
    lib.oracle_encode.argtypes = [C.POINTER(Csr), C.POINTER(PlanView), u32p, u32p, u32p]
    lib.oracle_count_budget.argtypes = [C.POINTER(Csr), C.POINTER(QueryDesc), u32p, C.c_int, C.c_uint64, u64p,
                                        u64p]
    lib.oracle_ref_rows.argtypes = [C.POINTER(Csr), C.c_uint32, C.c_uint32, u32p, u32p, u32p, C.c_int, C.c_uint64,
                                    u64p]
    for f in ("oracle_ref_rows", "oracle_count_budget", "oracle_count", "oracle_embeddings", "oracle_count_roots", "oracle_nlc_filter", "oracle_encode"):
        getattr(lib, f).restype = C.c_int
    return lib


_lib = _load()


def count(graph, query, candmask=None, threads: int = 0) -> int:
    """Exact embedding count by backtracking (graph must have sorted lists)."""
    out = C.c_uint64()
    cm = None
    if candmask is not None:
        candmask = np.ascontiguousarray(candmask, dtype=np.uint32)
        cm = candmask.ctypes.data_as(u32p)
    rc = _lib.oracle_count(C.byref(graph.csr), C.byref(query.desc), cm, threads, C.byref(out))
    if rc:
        raise ValueError("oracle_count rejected the input")
    return out.value


def count_budget(graph, query, budget: int, candmask=None, threads: int = 0):
    """(count, partial matches used) or (lower bound, None) when the budget ran out."""
    out, used = C.c_uint64(), C.c_uint64()
    cm = None
    if candmask is not None:
        candmask = np.ascontiguousarray(candmask, dtype=np.uint32)
        cm = candmask.ctypes.data_as(u32p)
    rc = _lib.oracle_count_budget(C.byref(graph.csr), C.byref(query.desc), cm, threads, budget, C.byref(out),
                                  C.byref(used))
    if rc:
        raise ValueError("oracle_count_budget rejected the input")
    return out.value, (None if used.value == (1 << 64) - 1 else used.value)


def count_roots(graph, query, lo, hi, threads: int = 0):
    """Count restricted to a slice of the oracle's root candidates: (count, total roots)."""
    out, nr = C.c_uint64(), C.c_uint64()
    rc = _lib.oracle_count_roots(C.byref(graph.csr), C.byref(query.desc), threads, lo, hi, C.byref(out),
                                 C.byref(nr))
    if rc:
        raise ValueError("oracle_count_roots rejected the input")
    return out.value, nr.value


def embeddings(graph, query, max_rows: int = 1 << 20):
    """(count, sorted embeddings array [rows, k]) for small cases."""
    k = query.k
    buf = np.zeros((max_rows, k), dtype=np.uint32)
    rows, cnt = C.c_uint64(), C.c_uint64()
    rc = _lib.oracle_embeddings(C.byref(graph.csr), C.byref(query.desc), max_rows, buf.ctypes.data_as(u32p),
                                C.byref(rows), C.byref(cnt))
    if rc:
        raise ValueError("oracle_embeddings rejected the input")
    return cnt.value, buf[: rows.value]


def nlc_filter(graph, plan):
    vm = np.zeros(graph.n, dtype=np.uint32)
    if _lib.oracle_nlc_filter(C.byref(graph.csr), C.byref(plan.view), vm.ctypes.data_as(u32p)):
        raise ValueError("oracle_nlc_filter failed")
    return vm


def encode(graph, plan, vmask0):
    vmask0 = np.ascontiguousarray(vmask0, dtype=np.uint32)
    enc = np.zeros(graph.n * plan.view.num_words, dtype=np.uint32)
    cm = np.zeros(graph.n, dtype=np.uint32)
    if _lib.oracle_encode(C.byref(graph.csr), C.byref(plan.view), vmask0.ctypes.data_as(u32p),
                          enc.ctypes.data_as(u32p), cm.ctypes.data_as(u32p)):
        raise ValueError("oracle_encode failed")
    return enc, cm


def ref_rows(graph, plan, candmask, limit: int = (1 << 64) - 2, threads: int = 0):
    """Rows of the reference's breadth-first join tables after each step of
    its edge order (the plan's edge_order_first/second): a list of
    num_edges + 1 ints, None from the first level holding more than `limit`."""
    v = plan.view
    E = v.num_edges
    first = np.ctypeslib.as_array(v.edge_order_first, shape=(E,)).astype(np.uint32)
    second = np.ctypeslib.as_array(v.edge_order_second, shape=(E,)).astype(np.uint32)
    candmask = np.ascontiguousarray(candmask, dtype=np.uint32)
    rows = np.zeros(E + 1, dtype=np.uint64)
    rc = _lib.oracle_ref_rows(C.byref(graph.csr), v.k, E, first.ctypes.data_as(u32p), second.ctypes.data_as(u32p),
                              candmask.ctypes.data_as(u32p), threads, limit, rows.ctypes.data_as(u64p))
    if rc:
        raise ValueError("oracle_ref_rows rejected the input")
    return [None if int(r) == (1 << 64) - 1 else int(r) for r in rows.tolist()]
