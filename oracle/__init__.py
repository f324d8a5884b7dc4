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
vp = C.c_void_p


# The oracle's own views of include/smg.h's smg_csr and smg_query_desc (the
# same layouts), so that loading the oracle maps nothing of the library.  The
# functions take the address of any structure with these layouts: the
# library's Python objects (HostGraph.csr, Query.desc, Plan.view) and the
# oracle's own (Graph, QueryArrays) alike.
class Csr(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint64), ("offsets", u64p), ("neighbors", u32p),
                ("labels", u32p)]


class QueryDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint32), ("labels", u32p), ("edges", u32p)]


def _addr(struct):
    return C.c_void_p(C.addressof(struct))


def _load():
    if not _LIB.exists():
        raise ImportError(f"{_LIB} missing: run `python -m clustersm_gb300.build`")
    lib = C.CDLL(str(_LIB))
    lib.oracle_count.argtypes = [vp, vp, u32p, C.c_int, u64p]
    lib.oracle_embeddings.argtypes = [vp, vp, C.c_uint64, u32p, u64p, u64p]
    lib.oracle_count_roots.argtypes = [vp, vp, C.c_int, C.c_uint64, C.c_uint64, u64p, u64p]
    lib.oracle_nlc_filter.argtypes = [vp, vp, u32p]
    lib.oracle_encode.argtypes = [vp, vp, u32p, u32p, u32p]
    lib.oracle_count_budget.argtypes = [vp, vp, u32p, C.c_int, C.c_uint64, u64p, u64p]
    lib.oracle_ref_rows.argtypes = [vp, C.c_uint32, C.c_uint32, u32p, u32p, u32p, C.c_int, C.c_uint64, u64p]
    gen = [C.POINTER(u64p), C.POINTER(u32p), C.POINTER(u32p), u64p]
    lib.oracle_gen_rmat.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, *gen]
    lib.oracle_gen_er.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, *gen]
    lib.oracle_free.argtypes = [vp]
    lib.oracle_free.restype = None
    for f in ("oracle_ref_rows", "oracle_count_budget", "oracle_count", "oracle_embeddings", "oracle_count_roots",
              "oracle_nlc_filter", "oracle_encode", "oracle_gen_rmat", "oracle_gen_er"):
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
    rc = _lib.oracle_count(_addr(graph.csr), _addr(query.desc), cm, threads, C.byref(out))
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
    rc = _lib.oracle_count_budget(_addr(graph.csr), _addr(query.desc), cm, threads, budget, C.byref(out),
                                  C.byref(used))
    if rc:
        raise ValueError("oracle_count_budget rejected the input")
    return out.value, (None if used.value == (1 << 64) - 1 else used.value)


def count_roots(graph, query, lo, hi, threads: int = 0):
    """Count restricted to a slice of the oracle's root candidates: (count, total roots)."""
    out, nr = C.c_uint64(), C.c_uint64()
    rc = _lib.oracle_count_roots(_addr(graph.csr), _addr(query.desc), threads, lo, hi, C.byref(out),
                                 C.byref(nr))
    if rc:
        raise ValueError("oracle_count_roots rejected the input")
    return out.value, nr.value


def embeddings(graph, query, max_rows: int = 1 << 20):
    """(count, sorted embeddings array [rows, k]) for small cases."""
    k = query.k
    buf = np.zeros((max_rows, k), dtype=np.uint32)
    rows, cnt = C.c_uint64(), C.c_uint64()
    rc = _lib.oracle_embeddings(_addr(graph.csr), _addr(query.desc), max_rows, buf.ctypes.data_as(u32p),
                                C.byref(rows), C.byref(cnt))
    if rc:
        raise ValueError("oracle_embeddings rejected the input")
    return cnt.value, buf[: rows.value]


def nlc_filter(graph, plan):
    vm = np.zeros(graph.n, dtype=np.uint32)
    if _lib.oracle_nlc_filter(_addr(graph.csr), _addr(plan.view), vm.ctypes.data_as(u32p)):
        raise ValueError("oracle_nlc_filter failed")
    return vm


def encode(graph, plan, vmask0):
    vmask0 = np.ascontiguousarray(vmask0, dtype=np.uint32)
    enc = np.zeros(graph.n * plan.view.num_words, dtype=np.uint32)
    cm = np.zeros(graph.n, dtype=np.uint32)
    if _lib.oracle_encode(_addr(graph.csr), _addr(plan.view), vmask0.ctypes.data_as(u32p),
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
    rc = _lib.oracle_ref_rows(_addr(graph.csr), v.k, E, first.ctypes.data_as(u32p), second.ctypes.data_as(u32p),
                              candmask.ctypes.data_as(u32p), threads, limit, rows.ctypes.data_as(u64p))
    if rc:
        raise ValueError("oracle_ref_rows rejected the input")
    return [None if int(r) == (1 << 64) - 1 else int(r) for r in rows.tolist()]


class Graph:
    """A seeded workload graph generated by the oracle itself (CSR with
    sorted lists, labels): the same graph as the library's HostGraph.rmat /
    HostGraph.er for the same arguments."""

    def __init__(self, off, adj, labels):
        self.offsets_arr = np.ascontiguousarray(off, dtype=np.uint64)
        self.adj = np.ascontiguousarray(adj, dtype=np.uint32)
        self.labels_arr = np.ascontiguousarray(labels, dtype=np.uint32)
        self.n = len(self.labels_arr)
        self.m = len(self.adj) // 2
        self.csr = Csr(self.n, self.m, self.offsets_arr.ctypes.data_as(u64p), self.adj.ctypes.data_as(u32p),
                       self.labels_arr.ctypes.data_as(u32p))

    @classmethod
    def rmat(cls, scale, avg_degree, num_labels, seed, zipf=True):
        off, adj, lab, m2 = u64p(), u32p(), u32p(), C.c_uint64()
        if _lib.oracle_gen_rmat(scale, avg_degree, num_labels, 1 if zipf else 0, seed, C.byref(off), C.byref(adj),
                                C.byref(lab), C.byref(m2)):
            raise ValueError("oracle_gen_rmat rejected its arguments")
        return cls._own(1 << scale, off, adj, lab, m2.value)

    @classmethod
    def er(cls, n, m, num_labels, seed, zipf=False):
        off, adj, lab, m2 = u64p(), u32p(), u32p(), C.c_uint64()
        if _lib.oracle_gen_er(n, m, num_labels, 1 if zipf else 0, seed, C.byref(off), C.byref(adj), C.byref(lab),
                              C.byref(m2)):
            raise ValueError("oracle_gen_er rejected its arguments")
        return cls._own(n, off, adj, lab, m2.value)

    @classmethod
    def _own(cls, n, off, adj, lab, m2):
        try:
            g = cls(np.ctypeslib.as_array(off, shape=(n + 1,)).copy(),
                    np.ctypeslib.as_array(adj, shape=(max(m2, 1),))[:m2].copy(),
                    np.ctypeslib.as_array(lab, shape=(n,)).copy())
        finally:
            for ptr in (off, adj, lab):
                _lib.oracle_free(C.cast(ptr, C.c_void_p))
        return g

    def offsets(self):
        return self.offsets_arr

    def neighbors(self):
        return self.adj

    def labels(self):
        return self.labels_arr


class QueryArrays:
    """A query from its labels and file-order edge list, for the oracle."""

    def __init__(self, labels, edges):
        self.labels = np.ascontiguousarray(labels, dtype=np.uint32)
        self.edges = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1)
        self.k = len(self.labels)
        self.desc = QueryDesc(self.k, len(self.edges) // 2, self.labels.ctypes.data_as(u32p),
                              self.edges.ctypes.data_as(u32p))
