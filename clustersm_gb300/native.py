"""ctypes binding of libsmg (include/smg.h) with thin Python wrappers.

The library is loaded from clustersm_gb300/lib/libsmg.so, built in-tree by
clustersm_gb300.build.  There is no fallback: if the shared library is missing
the import fails with an error naming the build command.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_LIB_PATH = Path(os.environ.get("SMG_LIB_PATH", Path(__file__).resolve().parent / "lib" / "libsmg.so"))

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)

SMG_OK = 0
STATUS = {0: "SMG_OK", 1: "SMG_ERR_INVALID", 2: "SMG_ERR_IO", 3: "SMG_ERR_FORMAT", 4: "SMG_ERR_QUERY",
          5: "SMG_ERR_LIMIT", 6: "SMG_ERR_CUDA", 7: "SMG_ERR_OOM", 8: "SMG_ERR_TIMEOUT",
          9: "SMG_ERR_NO_DEVICE", 10: "SMG_ERR_BUDGET", 11: "SMG_ERR_CANCELLED", 12: "SMG_ERR_NOT_READY",
          13: "SMG_ERR_INTERNAL"}
SHAPES = {"tree": 0, "sparse": 1, "dense": 2, "induced": 3}
LABELS_UNIFORM, LABELS_ZIPF1 = 0, 1
FLAG_EMIT, FLAG_PROFILE, FLAG_NO_GRAPH, FLAG_MODEL = 1, 2, 4, 8


class SmgError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)} ({detail})")


class Csr(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint64), ("offsets", u64p),
                ("neighbors", u32p), ("labels", u32p)]


class QueryDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint32), ("labels", u32p), ("edges", u32p)]


_PLAN_FIELDS = [
    ("k", C.c_uint32), ("num_edges", C.c_uint32), ("nvlq", C.c_uint32), ("root", C.c_uint32),
    ("labels", u32p), ("degrees", u32p), ("nlc", u32p), ("tree_offsets", u32p), ("tree_neighbors", u32p),
    ("cover_size", C.c_uint32), ("cover", u32p), ("num_clusters", C.c_uint32), ("num_slots", C.c_uint32),
    ("num_words", C.c_uint32), ("cluster_offsets", u32p), ("slots", u32p), ("cluster_layer", u32p),
    ("cluster_kind", u32p), ("num_layers", C.c_uint32), ("num_merges", C.c_uint32), ("merge_cluster", u32p),
    ("merge_left", u32p), ("merge_right", u32p), ("merge_vertex", u32p), ("num_combines", C.c_uint32),
    ("combine_out", u32p), ("combine_type", u32p), ("combine_layer", u32p), ("combine_other_offsets", u32p),
    ("combine_others", u32p), ("last_slot", u32p), ("edge_order_first", u32p), ("edge_order_second", u32p),
    ("order", u32p), ("anchor_level", u32p), ("back_mask", u32p),
]


class PlanView(C.Structure):
    _fields_ = _PLAN_FIELDS


class MatchOpts(C.Structure):
    _fields_ = [("flags", C.c_uint32), ("bfs_depth", C.c_uint32), ("root_chunk", C.c_uint32),
                ("reserved", C.c_uint32), ("max_embeddings", C.c_uint64), ("embeddings", u32p),
                ("max_count", C.c_uint64), ("max_work", C.c_uint64)]


class MatchResult(C.Structure):
    _fields_ = [("count", C.c_uint64), ("embeddings_written", C.c_uint64), ("overflow", C.c_uint32),
                ("num_candidates_root", C.c_uint32), ("candidates_total", C.c_uint64),
                ("filter_ms", C.c_float), ("join_ms", C.c_float), ("tasks", C.c_uint64),
                ("filter_bytes", C.c_uint64), ("join_bytes", C.c_uint64), ("limit_hit", C.c_uint32),
                ("reserved", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("filter_ms", C.c_float), ("join_ms", C.c_float), ("tasks", C.c_uint64),
                ("total_embeddings", C.c_uint64), ("kernel_launches", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("filter_bytes", C.c_uint64), ("join_bytes", C.c_uint64),
                ("chunks", C.c_uint32), ("reserved", C.c_uint32), ("scanned", C.c_uint64),
                ("descents", C.c_uint64), ("probes", C.c_uint64), ("last_count_entries", C.c_uint64),
                ("donations", C.c_uint64), ("model_bytes", C.c_uint64), ("bfs_tasks", C.c_uint64)]


class TuneEntry(C.Structure):
    _fields_ = [("shape_class", C.c_uint32), ("root_chunk", C.c_uint32), ("donate_min", C.c_uint32),
                ("samples", C.c_uint32), ("best_ms", C.c_float), ("default_ms", C.c_float),
                ("split_len", C.c_uint32), ("hoist_cap", C.c_uint32), ("bfs_depth", C.c_uint32),
                ("reserved", C.c_uint32)]


class GraphStats(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint64), ("num_labels", C.c_uint32),
                ("max_degree", C.c_uint32), ("device_bytes", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_uint64), ("max_inflight", C.c_uint32),
                ("max_query_vertices", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("slices", C.c_uint64), ("bells", C.c_uint64), ("admitted", C.c_uint64),
                ("retired_in_slice", C.c_uint64), ("carried_tasks", C.c_uint64), ("slice_s", C.c_double),
                ("between_s", C.c_double), ("admitted_live", C.c_uint64)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("reserved", C.c_uint32), ("count", C.c_uint64),
                ("submit_s", C.c_double), ("start_s", C.c_double), ("finish_s", C.c_double)]


def _load():
    if not _LIB_PATH.exists():
        raise ImportError(f"{_LIB_PATH} is missing: build it with `python -m clustersm_gb300.build` "
                          "(or __graft_entry__.build())")
    lib = C.CDLL(str(_LIB_PATH))
    vp = C.c_void_p
    st = C.c_int32
    sig = {
        "smg_strerror": (C.c_char_p, [st]),
        "smg_last_error": (C.c_char_p, []),
        "smg_read_graph": (st, [C.c_char_p, C.POINTER(vp)]),
        "smg_read_query": (st, [C.c_char_p, C.POINTER(vp)]),
        "smg_write_graph": (st, [C.c_char_p, C.POINTER(Csr)]),
        "smg_write_query": (st, [C.c_char_p, C.POINTER(QueryDesc)]),
        "smg_host_graph_view": (st, [vp, C.POINTER(Csr)]),
        "smg_host_query_view": (st, [vp, C.POINTER(QueryDesc)]),
        "smg_host_graph_from_csr": (st, [C.POINTER(Csr), C.POINTER(vp)]),
        "smg_host_graph_free": (None, [vp]),
        "smg_host_query_free": (None, [vp]),
        "smg_gen_er": (st, [C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(vp)]),
        "smg_gen_rmat": (st, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_int,
                              C.POINTER(vp)]),
        "smg_gen_query": (st, [C.POINTER(Csr), C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(vp), u32p]),
        "smg_gen_rmat_pairs": (st, [C.c_uint32, C.c_uint32, C.c_uint64, C.c_int, u32p, u64p]),
        "smg_gen_labels": (st, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, u32p]),
        "smg_plan_create": (st, [C.POINTER(QueryDesc), C.POINTER(vp)]),
        "smg_plan_create_batch": (st, [C.POINTER(QueryDesc), C.c_uint32, C.POINTER(vp)]),
        "smg_plan_free": (None, [vp]),
        "smg_plan_get": (st, [vp, C.POINTER(PlanView)]),
    }
    dev = {
        "smg_open": (st, [C.c_int, C.POINTER(vp)]),
        "smg_close": (None, [vp]),
        "smg_ctx_stream": (vp, [vp]),
        "smg_graph_upload": (st, [vp, C.POINTER(Csr), C.POINTER(vp)]),
        "smg_graph_build": (st, [vp, C.c_uint32, C.c_uint64, u32p, u32p, C.POINTER(vp), u64p]),
        "smg_graph_download": (st, [vp, vp, u64p, u32p]),
        "smg_graph_free": (None, [vp]),
        "smg_graph_get_stats": (st, [vp, C.POINTER(GraphStats)]),
        "smg_match": (st, [vp, vp, vp, C.POINTER(MatchOpts), C.POINTER(MatchResult)]),
        "smg_match_batch": (st, [vp, vp, C.POINTER(vp), C.c_uint32, C.POINTER(MatchOpts), u64p,
                                 C.POINTER(BatchStats)]),
        "smg_filter_inspect": (st, [vp, vp, vp, u32p, u32p, u32p]),
        "smg_autotune": (st, [vp, vp, C.POINTER(vp), C.c_uint32, C.POINTER(TuneEntry)]),
        "smg_join_noalloc": (st, [vp, vp, vp, C.c_void_p, C.c_void_p, C.c_uint32, u64p]),
        "smg_set_tuning": (st, [vp, C.POINTER(TuneEntry), C.c_uint32]),
        "smg_plan_class": (C.c_uint32, [vp]),
        "smg_server_create": (st, [vp, vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
        "smg_server_submit": (st, [vp, vp, u64p]),
        "smg_server_poll": (st, [vp, C.c_uint64, C.POINTER(RequestResult)]),
        "smg_server_cancel": (st, [vp, C.c_uint64]),
        "smg_server_drain": (st, [vp]),
        "smg_server_step": (st, [vp]),
        "smg_server_destroy": (None, [vp]),
        "smg_server_get_stats": (st, [vp, C.POINTER(ServerStats)]),
    }
    sig.update(dev)
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)  # a missing export raises here: no silent fallback
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(status: int, where: str):
    if status != SMG_OK:
        raise SmgError(status, where, lib.smg_last_error().decode())


def _arr(ptr, n, dtype=np.uint32):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


class HostGraph:
    """A data graph in host memory (CSR, sorted neighbour lists unless read from a file)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        self._csr = Csr()
        check(lib.smg_host_graph_view(self._h, C.byref(self._csr)), "smg_host_graph_view")

    @classmethod
    def read(cls, path):
        h = C.c_void_p()
        check(lib.smg_read_graph(str(path).encode(), C.byref(h)), f"smg_read_graph({path})")
        return cls(h)

    @classmethod
    def from_arrays(cls, offsets, neighbors, labels):
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        neighbors, labels = _u32(neighbors), _u32(labels)
        c = Csr(len(labels), len(neighbors) // 2, offsets.ctypes.data_as(u64p), neighbors.ctypes.data_as(u32p),
                labels.ctypes.data_as(u32p))
        h = C.c_void_p()
        check(lib.smg_host_graph_from_csr(C.byref(c), C.byref(h)), "smg_host_graph_from_csr")
        return cls(h)

    @classmethod
    def er(cls, n, m, num_labels, seed, zipf=False):
        h = C.c_void_p()
        check(lib.smg_gen_er(n, m, num_labels, LABELS_ZIPF1 if zipf else LABELS_UNIFORM, seed, C.byref(h)),
              "smg_gen_er")
        return cls(h)

    @classmethod
    def rmat(cls, scale, avg_degree, num_labels, seed, zipf=True, threads=0):
        h = C.c_void_p()
        check(lib.smg_gen_rmat(scale, avg_degree, num_labels, LABELS_ZIPF1 if zipf else LABELS_UNIFORM, seed,
                               threads, C.byref(h)), "smg_gen_rmat")
        return cls(h)

    @staticmethod
    def rmat_pairs(scale, avg_degree, seed, threads=0):
        """The raw R-MAT edge draws of rmat() for the same seed: uint32 [m, 2]."""
        m = C.c_uint64()
        check(lib.smg_gen_rmat_pairs(scale, avg_degree, seed, threads, None, C.byref(m)), "smg_gen_rmat_pairs")
        out = np.zeros((m.value, 2), dtype=np.uint32)
        check(lib.smg_gen_rmat_pairs(scale, avg_degree, seed, threads, out.ctypes.data_as(u32p), C.byref(m)),
              "smg_gen_rmat_pairs")
        return out

    @staticmethod
    def labels_for(n, num_labels, seed, zipf=True):
        """The labels er()/rmat() draw for the same seed."""
        out = np.zeros(n, dtype=np.uint32)
        check(lib.smg_gen_labels(n, num_labels, 1 if zipf else 0, seed, out.ctypes.data_as(u32p)), "smg_gen_labels")
        return out

    @property
    def csr(self) -> Csr:
        return self._csr

    @property
    def n(self):
        return self._csr.num_vertices

    @property
    def m(self):
        return self._csr.num_edges

    def offsets(self):
        return np.ctypeslib.as_array(self._csr.offsets, shape=(self.n + 1,))

    def neighbors(self):
        return np.ctypeslib.as_array(self._csr.neighbors, shape=(2 * self.m,)) if self.m else np.zeros(0, np.uint32)

    def labels(self):
        return np.ctypeslib.as_array(self._csr.labels, shape=(self.n,))

    def write(self, path):
        check(lib.smg_write_graph(str(path).encode(), C.byref(self._csr)), "smg_write_graph")

    def sorted_copy(self):
        """Host graph with sorted neighbour lists (what the device and the oracle expect)."""
        return HostGraph.from_arrays(self.offsets(), self.neighbors(), self.labels())

    def __del__(self):
        if getattr(self, "_h", None):
            lib.smg_host_graph_free(self._h)
            self._h = None


class Query:
    """A query graph: labels + edge list in file order."""

    def __init__(self, labels, edges, data_vertices=None):
        self.labels = _u32(labels)
        self.edges = _u32(np.asarray(edges).reshape(-1))
        self.data_vertices = data_vertices
        self._desc = QueryDesc(len(self.labels), len(self.edges) // 2, self.labels.ctypes.data_as(u32p),
                               self.edges.ctypes.data_as(u32p))

    @property
    def desc(self) -> QueryDesc:
        return self._desc

    @property
    def k(self):
        return len(self.labels)

    @classmethod
    def _from_handle(cls, h, data_vertices=None):
        d = QueryDesc()
        check(lib.smg_host_query_view(h, C.byref(d)), "smg_host_query_view")
        q = cls(_arr(d.labels, d.num_vertices), _arr(d.edges, 2 * d.num_edges), data_vertices)
        lib.smg_host_query_free(h)
        return q

    @classmethod
    def read(cls, path):
        h = C.c_void_p()
        check(lib.smg_read_query(str(path).encode(), C.byref(h)), f"smg_read_query({path})")
        return cls._from_handle(h)

    @classmethod
    def generate(cls, graph: HostGraph, k: int, shape: str, seed: int):
        h = C.c_void_p()
        dv = np.zeros(k, dtype=np.uint32)
        check(lib.smg_gen_query(C.byref(graph.csr), k, SHAPES[shape], seed, C.byref(h), dv.ctypes.data_as(u32p)),
              "smg_gen_query")
        return cls._from_handle(h, dv)

    def write(self, path):
        check(lib.smg_write_query(str(path).encode(), C.byref(self._desc)), "smg_write_query")

    def to_dict(self):
        return {"labels": self.labels.tolist(), "edges": self.edges.tolist()}


class Plan:
    """Host-side plan of one query (spanning tree, clusters, matching order)."""

    def __init__(self, query: Query, handle=None):
        self.query = query
        if handle is None:
            self._h = C.c_void_p()
            check(lib.smg_plan_create(C.byref(query.desc), C.byref(self._h)), "smg_plan_create")
        else:
            self._h = handle
        self._view = None

    @property
    def view(self) -> PlanView:
        """The plan's read-only view (smg_plan_get), fetched on first use."""
        if self._view is None:
            v = PlanView()
            check(lib.smg_plan_get(self._h, C.byref(v)), "smg_plan_get")
            self._view = v
        return self._view

    @classmethod
    def batch(cls, queries) -> list:
        """Plans of many queries, made on all host threads (smg_plan_create_batch)."""
        n = len(queries)
        descs = (QueryDesc * n)(*[q.desc for q in queries])
        hs = (C.c_void_p * n)()
        check(lib.smg_plan_create_batch(descs, n, hs), "smg_plan_create_batch")
        return [cls(q, C.c_void_p(h)) for q, h in zip(queries, hs)]

    @property
    def handle(self):
        return self._h

    def to_dict(self) -> dict:
        v = self.view
        k, C_, S = v.k, v.num_clusters, v.num_slots
        nm, nc = v.num_merges, v.num_combines
        oth_off = _arr(v.combine_other_offsets, nc + 1)
        return {
            "k": k, "num_edges": v.num_edges, "nvlq": v.nvlq, "root": v.root,
            "labels": _arr(v.labels, k).tolist(), "degrees": _arr(v.degrees, k).tolist(),
            "nlc": _arr(v.nlc, k * v.nvlq).tolist(),
            "tree_offsets": _arr(v.tree_offsets, k + 1).tolist(),
            "tree_neighbors": _arr(v.tree_neighbors, int(_arr(v.tree_offsets, k + 1)[-1])).tolist(),
            "cover": _arr(v.cover, v.cover_size).tolist(),
            "num_clusters": C_, "num_slots": S, "num_words": v.num_words, "num_layers": v.num_layers,
            "cluster_offsets": _arr(v.cluster_offsets, C_ + 1).tolist(), "slots": _arr(v.slots, S).tolist(),
            "cluster_layer": _arr(v.cluster_layer, C_).tolist(), "cluster_kind": _arr(v.cluster_kind, C_).tolist(),
            "merge_cluster": _arr(v.merge_cluster, nm).tolist(), "merge_left": _arr(v.merge_left, nm).tolist(),
            "merge_right": _arr(v.merge_right, nm).tolist(), "merge_vertex": _arr(v.merge_vertex, nm).tolist(),
            "combine_out": _arr(v.combine_out, nc).tolist(), "combine_type": _arr(v.combine_type, nc).tolist(),
            "combine_layer": _arr(v.combine_layer, nc).tolist(),
            "combine_others": [_arr(v.combine_others, int(oth_off[-1]))[oth_off[i]:oth_off[i + 1]].tolist()
                               for i in range(nc)],
            "last_slot": _arr(v.last_slot, k).tolist(),
            "edge_order": list(zip(_arr(v.edge_order_first, v.num_edges).tolist(),
                                   _arr(v.edge_order_second, v.num_edges).tolist())),
            "order": _arr(v.order, k).tolist(), "anchor_level": _arr(v.anchor_level, k).tolist(),
            "back_mask": _arr(v.back_mask, k).tolist(),
        }

    def __del__(self):
        if getattr(self, "_h", None):
            lib.smg_plan_free(self._h)
            self._h = None


class Context:
    """A device context (one CUDA device, one stream)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        self.device = device
        check(lib.smg_open(device, C.byref(self._h)), "smg_open")

    @property
    def handle(self):
        return self._h

    @property
    def stream_ptr(self) -> int:
        """The library's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        return lib.smg_ctx_stream(self._h) or 0

    def close(self):
        if getattr(self, "_h", None):
            lib.smg_close(self._h)
            self._h = None

    def __del__(self):
        self.close()


class DeviceGraph:
    """A data graph resident in device memory."""

    def __init__(self, ctx: Context, host: HostGraph | None):
        self.ctx = ctx
        self.host = host
        self._h = C.c_void_p()
        if host is not None:
            self.n = host.n
            check(lib.smg_graph_upload(ctx.handle, C.byref(host.csr), C.byref(self._h)), "smg_graph_upload")

    @classmethod
    def build(cls, ctx: Context, num_vertices: int, pairs, labels):
        """smg_graph_build: the CSR is sorted and de-duplicated on the device
        from an undirected edge list (pairs: [m, 2] or flat uint32)."""
        g = cls(ctx, None)
        g.n = int(num_vertices)
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1)
        labels = np.ascontiguousarray(labels, dtype=np.uint32)
        ne = C.c_uint64()
        check(lib.smg_graph_build(ctx.handle, g.n, pairs.size // 2, pairs.ctypes.data_as(u32p),
                                  labels.ctypes.data_as(u32p), C.byref(g._h), C.byref(ne)), "smg_graph_build")
        g.num_edges = ne.value
        return g

    def download(self):
        """(offsets uint64 [n+1], neighbors uint32 [2m]) of the resident CSR."""
        st = self.stats()
        off = np.zeros(st.num_vertices + 1, dtype=np.uint64)
        nb = np.zeros(max(1, 2 * st.num_edges), dtype=np.uint32)
        check(lib.smg_graph_download(self.ctx.handle, self._h, off.ctypes.data_as(u64p), nb.ctypes.data_as(u32p)),
              "smg_graph_download")
        return off, nb[: 2 * st.num_edges]

    @property
    def handle(self):
        return self._h

    def stats(self) -> GraphStats:
        s = GraphStats()
        check(lib.smg_graph_get_stats(self._h, C.byref(s)), "smg_graph_get_stats")
        return s

    def free(self):
        if getattr(self, "_h", None):
            lib.smg_graph_free(self._h)
            self._h = None

    def __del__(self):
        self.free()


def match(ctx: Context, graph: DeviceGraph, plan: Plan, emit: int = 0, profile=False,
          root_chunk=0, max_count=0, max_work=0, bfs_depth=0):
    """Plain path.  Returns (MatchResult, embeddings array or None)."""
    opts = MatchOpts()
    opts.bfs_depth = bfs_depth
    opts.max_count = max_count
    opts.max_work = max_work
    opts.flags = (FLAG_EMIT if emit else 0) | (FLAG_PROFILE if profile else 0)
    opts.root_chunk = root_chunk
    buf = None
    if emit:
        buf = np.zeros((emit, plan.view.k), dtype=np.uint32)
        opts.max_embeddings = emit
        opts.embeddings = buf.ctypes.data_as(u32p)
    res = MatchResult()
    check(lib.smg_match(ctx.handle, graph.handle, plan.handle, C.byref(opts), C.byref(res)), "smg_match")
    if emit:
        buf = buf[: res.embeddings_written]
    return res, buf


def match_batch(ctx: Context, graph: DeviceGraph, plans, root_chunk=0, profile=False, max_count=0,
                use_graph=True, max_work=0, model=False, bfs_depth=0):
    """Batched path.  Returns (counts, BatchStats); with max_count or
    max_work, queries over a limit report 2**64-1."""
    n = len(plans)
    arr = (C.c_void_p * n)(*[p.handle.value for p in plans])
    counts = np.zeros(n, dtype=np.uint64)
    opts = MatchOpts()
    opts.flags = (FLAG_PROFILE if profile else 0) | (0 if use_graph else FLAG_NO_GRAPH) | (FLAG_MODEL if model else 0)
    opts.root_chunk = root_chunk
    opts.bfs_depth = bfs_depth
    opts.max_count = max_count
    opts.max_work = max_work
    st = BatchStats()
    check(lib.smg_match_batch(ctx.handle, graph.handle, arr, n, C.byref(opts), counts.ctypes.data_as(u64p),
                              C.byref(st)), "smg_match_batch")
    return counts, st


def autotune(ctx: Context, graph: DeviceGraph, plans):
    """Tune the join per shape class on sample plans; returns the 12 entries."""
    arr = (C.c_void_p * len(plans))(*[p.handle.value for p in plans])
    out = (TuneEntry * 12)()
    check(lib.smg_autotune(ctx.handle, graph.handle, arr, len(plans), out), "smg_autotune")
    return list(out)


def filter_inspect(ctx: Context, graph: DeviceGraph, plan: Plan):
    n = graph.n
    vm = np.zeros(n, np.uint32)
    enc = np.zeros(n * plan.view.num_words, np.uint32)
    cm = np.zeros(n, np.uint32)
    check(lib.smg_filter_inspect(ctx.handle, graph.handle, plan.handle, vm.ctypes.data_as(u32p),
                                 enc.ctypes.data_as(u32p), cm.ctypes.data_as(u32p)), "smg_filter_inspect")
    return vm, enc, cm


class Server:
    """Continuous-batching request loop (smg_server_*).  Plans must outlive
    their requests; this wrapper keeps a reference until the result is read."""

    def __init__(self, ctx: Context, graph: DeviceGraph, memory_budget_bytes: int = 0, max_inflight: int = 0,
                 max_query_vertices: int = 0):
        self.ctx, self.graph = ctx, graph
        cfg = ServerConfig(memory_budget_bytes, max_inflight, max_query_vertices)
        self._h = C.c_void_p()
        check(lib.smg_server_create(ctx.handle, graph.handle, C.byref(cfg), C.byref(self._h)), "smg_server_create")
        self._plans = {}

    def submit(self, plan: Plan) -> int:
        t = C.c_uint64()
        check(lib.smg_server_submit(self._h, plan.handle, C.byref(t)), "smg_server_submit")
        self._plans[t.value] = plan
        return t.value

    def step(self):
        check(lib.smg_server_step(self._h), "smg_server_step")

    def stats(self) -> ServerStats:
        out = ServerStats()
        check(lib.smg_server_get_stats(self._h, C.byref(out)), "smg_server_get_stats")
        return out

    def poll(self, ticket: int):
        """RequestResult, or None while the request is queued or running."""
        r = RequestResult()
        st = lib.smg_server_poll(self._h, ticket, C.byref(r))
        if st == 12:
            return None
        check(st, "smg_server_poll")
        self._plans.pop(ticket, None)
        return r

    def cancel(self, ticket: int):
        check(lib.smg_server_cancel(self._h, ticket), "smg_server_cancel")

    def drain(self):
        check(lib.smg_server_drain(self._h), "smg_server_drain")

    def close(self):
        if getattr(self, "_h", None):
            lib.smg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
