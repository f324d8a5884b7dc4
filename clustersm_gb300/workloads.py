"""Seeded synthetic workloads (the reference's github / gowalla / dblp query
sets are not available; runClusterSM.sh:9-27).

A workload is a data graph plus a list of queries, both generated from fixed
seeds by the library's integer-only generators, so every host builds the same
inputs.  `queries_file` workloads read their queries (labels + edges in file
order, plus the expected counts) from a committed JSON fixture instead of
regenerating them.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path


ROOT = Path(__file__).resolve().parents[1]


@dataclass
class Workload:
    name: str
    kind: str                 # "er" or "rmat"
    scale: int = 0            # rmat: log2 vertices
    n: int = 0                # er: vertices
    m: int = 0                # er: edges
    avg_degree: int = 16
    labels: int = 16
    zipf: bool = True
    seed: int = 1
    queries_file: str | None = None
    description: str = ""
    extra: dict = field(default_factory=dict)

    def graph(self, threads: int = 0):
        from .native import HostGraph  # the library is loaded only when a graph is made
        if self.kind == "er":
            return HostGraph.er(self.n, self.m, self.labels, seed=self.seed, zipf=self.zipf)
        return HostGraph.rmat(self.scale, self.avg_degree, self.labels, seed=self.seed, zipf=self.zipf,
                              threads=threads)

    def queries(self):
        """(queries, expected counts or None) from the committed fixture."""
        from .native import Query
        data = json.loads((ROOT / self.queries_file).read_text())
        qs = [Query(q["labels"], q["edges"]) for q in data["queries"]]
        counts = [q.get("count") for q in data["queries"]]
        return qs, counts, data


def load(name: str) -> Workload:
    return WORKLOADS[name]


def shard(n: int, rank: int, world: int) -> list[int]:
    """Query indices of `rank` when n queries are dealt round-robin to `world`
    ranks.  Each rank matches its share against its own replica of the data
    graph; no data moves between ranks (embeddings are independent per query)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(range(rank, n, world))


WORKLOADS = {
    "er1k": Workload("er1k", "er", n=1000, m=4000, labels=4, zipf=False, seed=1,
                     queries_file="tests/golden/workload_er1k.json",
                     description="ER G(1000, 4000), 4 uniform labels, 4-vertex walk queries"),
    "rmat20": Workload("rmat20", "rmat", scale=20, avg_degree=16, labels=16, seed=1,
                       queries_file="tests/golden/workload_rmat20.json",
                       description="R-MAT(0.57,0.19,0.19,0.05) 2^20 vertices, avg degree 16, 16 Zipf labels, "
                                   "80 4-5-vertex tree/sparse/dense walk queries of at most 10^8 embeddings"),
    "rmat22": Workload("rmat22", "rmat", scale=22, avg_degree=16, labels=32, seed=1,
                       queries_file="tests/golden/workload_rmat22.json",
                       description="R-MAT(0.57,0.19,0.19,0.05) 2^22 vertices, avg degree 16, 32 Zipf labels, "
                                   "1,024 4-5-vertex tree/sparse/dense walk queries of at most 10^7 embeddings"),
    "rmat24": Workload("rmat24", "rmat", scale=24, avg_degree=16, labels=32, seed=1,
                       queries_file="tests/golden/workload_rmat24.json",
                       description="R-MAT(0.57,0.19,0.19,0.05) 2^24 vertices, avg degree 16, 32 Zipf labels, "
                                   "170 4-5-vertex sparse/dense walk queries of at most 10^7 embeddings "
                                   "(the serving configuration; 34,384 draws filled 170 of 256 slots, no "
                                   "tree stays within 10^7)"),
    "rmat22_k4to7": Workload("rmat22_k4to7", "rmat", scale=22, avg_degree=16, labels=32, seed=1,
                             queries_file="tests/golden/workload_rmat22_k4to7.json",
                             description="R-MAT(0.57,0.19,0.19,0.05) 2^22 vertices, avg degree 16, 32 Zipf labels, "
                                         "64 walk queries of 4, 5, 6 and 7 vertices (16 each; tree/sparse/dense "
                                         "where decidable, else dense) of at most 10^9 embeddings"),
    "rmat24_k4to7": Workload("rmat24_k4to7", "rmat", scale=24, avg_degree=16, labels=32, seed=1,
                             queries_file="tests/golden/workload_rmat24_k4to7.json",
                             description="R-MAT(0.57,0.19,0.19,0.05) 2^24 vertices, avg degree 16, 32 Zipf labels, "
                                         "47 walk queries of 4, 5 and 6 vertices (tree/sparse/dense where "
                                         "decidable, else dense) of at most 10^9 embeddings: the serving graph's "
                                         "widest decidable requests (no 7-vertex draw within 10^9 embeddings in "
                                         "420 s of screening)"),
}
