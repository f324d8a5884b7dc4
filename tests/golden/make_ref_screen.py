"""Screen workload queries for the reference's own GPU filter and join, and
commit the result as tests/golden/ref_screen_<workload>.json.

Run from the repository root (CPU only; uses the oracle):
    python tests/golden/make_ref_screen.py er1k rmat20

The reference's kernels write out of bounds, or read uninitialised memory, on
some inputs.  A query is handed to the reference (oracle/_ref/ClusterSM or
oracle/_ref/ref_match) only when, by reading its code, every access stays in
bounds:

  labels   every query label < 16: the initial filter keeps query
           neighbour-label counts in a [32][16] shared table
           (filter.cu:426-437); k <= 16 (C_MAX_VQ, globals.cu:59) and at most
           64 query edges (MAX_EQ, defs.h:12).
  clusters at most 150 clusters and 100 layers (MAX_CLUSTERS, MAX_LAYERS,
           defs.h:15-16; filter.cu:148, structure.cu:157-181).
  combine  no combine records.  combineMultipleClustersKernel indexes its
           in-place AND with num_small_clusters as the row width
           (filter.cu:861), which runs past the bitmap when there are more
           small clusters than bitmap words, and its new-cluster OR sets bits
           without a label test (filter.cu:858-863), after which
           collectCandidatesKernel can write more candidates than the
           MAX_L_FREQ-row list holds (filter.cu:1206).
  encode   every layer-0 cluster core has 0 or at least 16 initial
           candidates.  encode() sizes the grid from a host count that is
           still zero (filter.cu:982-983; main.cu:102-103), so encodeKernel
           runs one block of 16 warps; a warp whose index is not below the
           candidate count then uses s_core_v[wid] without writing it
           (filter.cu:618-634), an uninitialised shared word used as a vertex
           id.
  rows     every level of the breadth-first join holds at most
           min(MAX_RES, 2^32 / k) / 2 rows (MAX_RES defs.h:20).  Row writes
           are unchecked (join.cu:158-166) and their index is 32-bit
           (join.cu:163-165).  Levels are counted by oracle_ref_rows in the
           reference's own edge order with the oracle's final candidates.
           Without combines those are the reference's candidates, or a
           superset: encodeKernel's and mergeKernel's plain |= on the core
           word (filter.cu:633, 713) can only lose bits.

The data graph labels are as generated (er1k: 4 labels, rmat20: 16 labels).
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from clustersm_gb300.native import Plan  # noqa: E402
from clustersm_gb300.workloads import load  # noqa: E402

MAX_RES = 500_000_000


def screen(host, q, plan):
    """(reason or None, rows per level or None, initial candidates of layer-0 cores)."""
    v = plan.view
    k, E = v.k, v.num_edges
    labels = list(q.labels.tolist())
    if max(labels) >= 16 or k > 16 or E > 64:
        return "labels", None, None
    if v.num_clusters > 150 or v.num_layers > 100:
        return "clusters", None, None
    if v.num_combines:
        return "combine", None, None
    vm0 = oracle.nlc_filter(host, plan)
    cores = {}
    for c in range(v.num_clusters):
        if v.cluster_layer[c] == 0:
            u = v.slots[v.cluster_offsets[c]]
            cores[int(u)] = int(np.count_nonzero((vm0 >> np.uint32(u)) & np.uint32(1)))
    if any(0 < n < 16 for n in cores.values()):
        return "encode", None, cores
    _, cm = oracle.encode(host, plan, vm0)
    limit = min(MAX_RES, (1 << 32) // k) // 2
    rows = oracle.ref_rows(host, plan, cm, limit=limit)
    if any(r is None for r in rows):
        return "rows", rows, cores
    return None, rows, cores


def main(names):
    for name in names:
        wl = load(name)
        host = wl.graph()
        qs, counts, _ = wl.queries()
        t0 = time.time()
        out = []
        for i, (q, want) in enumerate(zip(qs, counts)):
            plan = Plan(q)
            why, rows, cores = screen(host, q, plan)
            if why is None and rows[-1] != want:
                sys.exit(f"{name} query {i}: last level {rows[-1]} != committed count {want}")
            out.append({"index": i, "k": q.k, "edges": int(plan.view.num_edges), "run": why is None,
                        "excluded_by": why, "rows": rows, "core_candidates": cores, "count": want})
        kept = sum(r["run"] for r in out)
        reasons = {}
        for r in out:
            if r["excluded_by"]:
                reasons[r["excluded_by"]] = reasons.get(r["excluded_by"], 0) + 1
        dst = ROOT / "tests" / "golden" / f"ref_screen_{name}.json"
        dst.write_text(json.dumps({"workload": name, "queries": len(out), "run": kept, "excluded": reasons,
                                   "seconds": round(time.time() - t0, 1), "screen": out},
                                  separators=(",", ":")))
        print(f"{name}: {kept} of {len(out)} queries screened in, excluded {reasons} -> {dst}")


if __name__ == "__main__":
    main(sys.argv[1:] or ["er1k", "rmat20"])
