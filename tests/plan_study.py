"""Study of alternative query plans: how much smaller could the cluster
filter's candidate sets be under another spanning tree, vertex cover and
cluster layout than under the reference's own (filter.cu:127-401)?

The reference's plan is a function of the query's vertex ids: the spanning
tree grows by BFS from the first vertex of maximum degree, neighbours in
file order (decycle.cpp:6-134), and the cover DP and the clustering follow
the tree (filter.cu:23-112, 127-401).  Renumbering the query's vertices gives
an isomorphic query (same embedding count, candidate sets carried along by
the renumbering) whose plan can differ in every one of those choices.  So
each plan here is the library's own plan of a renumbered query, and its
final candidate sets are the oracle's cluster filter (oracle_nlc_filter +
oracle_encode) for that plan, mapped back to the original vertex ids.

Per query it reports
  nlc    sum over u of |C(u)| after the NLC filter alone (filter.cu:404-539),
  ref    the same after the cluster filter under the reference's plan,
  best   the smallest sum over the renumberings tried,
  inter  the sum for the intersection of all tried plans' sets (still a
         necessary condition: every plan's filter is),
  ideal  the number of (u, v) pairs used by at least one embedding, where
         the embeddings are few enough to enumerate.

    python -m tests.plan_study --workload er1k
    python -m tests.plan_study --workload rmat20 --queries 24 --perms 24
"""
from __future__ import annotations

import argparse
import itertools
import json
import random
import time

import numpy as np

import oracle
from clustersm_gb300.native import Plan, Query


def renumbered(q: Query, perm):
    """The query with vertex u renamed perm[u]; edges keep their file order."""
    perm = np.asarray(perm, dtype=np.int64)
    labels = np.empty(q.k, dtype=np.uint32)
    labels[perm] = q.labels
    edges = perm[q.edges.astype(np.int64)]
    return Query(labels, edges)


def candidate_masks(graph, q: Query, perm):
    """Final candidate masks of the renumbered query's plan, with bit u meaning
    original query vertex u; also the NLC-only masks."""
    rq = renumbered(q, perm)
    plan = Plan(rq)
    vm0 = oracle.nlc_filter(graph, plan)
    _, cm = oracle.encode(graph, plan, vm0)
    back = np.zeros_like(cm)
    back0 = np.zeros_like(vm0)
    for u in range(q.k):
        back |= ((cm >> np.uint32(perm[u])) & np.uint32(1)) << np.uint32(u)
        back0 |= ((vm0 >> np.uint32(perm[u])) & np.uint32(1)) << np.uint32(u)
    return back, back0, plan


def popsum(masks) -> int:
    return int(np.unpackbits(masks.view(np.uint8)).sum())


def ideal_masks(graph, q: Query, max_rows: int):
    cnt, used = oracle.count_budget(graph, q, 16 * max_rows)
    if used is None or cnt > max_rows:
        return None
    cnt, rows = oracle.embeddings(graph, q, max_rows=max_rows)
    if cnt > max_rows:
        return None
    rows = np.asarray(rows, dtype=np.int64).reshape(-1, q.k)
    m = np.zeros(graph.n, dtype=np.uint32)
    for u in range(q.k):
        m[np.unique(rows[:, u])] |= np.uint32(1 << u)
    return m


def study_query(graph, q: Query, perms, max_rows=1 << 20):
    ident = tuple(range(q.k))
    cm_ref, nlc, _ = candidate_masks(graph, q, ident)
    sizes, inter, distinct = [], cm_ref.copy(), set()
    for p in perms:
        cm, _, plan = candidate_masks(graph, q, p)
        d = plan.to_dict()
        distinct.add(json.dumps([d.get("num_clusters"), d.get("num_slots"), d.get("root")]))
        sizes.append(popsum(cm))
        inter &= cm
    ideal = ideal_masks(graph, q, max_rows)
    out = {"k": q.k, "edges": len(q.edges) // 2, "nlc": popsum(nlc), "ref": popsum(cm_ref),
           "best": min(sizes + [popsum(cm_ref)]), "worst": max(sizes + [popsum(cm_ref)]),
           "inter": popsum(inter), "plans": len(perms) + 1, "shapes": len(distinct),
           "ideal": None if ideal is None else popsum(ideal)}
    if ideal is not None:
        # every filter is a necessary condition: the ideal pairs survive all of them
        out["sound"] = bool(np.all((ideal & ~inter) == 0) and np.all((ideal & ~cm_ref) == 0))
    return out, cm_ref, inter, ideal


def perms_for(k: int, limit: int, rng: random.Random):
    all_p = [p for p in itertools.permutations(range(k)) if p != tuple(range(k))]
    if limit <= 0 or len(all_p) <= limit:
        return all_p
    return rng.sample(all_p, limit)


def main():
    from clustersm_gb300 import workloads
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="er1k")
    ap.add_argument("--queries", type=int, default=0, help="first N queries (0 = all)")
    ap.add_argument("--perms", type=int, default=0, help="renumberings per query (0 = all)")
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args()
    wl = workloads.load(args.workload)
    t0 = time.time()
    graph = wl.graph()
    qs, _, _ = wl.queries()
    if args.queries:
        qs = qs[: args.queries]
    rng = random.Random(args.seed)
    rows = []
    for i, q in enumerate(qs):
        r, *_ = study_query(graph, q, perms_for(q.k, args.perms, rng))
        r["i"] = i
        rows.append(r)
        print(json.dumps(r), flush=True)
    tot = {key: sum(r[key] for r in rows) for key in ("nlc", "ref", "best", "inter")}
    with_ideal = [r for r in rows if r["ideal"] is not None]
    summary = {"workload": args.workload, "queries": len(rows), **tot,
               "best_over_ref": tot["best"] / max(tot["ref"], 1),
               "inter_over_ref": tot["inter"] / max(tot["ref"], 1),
               "queries_best_below_ref": sum(r["best"] < r["ref"] for r in rows),
               "ideal_queries": len(with_ideal),
               "ideal_over_ref": (sum(r["ideal"] for r in with_ideal) /
                                  max(sum(r["ref"] for r in with_ideal), 1)) if with_ideal else None,
               "all_sound": all(r.get("sound", True) for r in rows),
               "seconds": round(time.time() - t0, 1)}
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
