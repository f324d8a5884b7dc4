"""Generate the committed query sets of the benchmark workloads, with exact
embedding counts checked by two independent implementations.

    # on a GPU host: draw and screen queries (writes gpurun_out/workload_<name>.json)
    python tests/golden/make_workloads.py gpu rmat22 rmat20
    # on any host: recount every kept query with the CPU oracle and commit
    python tests/golden/make_workloads.py verify rmat22 rmat20
    # small workloads drawn and counted by the oracle alone
    python tests/golden/make_workloads.py cpu er1k

Queries are drawn by seeded random-walk extraction (smg_gen_query).  On R-MAT
graphs with Zipf labels, walk-extracted queries have embedding counts far
beyond exact enumeration: on R-MAT 2^22 / 32 labels only 13 of 187 drawn
queries (4..16 vertices) had at most 10^8 embeddings, and none of those had
more than 5 vertices.  A drawn query is therefore kept when its exact count is at
most the workload's count limit, decided on the GPU with the library's per-query count limit
(the join stops a query as soon as its running count passes the limit) and a
device deadline; each slot retries new seeds up to MAX_DRAWS times (drawn
and screened in rounds, one batched call per round).  The limit is 10^8 for the 2^20-vertex and
smaller graphs and 10^7 for the 1,024-query 2^22-vertex batch, which keeps
one batched pass over all 1,024 queries within seconds.
Every kept count is then recomputed by the CPU oracle; a fixture is written
only when all counts agree.
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import random
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from clustersm_gb300.workloads import load  # noqa: E402
from clustersm_gb300.native import Query, SmgError  # noqa: E402

MAX_DRAWS = 64
SPECS = {
    # name: (slots, vertex counts, shapes, count limit)
    "er1k": (96, [4], ["induced"], 10**8),
    "rmat20": (96, [4, 5], ["tree", "sparse", "dense"], 10**8),
    "rmat22": (1024, [4, 5], ["tree", "sparse", "dense"], 10**7),
}


def draws(name):
    nq, ks, shapes, _ = SPECS[name]
    rng = random.Random(f"{name}-slots")
    for slot in range(nq):
        k = rng.choice(ks)
        shape = shapes[slot % len(shapes)]
        for attempt in range(MAX_DRAWS):
            yield slot, attempt, k, shape, (slot << 20) | attempt


def record(slot, attempt, k, shape, seed, q, count, key):
    return {"slot": slot, "k": int(k), "shape": shape, "seed": seed, "draws": attempt + 1,
            "labels": q.labels.tolist(), "edges": q.edges.tolist(), key: int(count)}


def gen_gpu(name, seconds=None):
    """Screen drawn queries on the GPU in rounds: each round draws the next
    seed of every unfilled slot and matches them all in one batched call with
    the per-query count limit; queries that finish under the limit fill their
    slots.  A round that hits the device deadline (SMG_TIME_LIMIT_S, 120 s
    unless set) is re-screened one query at a time."""
    from clustersm_gb300 import native
    from clustersm_gb300.native import Context, DeviceGraph, Plan
    os.environ.setdefault("SMG_TIME_LIMIT_S", "120")
    wl = load(name)
    nq, ks, shapes, limit = SPECS[name]
    t0 = time.time()
    host = wl.graph()
    ctx = Context(0)
    dev = DeviceGraph(ctx, host)
    rng = random.Random(f"{name}-slots")
    slot_k = [rng.choice(ks) for _ in range(nq)]
    kept = {}
    tried = timeouts = 0
    path = ROOT / "gpurun_out" / f"workload_{name}.json"
    path.parent.mkdir(exist_ok=True)

    def save(complete):
        out = [kept[s] for s in sorted(kept)]
        path.write_text(json.dumps({"workload": name, "count_limit": limit, "max_draws": MAX_DRAWS,
                                    "slots": nq, "kept": len(out), "draws_total": tried, "timeouts": timeouts,
                                    "seconds": round(time.time() - t0, 1), "complete": complete,
                                    "queries": out}, separators=(",", ":")))

    for attempt in range(MAX_DRAWS):
        if seconds and time.time() - t0 > seconds:
            break
        todo = [(slot, slot_k[slot], shapes[slot % len(shapes)], (slot << 20) | attempt)
                for slot in range(nq) if slot not in kept]

        def draw(item):
            try:
                return item + (Query.generate(host, item[1], item[2], seed=item[3]),)
            except SmgError:
                return None

        # the generator runs in C with the interpreter lock released
        with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
            batch = [b for b in ex.map(draw, todo) if b is not None]
        if not batch:
            break
        tried += len(batch)
        plans = [Plan(b[4]) for b in batch]
        try:
            counts, _ = native.match_batch(ctx, dev, plans, max_count=limit)
            results = [None if c == 2**64 - 1 else int(c) for c in counts.tolist()]
        except SmgError as e:
            print(f"{name}: round {attempt}: batched screening failed ({e}); screening one by one", flush=True)
            results = []
            for p in plans:
                try:
                    r, _ = native.match(ctx, dev, p, max_count=limit)
                    results.append(None if r.limit_hit else int(r.count))
                except SmgError as e1:
                    timeouts += 1
                    if timeouts <= 5:
                        print(f"{name}: {e1}", flush=True)
                    results.append(None)
        for (slot, k, shape, seed, q), c in zip(batch, results):
            if c is not None:
                kept[slot] = record(slot, attempt, k, shape, seed, q, c, "gpu_count")
        save(False)
        print(f"{name}: round {attempt}: {len(kept)} kept, {tried} draws, {timeouts} timeouts, "
              f"{time.time() - t0:.0f} s", flush=True)
    save(True)
    print(f"{name}: kept {len(kept)} of {nq} slots, {tried} draws -> {path}", flush=True)


def verify(name, src=None):
    import oracle
    wl = load(name)
    src = Path(src) if src else ROOT / "gpurun_out" / f"workload_{name}.json"
    data = json.loads(src.read_text())
    host = wl.graph()
    t0 = time.time()
    bad = 0
    for rec in data["queries"]:
        q = Query(rec["labels"], rec["edges"])
        rec["count"] = oracle.count(host, q)
        if rec["count"] != rec["gpu_count"]:
            bad += 1
            print(f"MISMATCH slot {rec['slot']}: oracle {rec['count']} gpu {rec['gpu_count']}")
    data["oracle_seconds"] = round(time.time() - t0, 1)
    data["verified_by"] = "oracle_count (CPU backtracking) == GPU count for every query"
    if bad:
        sys.exit(f"{bad} mismatches: fixture not written")
    dst = ROOT / wl.queries_file
    dst.write_text(json.dumps(data, separators=(",", ":")))
    print(f"{name}: {len(data['queries'])} counts verified in {data['oracle_seconds']} s -> {dst}")


def gen_cpu(name):
    import oracle
    wl = load(name)
    host = wl.graph()
    out, done_slot, tried = [], -1, 0
    for slot, attempt, k, shape, seed in draws(name):
        if slot == done_slot:
            continue
        try:
            q = Query.generate(host, k, shape, seed=seed)
        except SmgError:
            continue
        tried += 1
        c, used = oracle.count_budget(host, q, 10**9)
        if used is None or c > SPECS[name][3]:
            continue
        out.append(record(slot, attempt, k, shape, seed, q, c, "count"))
        done_slot = slot
    dst = ROOT / wl.queries_file
    dst.write_text(json.dumps({"workload": name, "count_limit": SPECS[name][3], "max_draws": MAX_DRAWS,
                               "slots": SPECS[name][0], "kept": len(out), "draws_total": tried,
                               "verified_by": "oracle_count (CPU backtracking)", "queries": out},
                              separators=(",", ":")))
    print(f"{name}: kept {len(out)} -> {dst}")


if __name__ == "__main__":
    mode, names = sys.argv[1], sys.argv[2:]
    budget = float(os.environ.get("WORKLOAD_SECONDS", "0")) or None
    for n in names:
        if mode == "gpu":
            gen_gpu(n, budget)
        else:
            {"verify": verify, "cpu": gen_cpu}[mode](n)
