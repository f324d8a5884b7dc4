"""Generate the committed query sets of the benchmark workloads, with exact
embedding counts checked by two independent implementations.

    # on a GPU host: draw and screen queries (writes $WORKLOAD_DIR/workload_<name>.json,
    # default screened/ at the repository root)
    python tests/golden/make_workloads.py gpu rmat22 rmat20
    # on any host: recount every kept query with the CPU oracle and commit
    python tests/golden/make_workloads.py verify rmat22 rmat20
    # small workloads drawn and counted by the oracle alone
    python tests/golden/make_workloads.py cpu er1k
    # on a GPU host: per-(k, shape) feasibility of walk queries on a
    # workload's graph (writes tests/golden/feasibility_<name>.json)
    python tests/golden/make_workloads.py feasibility rmat22 rmat20

Queries are drawn by seeded random-walk extraction (smg_gen_query).  On R-MAT
graphs with Zipf labels, walk-extracted queries have embedding counts far
beyond exact enumeration: on R-MAT 2^22 / 32 labels only 13 of 187 drawn
queries (4..16 vertices) had at most 10^8 embeddings, and none of those had
more than 5 vertices.  A drawn query is therefore kept when its exact count
is at most the workload's count limit, decided on the GPU with the library's
per-query count limit (the join stops a query soon after its running count
passes the limit) and a device deadline.  Each slot draws new seeds in the
phases `phases()` lists (drawn and screened in rounds, one batched call per
round) and keeps its first draw under the limit.  The limit is 10^8 for the
2^20-vertex and smaller graphs and 10^7 for the 1,024-query 2^22-vertex batch,
which keeps one batched pass over all 1,024 queries within seconds.
WORKLOAD_RESUME=<earlier output> continues an interrupted screening.
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
# where screening writes its draws and verification reads them
SCREEN_DIR = Path(os.environ.get("WORKLOAD_DIR", str(ROOT / "screened")))
sys.path.insert(0, str(ROOT))

from clustersm_gb300.workloads import load  # noqa: E402
from clustersm_gb300.native import Query, SmgError  # noqa: E402

MAX_DRAWS = 64
SPECS = {
    # name: (slots, vertex counts, shapes, count limit)
    "er1k": (96, [4], ["induced"], 10**8),
    "rmat20": (96, [4, 5], ["tree", "sparse", "dense"], 10**8),
    "rmat22": (1024, [4, 5], ["tree", "sparse", "dense"], 10**7),
    # the widest query sizes with decidable draws on R-MAT 2^22 (the
    # feasibility table): k = 4..7 in turn, each with every shape in turn; at
    # most 10^9 embeddings, so that the CPU oracle can verify every count
    "rmat22_k4to7": (64, [4, 5, 6, 7], ["tree", "sparse", "dense"], 10**9),
    # the serving graph (R-MAT 2^24): requests of the sizes that stay exact
    # within a serving budget (at most 10^7 embeddings each)
    "rmat24": (256, [4, 5], ["tree", "sparse", "dense"], 10**7),
    # the serving graph's widest decidable requests, drawn like rmat22_k4to7
    "rmat24_k4to7": (64, [4, 5, 6, 7], ["tree", "sparse", "dense"], 10**9),
}
# join steps a screened query may take (bounds the draws whose count is out of reach)
WORK_LIMIT = {"rmat22_k4to7": 1 << 30, "rmat24_k4to7": 1 << 30}


def slot_shape(name, slot):
    """(k, shape) of a slot: the wide workload cycles k first, then shapes;
    the others draw k at random and cycle shapes."""
    nq, ks, shapes, _ = SPECS[name]
    if name.endswith("_k4to7"):
        return ks[slot % len(ks)], shapes[(slot // len(ks)) % len(shapes)]
    return None, shapes[slot % len(shapes)]


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


def phases(name):
    """Draw phases of a workload's slots: (draws, k or None for the slot's own,
    shape or None for the slot's own).  On R-MAT 2^22, 5-vertex trees and most
    5-vertex sparse queries exceed 10^7 embeddings in every one of 64 draws, so
    slots still empty after the first phase fall back to 4-vertex queries of
    their shape, and then to 4-vertex dense ones."""
    if name in ("rmat22", "rmat24"):
        return [(64, None, None), (256, 4, None), (64, 4, "dense")]
    if name.endswith("_k4to7"):
        # trees of 6 or more vertices and most sparse ones are out of reach:
        # such slots fall back to dense queries of their size (at k = 7 about
        # one dense draw in 800 has at most 10^9 embeddings)
        return [(64, None, None), (8192, None, "dense")]
    return [(MAX_DRAWS, None, None)]


def slot_attempts(name, slot, k, shape):
    """(attempt, k, shape, seed) for every draw of a slot, in order."""
    a = 0
    for draws, pk, pshape in phases(name):
        for _ in range(draws):
            yield a, pk or k, pshape or shape, (slot << 20) | a
            a += 1


def gen_gpu(name, seconds=None, resume=None, per_round=16):
    """Screen drawn queries on the GPU in rounds.  Each round draws the next
    `per_round` attempts of every unfilled slot and matches them all in one
    batched call with the per-query count limit; a slot keeps its lowest
    attempt that finishes under the limit, which is the query a one-by-one
    draw would keep.  A round that hits the device deadline (SMG_TIME_LIMIT_S,
    120 s unless set) is re-screened one query at a time.  `resume` names an
    earlier output whose kept slots stand and whose `next_attempt` (or, for a
    complete first-phase run, the first phase's size) says where each unfilled
    slot continues."""
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
    slot_sh = [shapes[s % len(shapes)] for s in range(nq)]
    for s in range(nq):
        k0, sh0 = slot_shape(name, s)
        if k0 is not None:
            slot_k[s], slot_sh[s] = k0, sh0
    plan_of = {s: list(slot_attempts(name, s, slot_k[s], slot_sh[s])) for s in range(nq)}
    kept, nxt = {}, {s: 0 for s in range(nq)}
    tried = timeouts = 0
    if resume:
        old = json.loads(Path(resume).read_text())
        for rec in old["queries"]:
            kept[rec["slot"]] = rec
        first = phases(name)[0][0]
        for s in range(nq):
            nxt[s] = int(old.get("next_attempt", {}).get(str(s), first if old.get("complete") else 0))
        tried = old.get("draws_total", 0)
    path = SCREEN_DIR / f"workload_{name}.json"
    path.parent.mkdir(parents=True, exist_ok=True)

    def save(complete):
        out = [kept[s] for s in sorted(kept)]
        path.write_text(json.dumps({"workload": name, "count_limit": limit, "phases": phases(name),
                                    "slots": nq, "kept": len(out), "draws_total": tried, "timeouts": timeouts,
                                    "seconds": round(time.time() - t0, 1), "complete": complete,
                                    "next_attempt": {str(s): nxt[s] for s in range(nq) if s not in kept},
                                    "queries": out}, separators=(",", ":")))

    rnd = 0
    while True:
        if seconds and time.time() - t0 > seconds:
            break
        todo = []
        for s in range(nq):
            if s in kept:
                continue
            todo += [(s,) + a for a in plan_of[s][nxt[s]:nxt[s] + per_round]]
        if not todo:
            break

        def draw(item):
            s, a, k, shape, seed = item
            try:
                return item + (Query.generate(host, k, shape, seed=seed),)
            except SmgError:
                return None

        # the generator runs in C with the interpreter lock released
        with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
            batch = [b for b in ex.map(draw, todo) if b is not None]
        tried += len(batch)
        plans = [Plan(b[5]) for b in batch]
        try:
            counts, _ = native.match_batch(ctx, dev, plans, max_count=limit, max_work=WORK_LIMIT.get(name, 0))
            results = [None if c == 2**64 - 1 else int(c) for c in counts.tolist()]
        except SmgError as e:
            print(f"{name}: round {rnd}: batched screening failed ({e}); screening one by one", flush=True)
            results = []
            for p in plans:
                try:
                    r, _ = native.match(ctx, dev, p, max_count=limit, max_work=WORK_LIMIT.get(name, 0))
                    results.append(None if r.limit_hit else int(r.count))
                except SmgError as e1:
                    timeouts += 1
                    if timeouts <= 5:
                        print(f"{name}: {e1}", flush=True)
                    results.append(None)
        best = {}
        for (s, a, k, shape, seed, q), c in zip(batch, results):
            if c is not None and (s not in best or a < best[s][0]):
                best[s] = (a, record(s, a, k, shape, seed, q, c, "gpu_count"))
        for s in {t[0] for t in todo}:
            if s in best:
                kept[s] = best[s][1]
            else:
                nxt[s] += per_round
        save(False)
        print(f"{name}: round {rnd}: {len(kept)} kept, {len(batch)} screened, {tried} draws, "
              f"{time.time() - t0:.0f} s", flush=True)
        rnd += 1
    save(True)
    print(f"{name}: kept {len(kept)} of {nq} slots, {tried} draws -> {path}", flush=True)


def verify(name, src=None):
    import oracle
    wl = load(name)
    src = Path(src) if src else SCREEN_DIR / f"workload_{name}.json"
    data = json.loads(src.read_text())
    host = wl.graph()
    t0 = time.time()
    bad = 0
    for j, rec in enumerate(data["queries"]):
        q = Query(rec["labels"], rec["edges"])
        t1 = time.time()
        rec["count"] = oracle.count(host, q)
        if os.environ.get("WORKLOAD_PROGRESS"):
            print(f"{name}: {j + 1}/{len(data['queries'])} k={rec['k']} count={rec['count']} "
                  f"{time.time() - t1:.1f} s", flush=True)
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


FEAS_KS = list(range(4, 17))
FEAS_SHAPES = ["tree", "sparse", "dense"]
FEAS_DRAWS = 64
FEAS_LIMITS = [10**7, 10**8, 10**10]
FEAS_WORK = 1 << 30  # join steps per query (about 0.1 s of the whole GPU)


def feasibility(name):
    """For every query size k = 4..16 and shape, draw FEAS_DRAWS walk queries
    (seeds apart from the workload's own) and count them in one batched call
    per cell with the count limit 10^10 and the work limit FEAS_WORK join
    steps per query.  A draw is decided when its exact count comes back; the
    cell records how many decided draws have at most 10^7, 10^8 and 10^10
    embeddings.  A cell whose batch hits the device deadline (SMG_TIME_LIMIT_S,
    set to 120 s here) is recorded as such."""
    from clustersm_gb300 import native
    from clustersm_gb300.native import Context, DeviceGraph, Plan
    os.environ.setdefault("SMG_TIME_LIMIT_S", "120")
    wl = load(name)
    host = wl.graph()
    ctx = Context(0)
    dev = DeviceGraph(ctx, host)
    cells = []
    t_all = time.time()
    for k in FEAS_KS:
        for si, shape in enumerate(FEAS_SHAPES):
            t0 = time.time()

            def draw(a):
                try:
                    return Query.generate(host, k, shape, seed=(1 << 40) | (k << 24) | (si << 20) | a)
                except SmgError:
                    return None

            with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
                qs = [q for q in ex.map(draw, range(FEAS_DRAWS)) if q is not None]
            cell = {"k": k, "shape": shape, "draws": FEAS_DRAWS, "generated": len(qs), "timeout": False}
            counts = []
            if qs:
                try:
                    got, _ = native.match_batch(ctx, dev, [Plan(q) for q in qs], max_count=FEAS_LIMITS[-1],
                                                max_work=FEAS_WORK)
                    counts = [None if c == 2**64 - 1 else int(c) for c in got.tolist()]
                except SmgError as e:
                    cell["timeout"] = True
                    cell["error"] = str(e)[:200]
            decided = sorted(c for c in counts if c is not None)
            for lim in FEAS_LIMITS:
                cell[f"le_{lim:.0e}".replace("+", "")] = sum(1 for c in decided if c <= lim)
            cell["undecided"] = len(counts) - len(decided)
            cell["median_decided"] = decided[len(decided) // 2] if decided else None
            cell["seconds"] = round(time.time() - t0, 2)
            cells.append(cell)
            print(json.dumps(cell), flush=True)
    dst = ROOT / "tests" / "golden" / f"feasibility_{name}.json"
    dst.write_text(json.dumps({"workload": name, "graph": wl.description.split(",")[0], "draws_per_cell": FEAS_DRAWS,
                               "count_limit": FEAS_LIMITS[-1], "work_limit_steps": FEAS_WORK,
                               "seconds": round(time.time() - t_all, 1), "cells": cells}, indent=0))
    print(f"{name}: feasibility table -> {dst}")


if __name__ == "__main__":
    mode, names = sys.argv[1], sys.argv[2:]
    budget = float(os.environ.get("WORKLOAD_SECONDS", "0")) or None
    resume = os.environ.get("WORKLOAD_RESUME") or None
    for n in names:
        if mode == "gpu":
            # rounds of the wide workload hold queries of up to 10^10 embeddings
            per_round = int(os.environ.get("WORKLOAD_PER_ROUND", "16"))
            gen_gpu(n, budget, resume, per_round=per_round)
        elif mode == "feasibility":
            feasibility(n)
        else:
            {"verify": verify, "cpu": gen_cpu}[mode](n)
