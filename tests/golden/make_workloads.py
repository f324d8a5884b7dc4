"""Generate the committed query sets of the benchmark workloads with their
exact embedding counts (computed here by the CPU oracle).

    python tests/golden/make_workloads.py er1k rmat20 rmat22

Queries are drawn by seeded random-walk extraction (smg_gen_query) with the
configured vertex counts and shapes.  On R-MAT graphs with Zipf labels almost
every walk-extracted query has far more embeddings than any exact enumerator
can count (on R-MAT 2^22 / 32 labels no drawn query with 6+ vertices stayed
under 10^8 partial matches), so a drawn query is kept only when the oracle
finishes it within BUDGET partial matches; otherwise the next seed is tried.
The acceptance budget and the number of draws per kept query are recorded in
the fixture.
"""
from __future__ import annotations

import json
import random
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from clustersm_gb300.workloads import load  # noqa: E402
from clustersm_gb300.native import Query  # noqa: E402

SPECS = {
    # name: (number of queries, k choices, shapes, oracle budget, max draws per slot)
    "er1k": (96, [4], ["tree", "sparse", "dense"], 10**8, 2000),
    "rmat20": (96, [8], ["tree", "sparse", "dense"], 5 * 10**7, 400),
    "rmat22": (1024, list(range(4, 17)), ["tree", "sparse", "dense"], 2 * 10**7, 60),
}


def main(names):
    for name in names:
        wl = load(name)
        nq, ks, shapes, budget, draws = SPECS[name]
        t0 = time.time()
        g = wl.graph()
        rng = random.Random(f"{name}-slots")
        out, tried = [], 0
        for slot in range(nq):
            k = rng.choice(ks)
            shape = shapes[slot % len(shapes)]
            kept = None
            for attempt in range(draws):
                seed = (slot << 20) | attempt
                try:
                    q = Query.generate(g, k, shape, seed=seed)
                except Exception:
                    continue
                tried += 1
                c, used = oracle.count_budget(g, q, budget)
                if used is not None:
                    kept = (q, c, attempt, seed)
                    break
            if kept is None:
                continue
            q, c, attempt, seed = kept
            out.append({"slot": slot, "k": int(q.k), "shape": shape, "seed": seed, "draws": attempt + 1,
                        "labels": q.labels.tolist(), "edges": q.edges.tolist(), "count": int(c)})
            print(f"{name} slot {slot}: k={q.k} {shape} count={c} draws={attempt + 1}", flush=True)
        path = ROOT / wl.queries_file
        path.write_text(json.dumps({
            "workload": name, "generator": "tests/golden/make_workloads.py", "oracle_budget": budget,
            "max_draws_per_slot": draws, "slots": nq, "kept": len(out), "draws_total": tried,
            "seconds": round(time.time() - t0, 1), "queries": out}, separators=(",", ":")))
        print(f"{name}: kept {len(out)} of {nq} slots ({tried} draws) -> {path}", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(SPECS))
