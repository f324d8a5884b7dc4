"""Generate tests/golden/ref_plans.json: query plans produced by the reference's
own host code (decycle.cpp, filter.cu clustering, order.cpp), run through
oracle/_ref/ref_plan (built by oracle/build_ref.sh from the reference sources).

Run from the repository root, in a container that has the reference tree:
    bash oracle/build_ref.sh && python tests/golden/make_ref_plans.py

Queries: random connected labelled graphs (2-24 vertices, random edge order
and orientation, sparse to complete) plus random-walk queries of every shape
extracted from a small R-MAT graph.  Queries whose clustering would exceed the
reference's fixed tables (MAX_CLUSTERS = 150, defs.h:15) are not run through
the reference.
"""
from __future__ import annotations

import json
import random
import subprocess
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from clustersm_gb300.native import HostGraph, Plan, Query  # noqa: E402

REF_BIN = ROOT / "oracle" / "_ref" / "ref_plan"
OUT = Path(__file__).resolve().parent / "ref_plans.json"


def random_connected(rng: random.Random, k: int, extra_p: float, nlabels: int) -> Query:
    perm = list(range(k))
    rng.shuffle(perm)
    edges = set()
    for i in range(1, k):
        a, b = perm[i], perm[rng.randrange(i)]
        edges.add((min(a, b), max(a, b)))
    for a in range(k):
        for b in range(a + 1, k):
            if rng.random() < extra_p:
                edges.add((a, b))
    edges = list(edges)
    rng.shuffle(edges)
    flat = []
    for a, b in edges:
        if rng.random() < 0.5:
            a, b = b, a
        flat += [a, b]
    labels = [rng.randrange(nlabels) for _ in range(k)]
    return Query(labels, flat)


def queries():
    rng = random.Random(20261203)
    out = []
    for i in range(360):
        k = rng.choice([2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 16, 20, 24])
        p = rng.choice([0.0, 0.05, 0.15, 0.3, 0.6, 1.0])
        out.append(("random", random_connected(rng, k, p, rng.choice([1, 2, 4, 8]))))
    g = HostGraph.rmat(12, 16, 8, seed=7)
    for i in range(150):
        k = 4 + i % 13
        shape = ["tree", "sparse", "dense"][i % 3]
        out.append((f"rmat-{shape}", Query.generate(g, k, shape, seed=1000 + i)))
    return out


def main():
    if not REF_BIN.exists():
        sys.exit(f"{REF_BIN} missing: run oracle/build_ref.sh first")
    cases = []
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for i, (kind, q) in enumerate(queries()):
            plan = Plan(q).to_dict()
            if plan["num_clusters"] > 150 or plan["num_layers"] > 99:
                continue
            p = Path(td) / f"q{i}.in"
            q.write(p)
            paths.append((p, kind, q))
        for p, kind, q in paths:
            r = subprocess.run([str(REF_BIN), str(p)], capture_output=True, text=True, timeout=60)
            if r.returncode != 0:
                print(f"reference failed on {kind} query {p.name}: rc={r.returncode}", file=sys.stderr)
                continue
            ref = json.loads(r.stdout)[0]
            ref.pop("file")
            cases.append({"kind": kind, "query": q.to_dict(), "ref": ref})
    OUT.write_text(json.dumps({"generator": "tests/golden/make_ref_plans.py", "cases": cases},
                              separators=(",", ":")))
    print(f"{len(cases)} cases -> {OUT}")


if __name__ == "__main__":
    main()
