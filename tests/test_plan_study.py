"""The cluster filter stays a necessary condition under every plan the
reference's rules can produce (filter.cu:127-401 driven by decycle.cpp:6-134
on renumbered queries), and so does the intersection of several plans'
candidate sets.  The plan study (tests/plan_study.py) relies on both."""
import numpy as np
import pytest

import oracle
from clustersm_gb300 import workloads
from clustersm_gb300.native import HostGraph, Plan, Query
from tests.plan_study import candidate_masks, perms_for, renumbered, study_query


def test_renumbered_query_keeps_count():
    g = HostGraph.er(300, 1500, 3, seed=4)
    q = Query.generate(g, 5, "dense", seed=2)
    base = oracle.count(g, q)
    for p in [(4, 3, 2, 1, 0), (1, 0, 3, 4, 2)]:
        assert oracle.count(g, renumbered(q, p)) == base


def test_er1k_plans_sound_and_identical():
    wl = workloads.load("er1k")
    g = wl.graph()
    qs, _, _ = wl.queries()
    import random
    rng = random.Random(3)
    for q in qs[:24]:
        r, cm_ref, inter, ideal = study_query(g, q, perms_for(q.k, 0, rng))
        assert r["sound"], r
        assert r["ideal"] <= r["inter"] <= r["best"] <= r["ref"] <= r["nlc"]


@pytest.mark.parametrize("kind,shape", [("rmat", "tree"), ("rmat", "sparse"), ("rmat", "dense"),
                                        ("er", "sparse"), ("er", "dense")])
def test_random_plans_sound(kind, shape):
    import random
    g = HostGraph.rmat(12, 8, 16, seed=9) if kind == "rmat" else HostGraph.er(400, 2400, 3, seed=5)
    rng = random.Random(kind + shape)
    checked = combines = 0
    for s in range(8):
        q = Query.generate(g, 5 + s % 3, shape, seed=100 + s)
        perms = perms_for(q.k, 8, rng)
        combines += sum(Plan(renumbered(q, p)).view.num_combines > 0 for p in perms)
        r, cm_ref, inter, ideal = study_query(g, q, perms, max_rows=1 << 16)
        checked += ideal is not None
        assert r["ideal"] is None or r["sound"], r
        assert r["inter"] <= r["best"] <= r["ref"] <= r["nlc"]
        # each plan's final sets contain the ideal pairs
        if ideal is not None:
            for p in perms[:3]:
                cm, _, _ = candidate_masks(g, q, p)
                assert np.all((ideal & ~cm) == 0)
    assert checked >= 2
    if (kind, shape) == ("er", "sparse"):
        assert combines >= 8      # plans with combine records (filter.cu:749-873) are covered
