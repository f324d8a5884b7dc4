"""The host-side plan equals what the reference's own host code produces
(tests/golden/ref_plans.json, made by tests/golden/make_ref_plans.py from
oracle/_ref/ref_plan, which runs decycle.cpp:6, filter.cu:127 clustering and
order.cpp:150 compiled from the reference's sources)."""
import json
from pathlib import Path

import pytest

from clustersm_gb300.native import Plan, Query, SmgError

CASES = json.loads((Path(__file__).parent / "golden" / "ref_plans.json").read_text())["cases"]


def compare(p, r):
    npl = [0] * p["num_layers"]
    for lay in p["cluster_layer"]:
        npl[lay] += 1
    assert p["tree_offsets"] == r["tree_offsets"]
    assert p["tree_neighbors"] == r["tree_neighbors"]
    assert p["num_clusters"] == r["num_clusters"]
    assert p["num_layers"] == r["num_layers"]
    assert p["cluster_offsets"] == r["cluster_offsets"]
    assert p["slots"] == r["slots"]
    assert npl == r["num_clusters_per_layer"]
    assert p["merge_left"] == r["merge_left"]
    assert p["merge_right"] == r["merge_right"]
    assert p["merge_vertex"] == r["merge_vertex"]
    assert [p["cluster_layer"][c] - 1 for c in p["merge_cluster"]] == r["merge_layer"]
    assert p["combine_out"] == r["combine_out"]
    assert p["combine_type"] == r["combine_type"]
    assert p["combine_others"] == r["combine_others"]
    assert p["root"] == r["root"]
    assert [list(e) for e in p["edge_order"]] == r["edge_order"]


def test_fixture_coverage():
    assert len(CASES) >= 500
    assert sum(1 for c in CASES if c["ref"]["combine_out"]) >= 100
    assert sum(1 for c in CASES if 0 in c["ref"]["combine_type"]) >= 50


@pytest.mark.parametrize("i", range(0, len(CASES)))
def test_plan_matches_reference(i):
    c = CASES[i]
    q = Query(c["query"]["labels"], c["query"]["edges"])
    compare(Plan(q).to_dict(), c["ref"])


def test_example_plan(example):
    _, q = example
    p = Plan(q).to_dict()
    assert p["slots"] == [1, 0, 2, 3, 3, 1, 4, 3, 1]
    assert p["root"] == 3
    assert p["order"] == [3, 1, 4, 0, 2]


@pytest.mark.parametrize("labels,edges", [
    ([0], []),                          # one vertex
    ([0, 0, 0, 0], [0, 1, 2, 3]),       # disconnected
    ([0, 0], [0, 0]),                   # self-loop
    ([0, 0], [0, 1, 1, 0]),             # repeated edge
    ([0] * 33, [i for j in range(32) for i in (j, j + 1)]),  # 33 vertices
])
def test_rejected_queries(labels, edges):
    with pytest.raises(SmgError) as e:
        Plan(Query(labels, edges))
    assert e.value.status == 4


def test_batch_plans_match_reference():
    """smg_plan_create_batch (all host threads) gives every golden case the
    same plan as the reference's own host code."""
    qs = [Query(c["query"]["labels"], c["query"]["edges"]) for c in CASES]
    for p, c in zip(Plan.batch(qs), CASES):
        compare(p.to_dict(), c["ref"])


def test_batch_plans_reject_like_single():
    """A rejected query fails the whole batch with the first failing query's
    status and reason, and no plan is handed out."""
    good = Query([0, 1, 0], [0, 1, 1, 2])
    bad = Query([0, 0], [0, 0])  # self-loop
    with pytest.raises(SmgError) as single:
        Plan(bad)
    with pytest.raises(SmgError) as e:
        Plan.batch([good, bad, good])
    assert e.value.status == single.value.status == 4
    # the same reason as the single call (the message past the call's name)
    assert str(e.value).split(":", 1)[-1] == str(single.value).split(":", 1)[-1]
    assert len(Plan.batch([])) == 0
