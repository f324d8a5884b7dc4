"""The CPU oracle against the known answer of the reference's example, against
brute force on tiny graphs, and the soundness of its cluster-bitmap
restatement (every embedding survives the filter)."""
import itertools
import random

import numpy as np
import pytest

import oracle
from clustersm_gb300.native import HostGraph, Plan, Query

EXAMPLE_EMBEDDINGS = [(0, 1, 4, 2, 3), (4, 1, 0, 2, 3), (5, 8, 7, 9, 10), (7, 8, 5, 9, 10)]


def test_example_known_answer(example):
    g, q = example
    g = g.sorted_copy()
    cnt, emb = oracle.embeddings(g, q)
    assert cnt == 4
    assert [tuple(r) for r in emb.tolist()] == EXAMPLE_EMBEDDINGS
    assert oracle.count(g, q) == 4


def brute(off, adj, lab, qlab, qedges):
    n, k = len(lab), len(qlab)
    es = set()
    for v in range(n):
        for w in adj[off[v]:off[v + 1]]:
            es.add((v, int(w)))
    cnt = 0
    for m in itertools.permutations(range(n), k):
        if any(lab[m[u]] != qlab[u] for u in range(k)):
            continue
        if all((m[a], m[b]) in es for a, b in qedges):
            cnt += 1
    return cnt


def random_graph(rng, n, p, L):
    edges = [(a, b) for a in range(n) for b in range(a + 1, n) if rng.random() < p]
    off = [0]
    adj = []
    for v in range(n):
        nb = sorted([b for a, b in edges if a == v] + [a for a, b in edges if b == v])
        adj += nb
        off.append(len(adj))
    lab = [rng.randrange(L) for _ in range(n)]
    return off, adj, lab


def random_query(rng, k, L):
    perm = list(range(k))
    rng.shuffle(perm)
    es = set()
    for i in range(1, k):
        a, b = perm[i], perm[rng.randrange(i)]
        es.add((min(a, b), max(a, b)))
    for a in range(k):
        for b in range(a + 1, k):
            if rng.random() < 0.3:
                es.add((a, b))
    return [rng.randrange(L) for _ in range(k)], sorted(es)


def test_brute_force_tiny():
    rng = random.Random(11)
    for _ in range(150):
        n = rng.randrange(2, 8)
        off, adj, lab = random_graph(rng, n, rng.choice([0.3, 0.6, 0.9]), rng.choice([1, 2]))
        if not adj:
            continue
        g = HostGraph.from_arrays(off, adj, lab)
        k = rng.randrange(2, min(n, 4) + 1)
        qlab, qe = random_query(rng, k, 2)
        q = Query(qlab, [x for e in qe for x in e])
        want = brute(off, adj, lab, qlab, qe)
        assert oracle.count(g, q) == want
        plan = Plan(q)
        vm = oracle.nlc_filter(g, plan)
        _, cm = oracle.encode(g, plan, vm)
        assert oracle.count(g, q, candmask=cm) == want


@pytest.mark.parametrize("shape", ["tree", "sparse", "dense"])
def test_cluster_filter_is_sound(shape):
    """No embedding is lost: each one's vertices keep their candidate bits."""
    g = HostGraph.rmat(9, 8, 3, seed=4)
    for s in range(12):
        q = Query.generate(g, 4 + s % 5, shape, seed=s)
        plan = Plan(q)
        vm = oracle.nlc_filter(g, plan)
        _, cm = oracle.encode(g, plan, vm)
        if oracle.count_budget(g, q, 400000)[1] is None:
            continue
        cnt, emb = oracle.embeddings(g, q, max_rows=200000)
        if cnt > 200000:
            continue
        for u in range(q.k):
            assert np.all((cm[emb[:, u]] >> u) & 1), (shape, s, u)
            assert np.all((vm[emb[:, u]] >> u) & 1)
        assert oracle.count(g, q, candmask=cm) == cnt


def test_filter_prunes():
    """The bitmap filter is never weaker than the initial filter."""
    g = HostGraph.rmat(10, 8, 4, seed=1)
    for s in range(8):
        plan = Plan(Query.generate(g, 6, "sparse", seed=s))
        vm = oracle.nlc_filter(g, plan)
        _, cm = oracle.encode(g, plan, vm)
        assert np.all((cm & ~vm) == 0)


@pytest.mark.parametrize("kind", ["rmat", "rmat_uniform", "er", "er_zipf"])
def test_oracle_generators_equal_the_library(kind):
    """The oracle's own restatement of the seeded generators (used by the CPU
    baseline so that it loads nothing of the library) gives the library's
    graphs bit for bit."""
    from clustersm_gb300.native import HostGraph
    if kind.startswith("rmat"):
        z = kind == "rmat"
        a, b = oracle.Graph.rmat(13, 12, 7, 3, zipf=z), HostGraph.rmat(13, 12, 7, seed=3, zipf=z)
    else:
        z = kind == "er_zipf"
        a, b = oracle.Graph.er(2000, 9000, 5, 4, zipf=z), HostGraph.er(2000, 9000, 5, seed=4, zipf=z)
    assert np.array_equal(a.offsets(), b.offsets())
    assert np.array_equal(a.neighbors(), b.neighbors())
    assert np.array_equal(a.labels(), b.labels())
