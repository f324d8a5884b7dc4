"""Seeded generators are deterministic on every host (integer-only RNG) and
produce what they promise.  The checksums in tests/golden/generator.json were
recorded on x86-64; the gpu-marked copy of the check runs on the aarch64 GPU
host."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from clustersm_gb300.native import HostGraph, Query

GOLD = json.loads((Path(__file__).parent / "golden" / "generator.json").read_text())


def digest(g):
    m = hashlib.sha256()
    m.update(g.offsets().tobytes())
    m.update(g.neighbors().tobytes())
    m.update(g.labels().tobytes())
    return m.hexdigest()[:32]


def check_checksums():
    assert digest(HostGraph.er(1000, 4000, 4, seed=1)) == GOLD["er_1000_4000_L4_s1"]
    g = HostGraph.rmat(12, 16, 8, seed=7)
    assert digest(g) == GOLD["rmat_12_16_L8_s7"]
    assert digest(HostGraph.rmat(16, 16, 16, seed=1, threads=2)) == GOLD["rmat_16_16_L16_s1"]
    for shape, want in GOLD["queries_rmat_12_16_L8_s7_k8_seed5"].items():
        q = Query.generate(g, 8, shape, seed=5)
        assert q.labels.tolist() == want["labels"]
        assert q.edges.tolist() == want["edges"]
        assert q.data_vertices.tolist() == want["data"]


def test_checksums():
    check_checksums()


@pytest.mark.gpu
def test_checksums_on_gpu_host():
    check_checksums()


def test_rmat_is_simple_and_symmetric():
    g = HostGraph.rmat(10, 8, 4, seed=2)
    off, adj = g.offsets().astype(np.int64), g.neighbors()
    for v in range(g.n):
        lst = adj[off[v]:off[v + 1]]
        assert np.all(np.diff(lst.astype(np.int64)) > 0)
        assert v not in lst
    # symmetric: rebuilding from the arrays checks it
    HostGraph.from_arrays(off, adj, g.labels())


@pytest.mark.parametrize("shape", ["tree", "sparse", "dense"])
def test_query_shapes(shape):
    g = HostGraph.rmat(12, 16, 8, seed=7)
    off, adj, lab = g.offsets().astype(np.int64), g.neighbors(), g.labels()
    for seed in range(10):
        k = 4 + seed % 5
        q = Query.generate(g, k, shape, seed=seed)
        e = q.edges.reshape(-1, 2)
        dv = q.data_vertices
        assert len(set(dv.tolist())) == k
        assert np.array_equal(q.labels, lab[dv])
        for a, b in e:  # the walk vertices are an embedding
            assert dv[b] in adj[off[dv[a]]:off[dv[a] + 1]]
        if shape == "tree":
            assert len(e) == k - 1
        elif shape == "sparse":
            assert len(e) == k + 1
        else:
            assert 2 * len(e) >= 3 * k


def _csr_from_pairs(n, pairs):
    """Reference CSR of an undirected edge list in numpy: both directions,
    self-loops dropped, duplicates removed, lists sorted."""
    import numpy as np
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    p = p[p[:, 0] != p[:, 1]]
    d = np.concatenate([p, p[:, ::-1]])
    key = np.unique(d[:, 0] * (1 << 32) + d[:, 1])
    src, dst = key >> 32, key & 0xFFFFFFFF
    off = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.uint64), dst.astype(np.uint32)


def test_rmat_pairs_make_the_rmat_graph():
    """smg_gen_rmat_pairs are smg_gen_rmat's draws: symmetrised and
    de-duplicated they give its CSR; smg_gen_labels gives its labels."""
    import numpy as np
    from clustersm_gb300.native import HostGraph
    g = HostGraph.rmat(12, 8, 6, seed=5)
    pairs = HostGraph.rmat_pairs(12, 8, 5)
    assert pairs.shape == ((1 << 12) * 8 // 2, 2)
    off, adj = _csr_from_pairs(g.n, pairs)
    assert np.array_equal(off, g.offsets()) and np.array_equal(adj, g.neighbors())
    assert np.array_equal(HostGraph.labels_for(g.n, 6, 5), g.labels())
