"""smg_graph_build: the CSR sorted and de-duplicated on the device from an
edge list (the reference builds it on the host, readGraphToCPU2
io.cu:60-96).  The downloaded CSR must equal the host-built one exactly
(integer data: bit-exact), and the resident graph must give the same masks
and counts as an upload of the host CSR."""
import numpy as np
import pytest

import oracle
from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, HostGraph, Plan, Query, SmgError

pytestmark = pytest.mark.gpu


def csr_from_pairs(n, pairs):
    """Reference CSR in numpy: both directions, self-loops dropped,
    duplicates removed, lists sorted."""
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    p = p[p[:, 0] != p[:, 1]]
    d = np.concatenate([p, p[:, ::-1]])
    key = np.unique(d[:, 0] * (1 << 32) + d[:, 1])
    src, dst = key >> 32, key & 0xFFFFFFFF
    off = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.uint64), dst.astype(np.uint32)


@pytest.mark.parametrize("scale,deg", [(12, 8), (16, 16), (20, 16)])
def test_build_equals_generator_csr(ctx, scale, deg):
    host = HostGraph.rmat(scale, deg, 8, seed=11)
    pairs = HostGraph.rmat_pairs(scale, deg, 11)
    labels = HostGraph.labels_for(host.n, 8, 11)
    dev = DeviceGraph.build(ctx, host.n, pairs, labels)
    off, adj = dev.download()
    assert dev.num_edges == host.m
    assert np.array_equal(off, host.offsets()) and np.array_equal(adj, host.neighbors())
    st = dev.stats()
    assert st.num_vertices == host.n and st.num_edges == host.m and st.num_labels == 8


def test_build_gives_same_masks_and_counts(ctx):
    host = HostGraph.rmat(14, 16, 8, seed=7)
    built = DeviceGraph.build(ctx, host.n, HostGraph.rmat_pairs(14, 16, 7), HostGraph.labels_for(host.n, 8, 7))
    up = DeviceGraph(ctx, host)
    checked = 0
    for shape in ("tree", "sparse", "dense"):
        for s in range(3):
            q = Query.generate(host, 4 + s, shape, seed=900 + s)
            want, used = oracle.count_budget(host, q, 10**8)
            if used is None:
                continue
            p = Plan(q)
            assert np.array_equal(native.filter_inspect(ctx, built, p)[2], native.filter_inspect(ctx, up, p)[2])
            assert native.match(ctx, built, p)[0].count == native.match(ctx, up, p)[0].count == want
            checked += 1
    assert checked >= 4


def test_build_edge_cases(ctx):
    rng = np.random.default_rng(3)
    n = 500
    base = rng.integers(0, n, size=(3000, 2), dtype=np.int64)
    # repeats in both orientations, self-loops, and vertices 450.. left isolated
    base = base[(base < 450).all(axis=1)]
    pairs = np.concatenate([base, base[:700, ::-1], base[:300], np.stack([np.arange(20)] * 2, axis=1)])
    pairs = pairs[rng.permutation(len(pairs))]
    labels = rng.integers(0, 3, size=n).astype(np.uint32)
    dev = DeviceGraph.build(ctx, n, pairs, labels)
    off, adj = dev.download()
    want_off, want_adj = csr_from_pairs(n, pairs)
    assert np.array_equal(off, want_off) and np.array_equal(adj, want_adj)
    # the resident graph counts like the host CSR built from the same lists
    host = HostGraph.from_arrays(want_off, want_adj, labels)
    q = Query([0, 1, 2], [0, 1, 1, 2, 2, 0])
    assert native.match(ctx, dev, Plan(q))[0].count == oracle.count(host, q)
    # no edges at all
    empty = DeviceGraph.build(ctx, 10, np.zeros((0, 2), np.uint32), np.zeros(10, np.uint32))
    off, adj = empty.download()
    assert not off.any() and adj.size == 0
    # an endpoint outside the vertex range is rejected
    with pytest.raises(SmgError) as e:
        DeviceGraph.build(ctx, 10, np.array([[1, 2], [3, 10]], np.uint32), np.zeros(10, np.uint32))
    assert e.value.status == 1  # SMG_ERR_INVALID
