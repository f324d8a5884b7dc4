"""The .in reader on files large enough to be parsed in pieces and scattered
in parallel: lists must come out exactly as the sequential fill of
io.cu:86-93 leaves them (file order), and errors anywhere in the file must
still be reported."""
import numpy as np
import pytest

from clustersm_gb300.native import HostGraph, SmgError


def _random_graph(n, m, labels, seed):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, n, size=3 * m, dtype=np.int64)
    b = rng.integers(0, n, size=3 * m, dtype=np.int64)
    keep = a != b
    a, b = a[keep], b[keep]
    key = np.minimum(a, b) * n + np.maximum(a, b)
    _, first = np.unique(key, return_index=True)
    first = np.sort(first)[:m]          # distinct undirected edges, random file order
    a, b = a[first], b[first]
    lab = rng.integers(0, labels, size=n, dtype=np.int64)
    return a, b, lab


def _text(n, a, b, lab, v_lines=None):
    deg = np.bincount(np.concatenate([a, b]), minlength=n)
    vs = v_lines if v_lines is not None else [f"v {i} {lab[i]} {deg[i]}" for i in range(n)]
    es = [f"e {x} {y}" for x, y in zip(a.tolist(), b.tolist())]
    return "\n".join([f"t {n} {len(a)}", *vs, *es]) + "\n"


def _file_order_csr(n, a, b):
    src = np.empty(2 * len(a), dtype=np.int64)
    dst = np.empty_like(src)
    src[0::2], src[1::2] = a, b
    dst[0::2], dst[1::2] = b, a
    order = np.argsort(src, kind="stable")
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(src, minlength=n), out=off[1:])
    return off, dst[order]


@pytest.fixture(scope="module")
def big(tmp_path_factory):
    n, m = 60_000, 700_000                # 1.4M adjacency entries, ~10 MB of text
    a, b, lab = _random_graph(n, m, 7, seed=11)
    return n, a, b, lab, tmp_path_factory.mktemp("io")


def test_parallel_read_keeps_file_order(big):
    n, a, b, lab, d = big
    p = d / "g.in"
    p.write_text(_text(n, a, b, lab))
    g = HostGraph.read(p)
    off, adj = _file_order_csr(n, a, b)
    assert (g.n, g.m) == (n, len(a))
    assert np.array_equal(g.offsets(), off)
    assert np.array_equal(g.neighbors(), adj)
    assert np.array_equal(g.labels(), lab)


def test_parallel_read_crlf_and_vertex_order(big):
    n, a, b, lab, d = big
    deg = np.bincount(np.concatenate([a, b]), minlength=n)
    perm = np.random.default_rng(5).permutation(n)
    vs = [f"v {i} {lab[i]} {deg[i]}" for i in perm.tolist()]
    p = d / "g_crlf.in"
    p.write_bytes(_text(n, a, b, lab, vs).replace("\n", "\r\n").encode())
    g = HostGraph.read(p)
    off, adj = _file_order_csr(n, a, b)
    assert np.array_equal(g.offsets(), off) and np.array_equal(g.neighbors(), adj)
    assert np.array_equal(g.labels(), lab)


def _read_fails(path):
    with pytest.raises(SmgError) as e:
        HostGraph.read(path)
    return e.value.status


def test_parallel_read_errors_late_in_file(big):
    n, a, b, lab, d = big
    text = _text(n, a, b, lab)
    lines = text.splitlines()
    # each case breaks one line near the end of the file, far from the first piece
    cases = {
        "range": (len(lines) - 3, f"e 0 {n}"),
        "self": (len(lines) - 3, f"e 7 7"),
        "type": (len(lines) - 3, "x 1 2"),
        "short": (len(lines) - 3, "e 1"),
    }
    for name, (i, repl) in cases.items():
        bad = lines.copy()
        bad[i] = repl
        p = d / f"bad_{name}.in"
        p.write_text("\n".join(bad) + "\n")
        assert _read_fails(p) == 3, name
    # a vertex declared twice: once early, once in the last piece
    bad = lines.copy()
    bad.insert(len(bad) - 2, lines[5])
    p = d / "bad_twice.in"
    p.write_text("\n".join(bad) + "\n")
    assert _read_fails(p) == 3
    # a repeated edge (the list check runs on a sorted copy)
    bad = lines.copy()
    x, y = a[-1], b[-1]
    bad.append(f"e {y} {x}")
    bad[0] = f"t {n} {len(a) + 1}"
    p = d / "bad_repeat.in"
    p.write_text("\n".join(bad) + "\n")
    assert _read_fails(p) == 3


def test_record_split_across_lines_reads_as_one(tmp_path):
    # tokens, not lines, make records (io.cu:60-96 reads with >>)
    p = tmp_path / "split.in"
    p.write_text("t 3 2\nv 0 0 1\nv 1 0\n2\nv 2 1 1\ne 0\n1\ne 1 2\n")
    g = HostGraph.read(p)
    assert g.offsets().tolist() == [0, 1, 3, 4]
    assert g.neighbors().tolist() == [1, 0, 2, 1]


def test_split_records_and_no_final_newline_in_large_file(big):
    # every 'e' record spans two lines, so pieces may only start at lines
    # that begin with a letter; the file also ends without a newline
    n, a, b, lab, d = big
    deg = np.bincount(np.concatenate([a, b]), minlength=n)
    vs = [f"v {i} {lab[i]}\n{deg[i]}" for i in range(n)]
    es = [f"e {x}\n{y}" for x, y in zip(a.tolist(), b.tolist())]
    p = d / "split_big.in"
    p.write_text("\n".join([f"t {n} {len(a)}", *vs, *es]))
    g = HostGraph.read(p)
    off, adj = _file_order_csr(n, a, b)
    assert np.array_equal(g.offsets(), off) and np.array_equal(g.neighbors(), adj)
    assert np.array_equal(g.labels(), lab)
