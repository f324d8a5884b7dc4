"""The drop-in ClusterSM binary on a GPU: the reference's example prints
`num_res: 4` as its last line (main.cu:172), a workload query prints its
committed count, and --emit writes exactly the oracle's sorted embeddings, as
text and in the binary layout (cli_main.cpp header)."""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from clustersm_gb300.native import Query
from clustersm_gb300.workloads import load

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "clustersm_gb300" / "bin" / "ClusterSM"
EX = ROOT / "tests" / "golden" / "example"

pytestmark = pytest.mark.gpu


def run(*args):
    r = subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def last_count(r):
    line = r.stdout.strip().splitlines()[-1]
    assert line.startswith("num_res: ")
    return int(line.split()[1])


def read_bin(path):
    raw = Path(path).read_bytes()
    assert raw[:8] == b"SMGEMB01"
    k, _, count, rows = struct.unpack_from("<IIQQ", raw, 8)
    ids = np.frombuffer(raw, dtype="<u4", offset=32)
    assert ids.size == rows * k
    return count, ids.reshape(rows, k)


def test_example_prints_four():
    r = run("-q", EX / "example_q_01.in", "-d", EX / "example_g_01.in", "--gpu", "0")
    assert last_count(r) == 4


def test_example_emit_text_and_binary(tmp_path, example):
    g, q = example
    want_count, want = oracle.embeddings(g.sorted_copy(), q)
    txt, bnr = tmp_path / "e.txt", tmp_path / "e.bin"
    r = run("-q", EX / "example_q_01.in", "-d", EX / "example_g_01.in", "--emit", txt)
    assert last_count(r) == want_count == 4
    got = np.array([[int(x) for x in line.split()] for line in txt.read_text().splitlines()], dtype=np.uint32)
    assert np.array_equal(got, want)
    run("-q", EX / "example_q_01.in", "-d", EX / "example_g_01.in", "--emit", bnr, "--emit-format", "bin")
    count, rows = read_bin(bnr)
    assert count == 4 and np.array_equal(rows, want)


def test_workload_queries(tmp_path):
    """er1k queries through the binary: counts equal the committed ones, and
    the binary dump with a row cap keeps the exact count and the first rows
    of the oracle's sorted set."""
    wl = load("er1k")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    gpath = tmp_path / "g.in"
    host.write(gpath)
    for i in (0, 17, 95):
        qpath = tmp_path / f"q{i}.in"
        qs[i].write(qpath)
        assert last_count(run("-q", qpath, "-d", gpath)) == counts[i]
    q = qs[3]
    qpath = tmp_path / "q3.in"
    q.write(qpath)
    want_count, want = oracle.embeddings(host, Query.read(qpath), max_rows=1 << 20)
    out = tmp_path / "e.bin"
    run("-q", qpath, "-d", gpath, "--emit", out, "--emit-format", "bin")
    count, rows = read_bin(out)
    assert count == want_count == counts[3] and np.array_equal(rows, want)
    cap = max(1, want_count // 3)
    run("-q", qpath, "-d", gpath, "--emit", out, "--emit-format", "bin", "--max-emit", cap)
    count, rows = read_bin(out)
    assert count == want_count and rows.shape[0] == cap
    # capped rows are some of the embeddings, written sorted
    wanted = {tuple(r) for r in want.tolist()}
    assert all(tuple(r) in wanted for r in rows.tolist())
    assert rows.tolist() == sorted(rows.tolist())
