"""The reference's own ClusterSM on the GPU, compiled from its sources for
sm_103a by oracle/build_ref.sh, against the library and the oracle.

Only queries that tests/golden/ref_screen_<workload>.json lets through are
given to the reference: on the others its kernels would write out of bounds
or read uninitialised memory (tests/golden/make_ref_screen.py lists the
reasons with their file:line).

  er1k    the unmodified binary, one process per query (runClusterSM.sh:9-13),
          last line `num_res: N` (main.cu:172), on every fourth screened
          query; oracle/_ref/ref_match (the same filter and join over many
          queries after one read of the data graph) on all of them
  rmat20  ref_match over every screened query of the 2^20-vertex graph

The library's count (smg_match through the C ABI) must equal the committed
oracle count on every query.  The reference's count must equal it too, with
one known exception: encodeKernel and mergeKernel set a candidate's core bit
with a plain read-modify-write (filter.cu:633, 713) while other warps
atomicOr bits into the same word, so a bit can be lost.  A lost bit removes
a candidate, never adds one, so a reference count may fall short of the
oracle's and never exceed it, and the shortfall changes from run to run.  The
tests assert that bound on every run, exact equality on at least 95% of them,
and, when SMG_TEST_RECORD_DIR names a directory, write the divergences there
for the record.  They skip when the reference's sources are not available to
build it.
"""
import json
import os
import subprocess
from pathlib import Path

import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import DeviceGraph, Plan
from clustersm_gb300.workloads import load

ROOT = Path(__file__).resolve().parents[1]
REF = ROOT / "oracle" / "_ref"

pytestmark = pytest.mark.gpu


def ref_binaries():
    if not (os.access(REF / "ClusterSM", os.X_OK) and os.access(REF / "ref_match", os.X_OK)):
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), "gpu"], check=True, capture_output=True)
    if not (os.access(REF / "ClusterSM", os.X_OK) and os.access(REF / "ref_match", os.X_OK)):
        pytest.skip("the reference's sources are not available to build it")
    return REF / "ClusterSM", REF / "ref_match"


def screened(name):
    data = json.loads((ROOT / "tests" / "golden" / f"ref_screen_{name}.json").read_text())
    return [r for r in data["screen"] if r["run"]]


def judge(runs, name):
    """runs: (how, query index, reference, oracle, library).  Returns the
    failures; records the reference's shortfalls."""
    lib_bad = [r for r in runs if r[4] != r[3]]
    over = [r for r in runs if r[2] > r[3]]
    short = [r for r in runs if r[2] < r[3]]
    out = Path(os.environ.get("SMG_TEST_RECORD_DIR", "")) if os.environ.get("SMG_TEST_RECORD_DIR") else None
    if out is not None and out.is_dir():
        (out / f"reference_divergence_{name}.json").write_text(json.dumps(
            {"runs": len(runs), "short": [list(r) for r in short]}))
    fails = []
    if lib_bad:
        fails.append(f"library != oracle on {lib_bad[:10]}")
    if over:
        fails.append(f"reference above the oracle on {over[:10]}")
    if len(short) > 0.05 * len(runs):
        fails.append(f"reference short of the oracle on {len(short)} of {len(runs)} runs: {short[:10]}")
    return fails


def run_harness(harness, gpath, qpaths):
    p = subprocess.run([str(harness), "0", str(gpath), *map(str, qpaths)], capture_output=True, text=True,
                       timeout=1800)
    assert p.returncode == 0, p.stderr[-2000:]
    out = [json.loads(line) for line in p.stdout.splitlines() if line.startswith("{")]
    res = [o for o in out if "query" in o]
    assert len(res) == len(qpaths)
    return res


def test_reference_binary_er1k(tmp_path, ctx):
    binary, harness = ref_binaries()
    wl = load("er1k")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    gpath = tmp_path / "g.in"
    host.write(gpath)
    dev = DeviceGraph(ctx, host)
    rows = screened("er1k")
    assert len(rows) >= 90
    qpaths = []
    for r in rows:
        qpaths.append(tmp_path / f"q{r['index']}.in")
        qs[r["index"]].write(qpaths[-1])
    lib = {r["index"]: native.match(ctx, dev, Plan(qs[r["index"]]))[0].count for r in rows}
    runs = []
    for r, qpath in list(zip(rows, qpaths))[::4]:
        p = subprocess.run([str(binary), "-q", str(qpath), "-d", str(gpath), "--gpu", "0"], capture_output=True,
                           text=True, timeout=300)
        assert p.returncode == 0, (r["index"], p.stderr[-2000:])
        ref = int(p.stdout.strip().splitlines()[-1].split()[1])
        runs.append(("binary", r["index"], ref, counts[r["index"]], lib[r["index"]]))
    for r, o in zip(rows, run_harness(harness, gpath, qpaths)):
        runs.append(("ref_match", r["index"], o["num_res"], counts[r["index"]], lib[r["index"]]))
    fails = judge(runs, "er1k")
    assert not fails, "; ".join(fails)


def test_reference_filter_join_rmat20(tmp_path, ctx):
    _, harness = ref_binaries()
    wl = load("rmat20")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    gpath = tmp_path / "g.in"
    host.write(gpath)
    rows = screened("rmat20")
    assert rows
    qfiles = []
    for r in rows:
        qpath = tmp_path / f"q{r['index']}.in"
        qs[r["index"]].write(qpath)
        qfiles.append(str(qpath))
    res = run_harness(harness, gpath, qfiles)
    dev = DeviceGraph(ctx, host)
    runs = []
    for r, o in zip(rows, res):
        i = r["index"]
        runs.append(("ref_match", i, o["num_res"], counts[i], native.match(ctx, dev, Plan(qs[i]))[0].count))
    fails = judge(runs, "rmat20")
    assert not fails, "; ".join(fails)
