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

Each count must equal the committed oracle count and the library's count
(smg_match through the C ABI).  The tests skip when the reference's sources
are not available to build it.
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
    bad = []
    for r, qpath in list(zip(rows, qpaths))[::4]:
        p = subprocess.run([str(binary), "-q", str(qpath), "-d", str(gpath), "--gpu", "0"], capture_output=True,
                           text=True, timeout=300)
        assert p.returncode == 0, (r["index"], p.stderr[-2000:])
        ref = int(p.stdout.strip().splitlines()[-1].split()[1])
        if not (ref == counts[r["index"]] == lib[r["index"]]):
            bad.append(("binary", r["index"], ref, counts[r["index"]], lib[r["index"]]))
    for r, o in zip(rows, run_harness(harness, gpath, qpaths)):
        if not (o["num_res"] == counts[r["index"]] == lib[r["index"]]):
            bad.append(("ref_match", r["index"], o["num_res"], counts[r["index"]], lib[r["index"]]))
    assert not bad, f"reference / oracle / library disagree on {len(bad)} runs: {bad[:10]}"


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
    bad = []
    for r, o in zip(rows, res):
        i = r["index"]
        lib = native.match(ctx, dev, Plan(qs[i]))[0].count
        if not (o["num_res"] == counts[i] == lib):
            bad.append((i, o["num_res"], counts[i], lib))
    assert not bad, f"reference / oracle / library disagree on {len(bad)} queries: {bad[:10]}"
