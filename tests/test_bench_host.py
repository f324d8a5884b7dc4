"""Host-side parts of bench.py that run without a GPU: the argument defaults
the timing rules depend on, and the CPU-baseline leg's record."""
import sys

import pytest

import bench
from clustersm_gb300.native import HostGraph, Query


def test_defaults_meet_timing_rules(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.workload == "rmat22" and a.impl == "gb300" and a.shape == ""
    # the serving leg's offered rates: 4-5-vertex requests, then the widest ones
    assert [float(r) for r in a.serve_rates.split(",")] == [100.0, 1000.0, 5000.0]
    assert [float(r) for r in a.serve_wide_rates.split(",")] == [25.0, 50.0]


def test_shape_choices(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py", "--shape", "dense", "--subset", "8"])
    a = bench.parse()
    assert a.shape == "dense" and a.subset == 8
    monkeypatch.setattr(sys, "argv", ["bench.py", "--shape", "cyclic"])
    with pytest.raises(SystemExit):
        bench.parse()


def test_cpu_baseline_record():
    g = HostGraph.er(300, 1200, 3, seed=2)
    qs = [Query.generate(g, 4, "sparse", seed=s) for s in range(6)]
    r = bench.cpu_baseline(g, qs, 0.5)
    assert r["kind"] == "port" and r["unit"] == "queries/s" and r["value"] > 0 and r["cores"] >= 1
    assert r["embeddings_per_s"] > 0
    one = r["single_core"]
    assert one["value"] > 0 and one["embeddings_per_s"] > 0 and "1 thread" in one["sample"]


def test_reference_arm_line():
    # the reference arm runs only on host cores: its JSON line is checked here
    import json
    import subprocess
    from pathlib import Path
    root = Path(bench.__file__).resolve().parent
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--workload", "er1k",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 1
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == "er1k"
    # the arm times the oracle alone: nothing of the library is loaded
    assert line.get("library_mapped", False) is False
