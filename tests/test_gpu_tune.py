"""The autotuner picks a setting per shape class; counts do not depend on it."""
import pytest

from clustersm_gb300 import native
from clustersm_gb300.native import Context, DeviceGraph, Plan
from clustersm_gb300.workloads import load

pytestmark = pytest.mark.gpu


def test_autotune_keeps_counts():
    ctx = Context(0)  # own context: tuning is per context
    wl = load("er1k")
    qs, want, _ = wl.queries()
    dev = DeviceGraph(ctx, wl.graph())
    plans = [Plan(q) for q in qs]
    entries = native.autotune(ctx, dev, plans[:24])
    tuned = [e for e in entries if e.samples]
    assert tuned, "no class was tuned"
    for e in tuned:
        assert e.best_ms <= e.default_ms + 1e-6
        assert e.root_chunk in (1, 8, 64) and e.donate_min in (2, 33, 129)
    counts, _ = native.match_batch(ctx, dev, plans)
    assert counts.tolist() == want
    ctx.close()
