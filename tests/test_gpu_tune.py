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
        assert e.split_len in (2048, 8192, 32768) and e.hoist_cap in (256, 1024, 4096)
        assert e.bfs_depth in (0, 2, 3)
    counts, _ = native.match_batch(ctx, dev, plans)
    assert counts.tolist() == want
    ctx.close()


def test_autotune_rmat22_counts_and_settings():
    """Tuned on R-MAT 2^22 queries (long last-level lists, hoisted sets): the
    kept settings reproduce every committed count, batched and plain, and
    smg_set_tuning carries them to another context."""
    ctx = Context(0)
    wl = load("rmat22")
    qs, want, _ = wl.queries()
    dev = DeviceGraph(ctx, wl.graph())
    plans = [Plan(q) for q in qs[:192]]
    entries = native.autotune(ctx, dev, plans)
    tuned = [e for e in entries if e.samples]
    assert len(tuned) >= 3
    counts, _ = native.match_batch(ctx, dev, plans)
    assert [int(c) for c in counts] == want[:192]
    for p, w in list(zip(plans, want))[:16]:
        assert native.match(ctx, dev, p)[0].count == w
    other = Context(0)
    arr = (native.TuneEntry * len(entries))(*entries)
    native.check(native.lib.smg_set_tuning(other.handle, arr, len(entries)), "smg_set_tuning")
    dev2 = DeviceGraph(other, wl.graph())
    counts2, _ = native.match_batch(other, dev2, plans)
    assert [int(c) for c in counts2] == want[:192]
    other.close()
    ctx.close()
