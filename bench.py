"""Benchmark of the subgraph-matching hot path (filter + join) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload rmat22] [--impl reference]

One step = one batched pass (smg_match_batch: one filter pass and one
persistent join launch per memory chunk) over the workload's queries against
the device-resident data graph.  Prints one JSON line (rank 0).

  value      queries/s of the batched path, device-timed with CUDA events on
             the library's stream, data graph resident, L2 flushed between
             steps (a 256 MB write)
  e2e        queries/s through the C ABI from host query descriptions: plan
             creation, host->device staging, matching, counts read back
  plain      queries/s of the one-query-per-call path on a sample of queries
  roofline   the join kernel's algorithmic bytes / its event-timed duration
             against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (backtracking, all host cores) on a bounded
             sample of the same queries
  serving    p50 / p99 latency and sustained rate of the continuous-batching
             server (smg_server_*) on the 2^24-vertex R-MAT graph under seeded
             Poisson arrivals of its 4..5-vertex requests at 100, 1,000 and
             5,000 queries/s offered, and of its 4..7-vertex requests (up to
             10^9 embeddings each, workload rmat24_k4to7) at 25 and 50/s

  wide       the batched path on the 4..7-vertex queries of the same 2^22
             graph (workload rmat22_k4to7, the widest query sizes with
             decidable draws): device-timed queries/s and embeddings/s,
             every count checked
  c4         the large graph: R-MAT 2^25 vertices, avg degree 32, 64 Zipf
             labels, built on the device from its raw edge draws
             (smg_graph_build: radix sort, de-duplication, 64-bit offsets),
             its resident bytes, and 12-vertex sparse and dense walk queries:
             how many are decidable under a work limit, and the filter's time
             and roofline on them
  reference_binary  the reference's own filter and join (compiled from its
             sources for sm_103a, oracle/_ref/ref_match) against the plain
             path on the same 2^20-vertex R-MAT queries (those the reference
             can run in bounds, tests/golden/ref_screen_rmat20.json): per-query
             hot-path wall time, graph resident, counts compared

--impl reference times the reference's algorithm on the host cores instead:
the reference has no CPU implementation of its path, so the arm runs the
oracle port, the CPU restatement of the same semantics.

For N > 1 (torchrun) the queries are dealt round-robin to ranks: each rank
matches its own share against its own replica of the graph (no collective on
the data path); value = all ranks' queries / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="rmat22")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--subset", type=int, default=0, help="use only the first N queries (profiling runs)")
    ap.add_argument("--shape", default="", choices=["", "tree", "sparse", "dense"],
                    help="use only the queries of one shape class (profiling runs)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-rates", default="100,1000,5000")
    ap.add_argument("--serve-wide-rates", default="25,50",
                    help="offered rates of the 4..7-vertex serving requests (empty: skip them)")
    ap.add_argument("--no-wide", action="store_true", help="skip the 4..7-vertex query leg")
    ap.add_argument("--no-c4", action="store_true", help="skip the 2^25-vertex graph leg")
    ap.add_argument("--c4-scale", type=int, default=25)
    ap.add_argument("--no-reference-binary", action="store_true",
                    help="skip the leg that runs the reference's own GPU filter and join")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the library's per-shape-class autotuner (run on the workload before timing, untimed)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.out.flush()
        rows = []
        for line in Path(self.out.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(host, queries, seconds, meta_queries=()):
    """The oracle (backtracking, all cores) on a shape- and size-stratified
    sample of the queries until `seconds` pass."""
    import oracle
    if meta_queries:
        queries = [queries[i] for i in stratified(list(meta_queries), len(queries))]
    t0 = time.perf_counter()
    done, emb = 0, 0
    for q in queries:
        emb += oracle.count(host, q)
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    # the same queries again on one thread, for a third of the time
    t1 = time.perf_counter()
    done1, emb1 = 0, 0
    for q in queries[:done]:
        emb1 += oracle.count(host, q, threads=1)
        done1 += 1
        if time.perf_counter() - t1 > seconds / 3:
            break
    dt1 = time.perf_counter() - t1
    return {"value": done / dt, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{done} of {len(queries)} queries of the workload (one per (shape, k) stratum in turn), "
                      f"oracle_count with "
                      f"{os.cpu_count()} OpenMP threads, {dt:.1f} s", "embeddings_per_s": emb / dt,
            "single_core": {"value": done1 / dt1, "unit": "queries/s", "embeddings_per_s": emb1 / dt1,
                            "sample": f"first {done1} of those queries on 1 thread, {dt1:.1f} s"}}


def serving(ctx, dev, plans, want, rates, seconds=2.0, max_requests=2048):
    """Poisson arrivals into the continuous-batching server (smg_server_*).
    Per rate, requests cycle through the workload's queries with seeded
    exponential gaps; between arrivals the loop calls the non-blocking
    smg_server_step.  Latency = finish - submit as the server stamps them;
    sustained rate = requests / (last finish - first submit)."""
    import random
    from clustersm_gb300 import native
    from clustersm_gb300.native import Server
    out = []
    for rate in rates:
        rng = random.Random(f"serve-{rate}")
        n = max(64, min(max_requests, int(rate * seconds)))
        # request state for up to 1,024 requests: 160 GB (measured 1,749
        # sustained at 5,000/s offered, against 1,501 with 96 GB), or the
        # device's memory less the resident graph and 40 GB for the server's
        # queues, the filter and other allocations (the server frees the
        # context's batch scratch when it needs the room)
        import torch
        total = torch.cuda.mem_get_info()[1]
        budget = min(160 << 30, max(16 << 30, total - dev.stats().device_bytes - (40 << 30)))
        kq = max(p.view.k for p in plans)
        try:
            srv = Server(ctx, dev, max_inflight=1024, memory_budget_bytes=budget, max_query_vertices=kq)
        except native.SmgError:  # less room than expected: what is free now, less 24 GB
            budget = max(16 << 30, torch.cuda.mem_get_info()[0] - (24 << 30))
            srv = Server(ctx, dev, max_inflight=1024, memory_budget_bytes=budget, max_query_vertices=kq)
        tickets = []
        t_next = time.perf_counter()
        while len(tickets) < n:
            if time.perf_counter() >= t_next:
                j = len(tickets) % len(plans)
                tickets.append((srv.submit(plans[j]), j))
                t_next += rng.expovariate(rate)
            else:
                srv.step()
        srv.drain()
        ss = srv.stats()
        lat, wait, run, ok, first, last = [], [], [], 0, None, None
        for tk, j in tickets:
            r = srv.poll(tk)
            lat.append((r.finish_s - r.submit_s) * 1e3)
            wait.append((r.start_s - r.submit_s) * 1e3)
            run.append((r.finish_s - r.start_s) * 1e3)
            ok += int(r.status == 0 and (want[j] is None or int(r.count) == int(want[j])))
            first = r.submit_s if first is None else min(first, r.submit_s)
            last = r.finish_s if last is None else max(last, r.finish_s)
        srv.close()
        lat.sort()
        wait.sort()
        run.sort()
        out.append({"offered_qps": rate, "requests": n, "p50_ms": lat[n // 2], "p99_ms": lat[(99 * (n - 1)) // 100],
                    "sustained_qps": n / (last - first), "counts_ok": ok,
                    # submit -> admission, and admission -> result
                    "wait_p50_ms": wait[n // 2], "wait_p99_ms": wait[(99 * (n - 1)) // 100],
                    "run_p50_ms": run[n // 2], "run_p99_ms": run[(99 * (n - 1)) // 100],
                    "memory_budget_gb": round(budget / 2**30, 1),
                    "slices": ss.slices, "bells": ss.bells, "admitted_live": ss.admitted_live,
                    "retired_in_slice": ss.retired_in_slice, "carried_tasks": ss.carried_tasks,
                    "slice_s": ss.slice_s, "between_s": ss.between_s})
    return out


def c4_leg(ctx, peak, scale=25, avg_degree=32, labels=64, seed=1, draws=64, k=12):
    """The large-graph configuration: build, resident bytes, and k-vertex
    sparse and dense walk queries (decided under a count and a work limit;
    the filter's device time and algorithmic bytes over all of them)."""
    from clustersm_gb300 import native
    from clustersm_gb300.native import DeviceGraph, HostGraph, Plan, Query, SmgError
    t0 = time.perf_counter()
    pairs = HostGraph.rmat_pairs(scale, avg_degree, seed)
    lab = HostGraph.labels_for(1 << scale, labels, seed)
    t_gen = time.perf_counter() - t0
    t1 = time.perf_counter()
    dev = DeviceGraph.build(ctx, 1 << scale, pairs, lab)
    t_build = time.perf_counter() - t1
    del pairs
    st = dev.stats()
    off, adj = dev.download()

    class CsrView:  # the downloaded CSR as the query generator's input (no copy)
        csr = native.Csr(len(lab), len(adj) // 2, off.ctypes.data_as(native.u64p), adj.ctypes.data_as(native.u32p),
                         lab.ctypes.data_as(native.u32p))
    host = CsrView()
    out = {"graph": f"R-MAT(0.57,0.19,0.19,0.05) 2^{scale} vertices, avg degree {avg_degree}, {labels} Zipf labels",
           "vertices": st.num_vertices, "edges": st.num_edges, "max_degree": st.max_degree,
           "device_bytes": st.device_bytes, "generate_s": t_gen, "smg_graph_build_s": t_build, "queries": {}}
    for shape in ("sparse", "dense"):
        qs = []
        for a in range(draws):
            try:
                qs.append(Query.generate(host, k, shape, seed=(1 << 41) | (k << 24) | a))
            except SmgError:
                pass
        plans = [Plan(q) for q in qs]
        try:
            counts, bst = native.match_batch(ctx, dev, plans, profile=True, max_count=10**10, max_work=1 << 30)
            decided = [int(c) for c in counts.tolist() if c != 2**64 - 1]
            fgb = bst.filter_bytes / (bst.filter_ms / 1e3) / 1e9 if bst.filter_ms > 0 else 0.0
            out["queries"][shape] = {"k": k, "drawn": len(qs), "decided": len(decided),
                                     "counts_decided": sorted(decided)[:8], "filter_ms": bst.filter_ms,
                                     "filter_bytes": bst.filter_bytes, "filter_gbs": fgb, "filter_frac": fgb / peak,
                                     "join_ms": bst.join_ms}
        except SmgError as e:
            out["queries"][shape] = {"k": k, "drawn": len(qs), "error": str(e)[:200]}
    dev.free()
    return out


def random_sector_peak(device, gib=8, reads=1 << 29, reps=3):
    """Throughput ceiling of random 32-byte sector reads on this GPU: a seeded
    random gather of 4-byte words from a buffer far larger than L2 (each word
    costs one DRAM sector), timed with CUDA events; reported as sectors x 32 B
    per second.  The join's DRAM traffic is such sectors, so this, not the
    streaming copy peak, is the ceiling its traffic can approach."""
    import torch
    n = (gib << 30) // 4
    buf = torch.ones(n, dtype=torch.int32, device=device)
    g = torch.Generator(device=device)
    g.manual_seed(12345)
    idx = torch.randint(0, n, (reads,), device=device, dtype=torch.int64, generator=g)
    out = torch.empty(reads, dtype=torch.int32, device=device)
    torch.index_select(buf, 0, idx, out=out)  # warm-up
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        torch.index_select(buf, 0, idx, out=out)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del buf, idx, out
    torch.cuda.empty_cache()
    return {"gbs": reads * 32 / (best / 1e3) / 1e9, "unit": "GB/s",
            "how": f"torch.index_select of {reads} random int32 words from a {gib} GiB buffer, best of {reps}, "
                   "32 B per read (one DRAM sector)"}


def wide_leg(ctx, dev, stream, flush, steps=3, warmup=2):
    """Batched path on the rmat22_k4to7 queries against the resident 2^22
    graph (the same graph as rmat22): device time of `steps` passes after
    `warmup`, L2 flushed before each, every count checked."""
    import torch
    from clustersm_gb300 import native
    from clustersm_gb300.native import Plan
    from clustersm_gb300.workloads import load
    wl = load("rmat22_k4to7")
    if not (ROOT / wl.queries_file).exists():
        return {"unavailable": f"{wl.queries_file} not generated"}
    qs, want, meta = wl.queries()
    plans = [Plan(q) for q in qs]
    counts, _ = native.match_batch(ctx, dev, plans)
    bad = sum(1 for c, w in zip(counts.tolist(), want) if w is not None and int(c) != int(w))
    for _ in range(warmup):
        native.match_batch(ctx, dev, plans, profile=True)
    ms, jms, fms = [], 0.0, 0.0
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        counts, st = native.match_batch(ctx, dev, plans, profile=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        jms += st.join_ms
        fms += st.filter_ms
    tot = sum(ms) / 1e3
    ks = sorted({q["k"] for q in meta["queries"]})
    return {"workload": wl.name, "description": wl.description, "queries": len(plans), "k": ks,
            "queries_per_s": len(plans) * steps / tot, "embeddings_per_s": int(counts.sum()) * steps / tot,
            "embeddings_per_step": int(counts.sum()), "ms_per_step": 1e3 * tot / steps,
            "join_ms_per_step": jms / steps, "filter_ms_per_step": fms / steps,
            "counts_checked": sum(1 for w in want if w is not None), "count_mismatches": bad,
            "verified_by": meta.get("verified_by")}


def reference_binary_leg(ctx, repeats=3):
    """The reference's filter and join (oracle/_ref/ref_match) and the plain
    path (smg_match, one call per query) on the screened queries of the
    2^20-vertex workload.  Per query, the reference's time is the wall time of
    its per-query work (candidate buffers, clusterFilter, edge order, join,
    with their allocations, memsets and copies); the plain path's is the wall
    time of one smg_match call, best of `repeats`.  Both with the data graph
    already on the device."""
    import os as _os
    from clustersm_gb300 import native
    from clustersm_gb300.native import DeviceGraph, Plan
    from clustersm_gb300.workloads import load
    harness = ROOT / "oracle" / "_ref" / "ref_match"
    if not _os.access(harness, _os.X_OK):
        return {"unavailable": "oracle/_ref/ref_match not built (the reference's sources were not available)"}
    screen = json.loads((ROOT / "tests" / "golden" / "ref_screen_rmat20.json").read_text())
    rows = [r for r in screen["screen"] if r["run"]]
    wl = load("rmat20")
    host = wl.graph()
    qs, counts, _ = wl.queries()
    with tempfile.TemporaryDirectory() as td:
        gpath = Path(td) / "g.in"
        host.write(gpath)
        qpaths = []
        for r in rows:
            qpaths.append(str(Path(td) / f"q{r['index']}.in"))
            qs[r["index"]].write(qpaths[-1])
        p = subprocess.run([str(harness), str(ctx.device), str(gpath), *qpaths], capture_output=True, text=True,
                           timeout=1800)
    if p.returncode != 0:
        return {"unavailable": f"ref_match exited {p.returncode}: {p.stderr[-300:]}"}
    out = [json.loads(line) for line in p.stdout.splitlines() if line.startswith("{")]
    load_s = out[0].get("load_s")
    res = [o for o in out if "query" in o]
    dev = DeviceGraph(ctx, host)
    plans = [Plan(qs[r["index"]]) for r in rows]
    for pl in plans:  # warm-up
        native.match(ctx, dev, pl)
    plain_ms, lib_counts = [], []
    for pl in plans:
        best = None
        for _ in range(repeats):
            t = time.perf_counter()
            r, _ = native.match(ctx, dev, pl)
            dt = (time.perf_counter() - t) * 1e3
            best = dt if best is None else min(best, dt)
        plain_ms.append(best)
        lib_counts.append(int(r.count))
    dev.free()
    ref_ms = [o["ms"] for o in res]
    ref_counts = [int(o["num_res"]) for o in res]
    want = [counts[r["index"]] for r in rows]
    return {"workload": "rmat20", "queries": len(rows), "screened_from": screen["queries"],
            "reference_queries_per_s": len(rows) / (sum(ref_ms) / 1e3),
            "plain_queries_per_s": len(rows) / (sum(plain_ms) / 1e3),
            "plain_over_reference": sum(ref_ms) / sum(plain_ms),
            "reference_ms_median": statistics.median(ref_ms), "plain_ms_median": statistics.median(plain_ms),
            "reference_filter_ms_median": statistics.median([o["filter_ms"] for o in res]),
            "reference_load_s": load_s,
            "counts_equal": ref_counts == want == lib_counts,
            "count_mismatches": sum(1 for a, b, c in zip(ref_counts, want, lib_counts) if not a == b == c)}


def stratified(meta_queries, n_all):
    """Query indices in an order that takes one query of every (shape, k)
    stratum in turn, each stratum in workload order, so that any prefix of
    it is a shape- and size-stratified sample."""
    strata = {}
    for i in range(n_all):
        q = meta_queries[i] if i < len(meta_queries) else {}
        strata.setdefault((q.get("shape", ""), q.get("k", 0)), []).append(i)
    order, lists = [], [strata[k] for k in sorted(strata)]
    for r in range(max((len(x) for x in lists), default=0)):
        order += [x[r] for x in lists if r < len(x)]
    return order


def run_reference(args, wl, host, queries, rank, meta_queries):
    if rank != 0:
        return
    import oracle
    order = stratified(meta_queries, len(queries))
    # calibrate a bounded per-step sample (about 5 s of CPU work), taken in
    # stratified order
    t0 = time.perf_counter()
    sample = 0
    for i in order:
        oracle.count(host, queries[i])
        sample += 1
        if time.perf_counter() - t0 > 5.0:
            break
    sub = [queries[i] for i in order[:sample]]
    for _ in range(args.warmup):
        for q in sub[: max(1, sample // 4)]:
            oracle.count(host, q)
    times, embs = [], 0
    for _ in range(args.steps):
        t = time.perf_counter()
        for q in sub:
            embs += oracle.count(host, q)
        times.append(time.perf_counter() - t)
    tot = sum(times)
    value = args.steps * sample / tot
    strata = sorted({(meta_queries[i].get("shape"), meta_queries[i].get("k")) for i in order[:sample]})
    line = {"metric": "queries/s (batched subgraph matching, exact uint64 counts)", "value": value,
            "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic", "impl": "reference",
            "config": {"workload": wl.name, "description": wl.description, "queries_per_step": sample},
            "embeddings_per_s": embs / tot,
            "cpu_baseline": {"value": value, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{sample} queries per step, one per (shape, k) stratum in turn "
                                       f"({len(strata)} strata)"},
            "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    maps = Path("/proc/self/maps")
    if maps.exists():  # this arm runs the oracle alone: the library must not be mapped
        line["library_mapped"] = "libsmg.so" in maps.read_text()
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    from clustersm_gb300.workloads import load, shard
    wl = load(args.workload)
    if args.impl == "reference":
        # the oracle's own graph generator and query records: this arm maps
        # nothing of the library
        import oracle
        meta = json.loads((ROOT / wl.queries_file).read_text())
        mq = meta["queries"]
        if args.shape:
            mq = [q for q in mq if q.get("shape") == args.shape]
        if args.subset:
            mq = mq[: args.subset]
        host = (oracle.Graph.er(wl.n, wl.m, wl.labels, wl.seed, zipf=wl.zipf) if wl.kind == "er"
                else oracle.Graph.rmat(wl.scale, wl.avg_degree, wl.labels, wl.seed, zipf=wl.zipf))
        qs = [oracle.QueryArrays(q["labels"], q["edges"]) for q in mq]
        return run_reference(args, wl, host, qs, rank, mq)
    queries_all, expected, meta = wl.queries()
    if args.shape:
        keep = [i for i, q in enumerate(meta["queries"]) if q.get("shape") == args.shape]
        queries_all, expected = [queries_all[i] for i in keep], [expected[i] for i in keep]
        meta["queries"] = [meta["queries"][i] for i in keep]
    if args.subset:
        queries_all, expected = queries_all[: args.subset], expected[: args.subset]
        meta["queries"] = meta["queries"][: args.subset]
    mine = shard(len(queries_all), rank, world)
    queries = [queries_all[i] for i in mine]
    host = wl.graph()

    import torch
    from clustersm_gb300 import native
    from clustersm_gb300.native import Context, DeviceGraph, Plan

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    ctx = Context(local)
    dev = DeviceGraph(ctx, host)
    plans = [Plan(q) for q in queries]
    stream = torch.cuda.ExternalStream(ctx.stream_ptr)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    tuning = None
    if not args.no_tune:  # setup, outside the timed region
        t_tune = time.perf_counter()
        tuning = {"classes": [{"shape_class": e.shape_class, "root_chunk": e.root_chunk, "donate_min": e.donate_min,
                               "split_len": e.split_len, "hoist_cap": e.hoist_cap, "bfs_depth": e.bfs_depth,
                               "samples": e.samples,
                               "best_ms": e.best_ms, "default_ms": e.default_ms}
                              for e in native.autotune(ctx, dev, plans) if e.samples]}
        tuning["seconds"] = time.perf_counter() - t_tune
    # correctness against the committed counts before timing
    counts, _ = native.match_batch(ctx, dev, plans)
    want = [expected[i] for i in mine]
    mismatches = sum(1 for c, w in zip(counts.tolist(), want) if w is not None and int(c) != int(w))
    # the per-level byte model of a breadth-first table join over the same
    # partial matches (one untimed pass with the model counter on)
    _, mst = native.match_batch(ctx, dev, plans, model=True)
    model_bytes = mst.model_bytes
    # warm-up with the timed call: the first captures the batch's CUDA graph
    # (with its filter/join event nodes), the rest replay it
    for _ in range(args.warmup):
        native.match_batch(ctx, dev, plans, profile=True)

    step_ms, join_ms, filt_ms, jbytes, fbytes, launches = [], 0.0, 0.0, 0, 0, 0
    work = {"scanned": 0, "descents": 0, "probes": 0, "last_count_entries": 0, "donations": 0, "bfs_tasks": 0,
            "tasks": 0}
    h2d = d2h = 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            counts, st = native.match_batch(ctx, dev, plans, profile=True)
            e1.record(stream)
            barrier()
            step_ms.append(e0.elapsed_time(e1))
            join_ms += st.join_ms
            filt_ms += st.filter_ms
            jbytes += st.join_bytes
            fbytes += st.filter_bytes
            launches += st.kernel_launches
            for key in work:
                work[key] += getattr(st, key)
            h2d, d2h = st.h2d_bytes, st.d2h_bytes
    clocks = clk.summary()
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    nq_all = len(queries_all)
    value = nq_all * args.steps / (total_ms / 1e3)
    embeddings = int(counts.sum())

    # end to end through the C ABI from host query descriptions
    e2e_value = None
    if not args.no_e2e:
        e2e_t = []
        for _ in range(max(1, min(3, args.steps))):
            barrier()
            t = time.perf_counter()
            ps = Plan.batch(queries)  # smg_plan_create_batch: the plans on all host threads
            _, est = native.match_batch(ctx, dev, ps)
            e2e_t.append(time.perf_counter() - t)
            h2d, d2h = est.h2d_bytes, est.d2h_bytes
        e2e_value = nq_all / (max(e2e_t) if world > 1 else statistics.median(e2e_t))

    # plain path (one query per call) on a sample
    plain_qps = None
    if not args.no_plain:
        ns = min(args.plain_sample, len(plans))
        barrier()
        t = time.perf_counter()
        for p in plans[:ns]:
            native.match(ctx, dev, p)
        plain_qps = ns / (time.perf_counter() - t)

    wide = None
    if not args.no_wide and world == 1 and wl.name == "rmat22" and not args.shape and not args.subset:
        wide = wide_leg(ctx, dev, stream, flush)
    graph_device_bytes = dev.stats().device_bytes
    dev_freed = not args.shape and not args.subset
    if dev_freed:
        dev.free()  # the legs below build their own graphs (each takes up to 64 GB of hub bitmaps)

    peaks0 = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    c4 = None
    if not args.no_c4 and world == 1 and not args.shape and not args.subset:
        c4 = c4_leg(ctx, peaks0.get("hbm_gbs", 6800.0), scale=args.c4_scale)

    ref_bin = None
    if not args.no_reference_binary and world == 1:
        ref_bin = reference_binary_leg(ctx)

    serve = None
    if not args.no_serve and world == 1:
        rates = [float(r) for r in args.serve_rates.split(",") if r]
        swl = load("rmat24")
        if not args.shape and not args.subset and (ROOT / swl.queries_file).exists():
            # the serving configuration: R-MAT 2^24 resident, its own requests
            sq, swant, _ = swl.queries()
            sdev = DeviceGraph.build(ctx, 1 << swl.scale, native.HostGraph.rmat_pairs(swl.scale, swl.avg_degree,
                                                                                      swl.seed),
                                     native.HostGraph.labels_for(1 << swl.scale, swl.labels, swl.seed))
            splans = [Plan(q) for q in sq]
            # the batch path on the same requests (about 1,024 per batch), the
            # server's capacity to compare the sustained rates with
            bplans = splans * max(1, 1024 // len(splans))
            native.match_batch(ctx, sdev, bplans)
            t0 = time.perf_counter()
            bcounts, _ = native.match_batch(ctx, sdev, bplans)
            batch_s = time.perf_counter() - t0
            bwant = swant * max(1, 1024 // len(splans))
            serve = {"workload": swl.name, "description": swl.description,
                     "batch_qps": len(bplans) / batch_s,
                     "batch_counts_ok": sum(int(c) == int(w) for c, w in zip(bcounts, bwant) if w is not None),
                     "rates": serving(ctx, sdev, splans, swant, rates)}
            # the same graph's widest decidable requests (4..7 vertices, up to
            # 10^9 embeddings each), at rates about a quarter and half of
            # their batch rate
            wwl = load("rmat24_k4to7")
            wide_rates = [float(r) for r in args.serve_wide_rates.split(",") if r]
            if (ROOT / wwl.queries_file).exists() and wide_rates:
                wq, wwant, _ = wwl.queries()
                wplans = [Plan(q) for q in wq]
                native.match_batch(ctx, sdev, wplans)
                t0 = time.perf_counter()
                wcounts, _ = native.match_batch(ctx, sdev, wplans)
                wbatch_s = time.perf_counter() - t0
                serve["wide"] = {"workload": wwl.name, "description": wwl.description,
                                 "batch_qps": len(wplans) / wbatch_s,
                                 "batch_counts_ok": sum(int(c) == int(w) for c, w in zip(wcounts, wwant)),
                                 "rates": serving(ctx, sdev, wplans, wwant, wide_rates, seconds=4.0)}
            sdev.free()
        else:
            if dev_freed:
                dev = DeviceGraph(ctx, host)
            serve = {"workload": wl.name, "rates": serving(ctx, dev, plans, want, rates)}

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    rpeak = random_sector_peak(f"cuda:{local}") if world == 1 else None
    achieved = jbytes / (join_ms / 1e3) / 1e9 if join_ms > 0 else 0.0
    traffic = None  # k_join DRAM bytes per step from an ncu capture of this workload
    tf = ROOT / "profiles" / "traffic.txt"
    if tf.exists():
        for line in tf.read_text().splitlines():
            parts = line.split()
            if len(parts) == 3 and not line.startswith("#") and parts[0] == wl.name and parts[1] == "k_join":
                traffic = int(parts[2])
    if rank == 0:
        line = {
            "metric": "queries/s (batched subgraph matching, exact uint64 counts)",
            "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": wl.name, "description": wl.description, "queries": nq_all,
                       "graph_vertices": host.n, "graph_edges": host.m, "graph_device_bytes": graph_device_bytes,
                       "l2": "flushed (256 MB write) between steps",
                       "parallelism": f"replicas{world}" if world > 1 else "single",
                       **({"shape": args.shape} if args.shape else {})},
            "embeddings_per_s": embeddings * world * args.steps / (total_ms / 1e3),
            "embeddings_per_step": embeddings,
            "counts_checked": len(want), "count_mismatches": mismatches,
            "plain_queries_per_s": plain_qps, "batched_over_plain": value / plain_qps if plain_qps else None,
            "plain_sample": None if args.no_plain else min(args.plain_sample, len(plans)),
            "filter_ms_per_step": filt_ms / args.steps, "join_ms_per_step": join_ms / args.steps,
            "join_work_per_step": {key: val // args.steps for key, val in work.items()},
            "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "kernel": "k_join", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                         "traffic": traffic,
                         "algorithmic_bytes_per_step": jbytes / args.steps,
                         # DRAM traffic of the same kernel (one ncu capture) over its event-timed duration
                         "traffic_gbs": traffic / (join_ms / args.steps / 1e3) / 1e9 if traffic and join_ms else None,
                         "traffic_frac": traffic / (join_ms / args.steps / 1e3) / 1e9 / peak if traffic and join_ms
                         else None,
                         # the same DRAM traffic against the measured ceiling of random 32-byte sector reads
                         "random_sector_peak": rpeak,
                         "traffic_frac_of_random_peak": traffic / (join_ms / args.steps / 1e3) / 1e9 / rpeak["gbs"]
                         if traffic and join_ms and rpeak else None},
            # the same join time against the per-level byte model of a breadth-first
            # table join over the same partial matches (rows read and written,
            # anchors' whole lists, adjacency scans per back edge): what the
            # reference's algorithm would have to move for this work
            "roofline_model": {"bound": "hbm", "kernel": "k_join", "model_bytes_per_step": model_bytes,
                               "achieved": model_bytes / (join_ms / args.steps / 1e3) / 1e9 if join_ms else None,
                               "peak": peak, "unit": "GB/s",
                               "frac": model_bytes / (join_ms / args.steps / 1e3) / 1e9 / peak if join_ms else None},
            # the filter kernels of the same passes (k_nlc_filter, k_cluster_walk, k_walk_chunks,
            # k_collect): their algorithmic bytes over their event-timed duration
            "roofline_filter": {"bound": "hbm", "kernels": "k_nlc_filter+k_cluster_walk+k_walk_chunks+k_collect",
                                "achieved": fbytes / (filt_ms / 1e3) / 1e9 if filt_ms > 0 else 0.0,
                                "peak": peak, "unit": "GB/s",
                                "frac": (fbytes / (filt_ms / 1e3) / 1e9 / peak) if filt_ms > 0 else 0.0,
                                "algorithmic_bytes_per_step": fbytes / args.steps},
            "clocks": clocks,
            "tuning": tuning,
            "wide": wide,
            "c4": c4,
            "reference_binary": ref_bin,
            "serving": serve,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(host, queries_all, args.cpu_seconds, meta["queries"])
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
