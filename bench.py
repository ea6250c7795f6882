#!/usr/bin/env python3
"""Benchmark: exact 3/4-node graphlet decomposition of an RMAT scale-20 graph.

Workload (the reference's headline shape): RMAT scale 20, edge factor 16,
(a, b, c, d) = (0.57, 0.19, 0.19, 0.05), seed 1, symmetrised, deduplicated,
self loops dropped; degeneracy (k-core) edge ordering; the 17 global counts
plus the 8 per-edge counts of every edge.  Metric: edges/s.

One step = sort_edges("kcore") + decomposition (global + per-edge) of the
HBM-resident graph, i.e. the span the reference times as "graphlet
decomposition time" (graphlet_driver.cpp:67-78).  L2 is flushed before every
step by a 256 MB device write.  `e2e` runs the same metric through the public
API from pinned host buffers: upload of the raw pairs, device CSR build,
ordering, k-core, decomposition and the copy of all per-edge rows back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With N > 1 (torchrun) the graph's ordered edge list is cut into N spans of
about equal estimated work (pgd_gb300/shard.py): every rank holds the whole
graph, decomposes its span, and the 15 partial sums are added with one NCCL
all-reduce before the totals are closed -- strong scaling (`--mode shard`,
the default).  `--mode replicas` instead decomposes an independent copy per
rank (no collective on the data path): weak scaling.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "edges/s full 4-node counts (bit-exact)"
UNIT = "edges/s"
RMAT = dict(a=0.57, b=0.19, c=0.19)

# ncu figures of one k_hub launch (the dominant kernel) on this workload, read
# from the committed summary: a `bench-figures:` line holding JSON with the
# DRAM traffic, the L2 request bytes, issue activity and the SHA-256 of the
# decompose.cu the capture ran.  A summary whose source hash differs from
# the current file is reported as stale.
PROFILE = os.path.join(ROOT, "profiles", "k_hub_rmat20_dram.md")
KERNEL_SRC = os.path.join(ROOT, "pgd_gb300", "csrc", "decompose.cu")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload_config(scale, order, n=None, m=None, world=1, mode="shard"):
    cfg = {
        "workload": "rmat%d_%s_global+micro" % (scale, order),
        "graph": "RMAT scale %d, edge factor 16, (a,b,c,d)=(0.57,0.19,0.19,0.05), seed 1, symmetrised, "
                 "deduplicated, self loops dropped" % scale,
        "ordering": "%s edge order (degeneracy)" % order if order == "kcore" else order,
        "counts": "17 global (uint64) + 8 per-edge columns for every edge",
        "step": "sort_edges + decomposition on the HBM-resident CSR",
        "l2": "flushed before every step (256 MB device write)",
    }
    if n is not None:
        cfg["n"] = int(n)
        cfg["m"] = int(m)
    if world > 1:
        cfg["parallelism"] = "%s%d" % ("shard" if mode == "shard" else "replicas", world)
    return cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = ""

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            self.out = ""
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(ev, eu, n, micro=True, anchor_hub=None, ids=None):
    """Bytes an edge-centric decomposition must stream: per edge both
    endpoint lists plus the 2-hop lists of the cheaper endpoint, 4 B per
    adjacency entry, plus 64 B of per-edge output (micro).  With anchor_hub,
    only the edges whose anchor (the endpoint of higher (degree, id)) has at
    least that degree: the units of the hub-anchored kernel.  With ids, only
    those edges (a rank's span).  Returns (bytes, edges counted)."""
    deg = np.bincount(ev, minlength=n) + np.bincount(eu, minlength=n)
    vol2 = np.bincount(ev, weights=deg[eu], minlength=n) + np.bincount(eu, weights=deg[ev], minlength=n)
    if ids is not None:
        ev, eu = ev[ids], eu[ids]
    sel = slice(None)
    if anchor_hub is not None:
        dv, du = deg[ev], deg[eu]
        dp = np.where((dv > du) | ((dv == du) & (ev > eu)), dv, du)
        sel = dp >= anchor_hub
    a, b = ev[sel], eu[sel]
    entries = (deg[a] + deg[b]).sum(dtype=np.float64) + np.minimum(vol2[a], vol2[b]).sum(dtype=np.float64)
    return 4.0 * entries + (64.0 * len(a) if micro else 0.0), int(len(a))


def profile_figures():
    """The bench-figures JSON of the committed k_hub summary, with whether it
    was taken on the current kernel source."""
    import hashlib

    out = {}
    if os.path.exists(PROFILE):
        for line in open(PROFILE):
            if line.startswith("bench-figures:"):
                out = json.loads(line.split(":", 1)[1])
    src = hashlib.sha256(open(KERNEL_SRC, "rb").read()).hexdigest()
    out["current_source"] = out.get("source_sha256") == src
    return out


def write_mtx(path, ev, eu):
    """A simple graph (each undirected edge once, 0-based ids) as the
    reference's benchmark file: an mtx file, 1-based, larger id first, with
    fixed-width right-aligned fields (the reader skips the leading blanks)."""
    ev = np.asarray(ev, np.int64)
    eu = np.asarray(eu, np.int64)
    lo = np.minimum(ev, eu) + 1
    hi = np.maximum(ev, eu) + 1
    n = int(hi.max())
    width = len(str(n))
    rows = np.full((len(lo), 2 * width + 2), ord(" "), np.uint8)
    for col, vals in ((0, hi), (width + 1, lo)):
        v = vals.copy()
        for k in range(width - 1, -1, -1):
            digit = (v % 10).astype(np.uint8) + ord("0")
            rows[:, col + k] = np.where((v > 0) | (k == width - 1), digit, ord(" "))
            v //= 10
    rows[:, -1] = ord("\n")
    with open(path, "wb") as f:
        f.write(b"%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, len(lo)))
        f.write(rows.tobytes())
    return os.path.getsize(path)


def golden_totals(scale, order):
    """The oracle's full-run totals of this workload, where committed."""
    p = os.path.join(GOLDEN, "rmat%d_%s.json" % (scale, order))
    if not os.path.exists(p):
        return None
    g = json.load(open(p))
    return g


def cpu_sample(src, dst, order, target_s, threads, stride=None, cache={}):
    """Edges/s of the reference's per-edge loop on the host cores over a
    bounded, evenly spaced sample of the ordered edges.  Uses the reference
    compiled from its sources where present (oracle/_ref), else the oracle
    port of it (same algorithm: mark e_v, scan e_u's 2-hop lists)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol

    if stride is not None and "runner" in cache:   # later steps: the same graph and sample size
        k, sec = cache["runner"](stride)
        return cache["kind"], k, sec, stride, cache["n"], cache["m"]
    og = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    n, m = og.n, og.m
    kind = "port"
    runner = None
    if ol.ref_available():
        try:
            off, adj = og.csr()
            rg = ol.RefGraph.from_csr(off, adj)
            kind = "reference"

            def runner(stride):
                return rg.time_sample(stride, order=order, workers=threads)
        except OSError:
            runner = None
    if runner is None:
        og.prepare(order=order)

        def runner(stride):
            return og.time_sample(stride, threads=threads)

    stride = max(1, m // 256)
    k, sec = runner(stride)
    # grow the sample toward target_s seconds
    while sec < target_s / 4 and stride > 1:
        stride = max(1, int(stride * max(sec, 1e-3) / target_s))
        k, sec = runner(stride)
    cache.update(runner=runner, kind=kind, n=n, m=m, graph=og)
    return kind, k, sec, stride, n, m


def run_reference_arm(args):
    """The reference's per-edge loop on the host cores (oracle/_ref where the
    reference was compiled, else the oracle's port of it).  The input comes
    from the oracle's own RMAT generator, so this arm never loads the
    product library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol

    threads = os.cpu_count() or 1
    src, dst = ol.rmat(args.scale, 16, seed=1, **RMAT)
    # each step a bounded sample, sized so that the whole run stays within a few minutes
    target = min(args.cpu_seconds, 150.0 / max(1, args.warmup + args.steps))
    per = []
    kind = None
    stride = None
    total_e, total_s = 0, 0.0
    for step in range(args.warmup + args.steps):
        kind, k, sec, stride, n, m = cpu_sample(src, dst, args.order, target, threads, stride)
        if step >= args.warmup:
            total_e += k
            total_s += sec
            per.append(sec)
    value = total_e / total_s
    sample = "every %d-th edge of the %s order (%d of %d edges) per step" % (stride, args.order, k, m)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded RMAT generator)",
        "config": workload_config(args.scale, args.order, n, m, int(os.environ.get("WORLD_SIZE", "1")), args.mode),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="shard", choices=["shard", "replicas"],
                    help="N > 1: one graph cut into spans (strong scaling) or a copy per rank (weak)")
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--order", default="kcore")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--batched-graphs", type=int, default=4096)
    ap.add_argument("--served-requests", type=int, default=2000)
    ap.add_argument("--served-rates", default="4000,1000000")
    args = ap.parse_args()

    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch

    import pgd_gb300 as pgd

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- input (host) and graph (device) ----------------------------------
    t0 = time.time()
    src, dst = pgd.rmat(args.scale, 16, seed=1, **RMAT)
    log("rank %d: generated %d pairs in %.1fs" % (rank, len(src), time.time() - t0))
    stream = torch.cuda.Stream(device=dev)
    ctx = pgd.Context(device=local, stream=stream.cuda_stream)
    t0 = time.time()
    g = ctx.graph_from_edges(src, dst, dedup=True)
    g.preprocess("deg")
    K = g.compute_cores()
    info = g.info()
    n, m = info.n, info.m
    log("rank %d: graph n=%d m=%d dmax=%d K=%d built in %.2fs" % (rank, n, m, info.max_degree, K, time.time() - t0))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sharded = world > 1 and args.mode == "shard"
    span_ids = None
    if sharded:
        from pgd_gb300 import shard

        g.sort_edges(args.order)
        sev, seu, sids = g.edges()
        sdeg = np.bincount(sev, minlength=n) + np.bincount(seu, minlength=n)
        lo, hi = shard.edge_spans(shard.edge_cost(sev, seu, sdeg, sids, ctx.thresholds()[1]), world)[rank]
        span_ids = sids[lo:hi].astype(np.int64)
        log("rank %d: span [%d, %d) of %d ordered edges" % (rank, lo, hi, m))

    def decompose_span(gr):
        """This rank's span (natural order keeps E_ordered's), then the one
        exchange: the wrapping sum of the 15 partials; totals closed here."""
        gr.sort_edges_sample(span_ids, "natural", s2l=True)
        r = gr.decompose(micro=True)
        r.sums = shard.reduce_sums(r.sums)
        r.totals = pgd.close_counts(r.sums, n, m)
        return r

    def step():
        if sharded:
            return decompose_span(g)
        g.sort_edges(args.order)
        return g.decompose(micro=True)

    ref_totals = None
    for w in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        r = step()
        log("rank %d: warmup %d kernel %.1f ms" % (rank, w, r.kernel_ms))
        if ref_totals is None:
            ref_totals = r.totals.copy()
            gold = golden_totals(args.scale, args.order)
            if gold is not None:
                got = {k_: int(v) for k_, v in zip(pgd.TOTAL_NAMES, r.totals)}
                if got != gold["totals"] or [int(x) for x in r.sums] != gold["sums"] or (n, m) != (gold["n"], gold["m"]):
                    raise SystemExit("the decomposition differs from the oracle's full run "
                                     "(tests/golden/rmat%d_%s.json): %s" % (args.scale, args.order, got))
                log("rank %d: totals and raw sums equal the oracle's full run" % rank)
        assert (r.totals == ref_totals).all(), "decomposition not repeatable"

    # ---- timed region ------------------------------------------------------
    clocks = ClockSampler(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kernel_ms, hub_ms = [], []
    launches0 = ctx.kernel_launches
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        r = step()
        kernel_ms.append(r.kernel_ms)
        hub_ms.append(r.hub_ms)
        if ref_totals is not None:
            assert (r.totals == ref_totals).all(), "decomposition not repeatable"
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = ctx.kernel_launches - launches0
    window_ms = max_over_ranks(ev0.elapsed_time(ev1))
    units = m if sharded else world * m     # edges decomposed by all ranks together
    value = units * args.steps / (window_ms / 1000.0)
    ms_per_step = window_ms / args.steps
    log("rank %d: %.1f ms/step, decomposition kernels %.1f ms (k_hub %.1f ms), %.3g edges/s"
        % (rank, ms_per_step, np.mean(kernel_ms), np.mean(hub_ms), value))

    # ---- roofline of the dominant kernel (k_hub) ----------------------------
    # achieved = the per-edge algorithmic bytes of the edges k_hub decomposes
    # (hub-anchored edges) over k_hub's own mean duration (CUDA events on the
    # launching stream); traffic, L2 bytes and issue activity come from the
    # committed ncu summary of the same launch on this workload.
    ev, eu, _ = g.edges(with_order=False)
    anchor_hub = ctx.thresholds()[0]
    b_alg, hub_units = algorithmic_bytes(ev, eu, n, micro=True, anchor_hub=anchor_hub, ids=span_ids)
    hub_s = float(np.mean(hub_ms)) / 1000.0
    peak, peak_src = peaks()
    achieved = b_alg / hub_s / 1e9
    prof = profile_figures() if (args.scale, args.order) == (20, "kcore") else {}
    traffic = prof.get("traffic_bytes")
    l2_bytes = prof.get("l2_bytes")
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "traffic": traffic, "kernel": "k_hub", "kernel_ms": 1000.0 * hub_s, "units": hub_units,
        "unit_name": "hub-anchored edges (anchor degree >= %d)" % anchor_hub,
        "algorithmic_bytes": b_alg,
        "dram_frac": (traffic / hub_s / 1e9 / peak) if traffic else None,
        "model_bytes": l2_bytes,
        "frac_model": (l2_bytes / hub_s / 1e9 / peak) if l2_bytes else None,
        "issue_active": prof.get("issue_active"),
        "profile_on_current_source": prof.get("current_source"),
        "decomposition_kernels_ms": float(np.mean(kernel_ms)),
        "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else "fallback 6.8 TB/s",
    }

    # ---- end to end through the public API --------------------------------
    e2e = None
    if not args.no_e2e:
        h_src = torch.from_numpy(src).pin_memory().numpy()
        h_dst = torch.from_numpy(dst).pin_memory().numpy()
        h_cols = torch.empty((m, pgd.NMICRO), dtype=torch.int64).pin_memory().numpy().view(np.uint64)
        h_s1 = torch.empty(m, dtype=torch.int64).pin_memory().numpy()
        h_d1 = torch.empty(m, dtype=torch.int64).pin_memory().numpy()

        def e2e_step():
            ge = ctx.graph_from_edges(h_src, h_dst, dedup=True)
            ge.preprocess("deg")
            ge.compute_cores()
            ge.sort_edges(args.order)
            res = decompose_span(ge) if sharded else ge.decompose(micro=True)
            lib = pgd.lib()
            st = lib.pgd_get_micro(ge.h, pgd._ptr(h_s1), pgd._ptr(h_d1), pgd._ptr(h_cols))
            assert st == 0
            ge.destroy()
            return res

        e2e_step()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.e2e_steps):
            res = e2e_step()
            assert (res.totals == ref_totals).all()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        e2e_ms = max_over_ranks(e0.elapsed_time(e1)) / args.e2e_steps
        e2e = {"value": units / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
               "h2d_bytes_per_step": int(src.nbytes + dst.nbytes),
               "d2h_bytes_per_step": int(m * (pgd.NMICRO * 8 + 12) + (pgd.NTOTALS + pgd.NSUMS) * 8)}
        log("rank %d: e2e %.1f ms/step" % (rank, e2e_ms))

    # ---- end to end from the graph file (device ingest) --------------------
    # the reference's benchmark input, an mtx file of the same graph, read by
    # pgd_graph_from_file (one copy of the file's bytes, parsing on the device)
    e2e_file = None
    if not args.no_e2e and world == 1:
        import tempfile

        tdir = tempfile.mkdtemp(prefix="pgd_bench_")
        path = os.path.join(tdir, "rmat%d.mtx" % args.scale)
        fbytes = write_mtx(path, ev, eu)

        def file_step():
            gf = ctx.graph_from_file(path)
            gf.preprocess("deg")
            gf.compute_cores()
            gf.sort_edges(args.order)
            res = gf.decompose(micro=True)
            st = pgd.lib().pgd_get_micro(gf.h, pgd._ptr(h_s1), pgd._ptr(h_d1), pgd._ptr(h_cols))
            assert st == 0
            gf.destroy()
            return res

        file_step()
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.e2e_steps):
            res = file_step()
            assert (res.totals == ref_totals).all()
        f1.record(stream)
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1) / args.e2e_steps
        os.remove(path)
        os.rmdir(tdir)
        e2e_file = {"value": m / (fms / 1000.0), "unit": UNIT, "ms_per_step": fms, "file_bytes": int(fbytes),
                    "h2d_bytes_per_step": int(fbytes),
                    "d2h_bytes_per_step": int(m * (pgd.NMICRO * 8 + 16) + (pgd.NTOTALS + pgd.NSUMS) * 8),
                    "what": "mtx file -> counts: file read, one copy of its bytes, device parsing with the reader's "
                            "rules, CSR build, neighbour order, k-core, sort, decomposition, per-edge rows to host"}
        log("rank %d: e2e from the %.0f MB mtx file %.1f ms/step" % (rank, fbytes / 1e6, fms))

    # ---- CPU baseline (rank 0, N = 1) ---------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        kind, k, sec, stride, _, _ = cpu_sample(src, dst, args.order, args.cpu_seconds, threads)
        cpu = {"value": k / sec, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": "every %d-th edge of the %s order: %d of %d edges, global counts, %.1f s" %
                         (stride, args.order, k, m, sec)}
        log("cpu baseline (%s, %d threads): %.3g edges/s" % (kind, threads, k / sec))

    # ---- the second half of the metric: batched and served graphs/s -------
    # (rank 0 at N = 1; wall-clock throughput through the public API, each
    # result checked against the plain one-graph-per-call path and a
    # stratified sample against the oracle, outside the timed regions)
    batched = served = None
    if rank == 0 and world == 1:
        from benchmarks import suite

        if not args.no_batched:
            b = suite.run_batch(argparse.Namespace(graphs=args.batched_graphs, seed=1, reps=2, plain_sample=256),
                                emit=False)
            batched = {k_: b[k_] for k_ in (
                "graphs", "pairs", "seconds", "graphs_per_s", "plain_graphs", "plain_graphs_per_s",
                "speedup_vs_single_graph_api", "speedup_vs_batch_of_one", "mismatches_vs_plain", "oracle_checked",
                "oracle_mismatches", "thresholds", "workload")}
            batched["unit"] = "graphs/s"
            log("batched: %.0f graphs/s, %.1fx the single-graph API, %.1fx the batch kernels one graph per call"
                % (b["graphs_per_s"], b["speedup_vs_single_graph_api"], b["speedup_vs_batch_of_one"]))
        if not args.no_served:
            lines = suite.run_serve(argparse.Namespace(requests=args.served_requests, seed=1, rates=args.served_rates,
                                                       rate=4000.0, workers=2), emit=False)
            served = {"unit": "graphs/s", "workload": lines[0]["workload"], "requests": lines[0]["requests"],
                      "plain_graphs_per_s": lines[0]["plain_graphs_per_s"],
                      "oracle_checked": lines[0]["oracle_checked"], "oracle_mismatches": lines[0]["oracle_mismatches"],
                      "rates": [{k_: ln[k_] for k_ in (
                          "offered_rate", "graphs_per_s", "p50_ms", "p99_ms", "queue_p50_ms", "queue_p99_ms",
                          "service_p50_ms", "service_p99_ms", "speedup_vs_best_plain", "mismatches_vs_plain",
                          "batches", "skipped_ahead")} for ln in lines]}
            for ln in lines:
                log("served at %.0f/s offered: %.0f graphs/s, p50 %.2f ms, p99 %.2f ms, %.1fx the plain loop"
                    % (ln["offered_rate"], ln["graphs_per_s"], ln["p50_ms"], ln["p99_ms"], ln["speedup_vs_best_plain"]))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "strong" if sharded else "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded RMAT generator)",
            "config": workload_config(args.scale, args.order, n, m, world, args.mode), "roofline": roofline,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(launches),
            "totals": {k_: int(v) for k_, v in zip(pgd.TOTAL_NAMES, ref_totals)},
            "e2e_file": e2e_file, "batched": batched, "served": served,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
