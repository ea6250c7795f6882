"""Benchmarks of the batched and served decomposition paths.

    python -m pgd_gb300.benchmarks batch [--graphs 4096] [--seed 1]
    python -m pgd_gb300.benchmarks serve [--requests 2000] [--rate 2000] [--seed 1]

batch: 4096 independent graphs, n uniform in [16, 2048]; half G(n, p) with p
uniform in [0.01, 0.5], half Barabasi-Albert with m uniform in {2..8}; all
from one seed.  The thresholds are autotuned on a sample, then the whole set
is decomposed in one call (one device build, one pass of the persistent
kernels) and compared with the plain loop: one graph per call
(pgd_graph_from_edges + pgd_decompose).  graphs/s for both.

serve: requests arrive as a Poisson process of `rate` per second; each
request's edge count is lognormal (median 5000, sigma 1.2, clipped at 50 M),
half RMAT (scale ceil(log2(m/16)), edge factor chosen to hit m) and half
G(n, p) with mean degree 16.  They go to the continuous-batching server;
reported: graphs/s, p50/p99 latency (submit to result), and the same
request list through the plain one-graph-per-call loop.

Every result is checked against the plain path's counts.  Prints one JSON
line per mode.
"""
import argparse
import concurrent.futures as cf
import json
import math
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import pgd_gb300 as pgd  # noqa: E402


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def batch_graphs(count, seed):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        n = int(rng.integers(16, 2049))
        if i % 2 == 0:
            specs.append(("er", n, float(rng.uniform(0.01, 0.5)), seed * 1000003 + i))
        else:
            specs.append(("ba", n, int(rng.integers(2, 9)), seed * 1000003 + i))

    def make(spec):
        kind, n, param, s = spec
        if kind == "er":
            return pgd.erdos_renyi(n, param, seed=s)
        return pgd.barabasi_albert(n, param, seed=s)

    with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        return list(ex.map(make, specs)), specs


def plain_loop(ctx, graphs):
    """One graph per call: upload, build, decompose."""
    out = []
    t0 = time.perf_counter()
    for s, d in graphs:
        g = ctx.graph_from_edges(s, d)
        out.append(g.decompose(micro=False).totals)
        g.destroy()
    return out, time.perf_counter() - t0


def run_batch(args):
    t0 = time.perf_counter()
    graphs, specs = batch_graphs(args.graphs, args.seed)
    pairs = sum(len(s) for s, _ in graphs)
    log("generated %d graphs, %d pairs in %.1fs" % (len(graphs), pairs, time.perf_counter() - t0))
    ctx = pgd.Context()
    # autotune on a stratified sample (every 16th graph)
    sample = [ctx.graph_from_edges(s, d) for s, d in graphs[:: max(1, len(graphs) // 256)]]
    a, c, dm, ms = ctx.autotune(sample, reps=1)
    for g in sample:
        g.destroy()
    log("autotuned thresholds: anchor_hub=%d cache_hub=%d dense_max=%d" % (a, c, dm))
    # warm-up, then timed runs of the whole set in one call
    ctx.decompose_pairs_batch(graphs[:64])
    times = []
    res = None
    for _ in range(args.reps):
        t0 = time.perf_counter()
        res = ctx.decompose_pairs_batch(graphs)
        times.append(time.perf_counter() - t0)
    best = min(times)
    # plain loop over an evenly spaced sample of the same graphs
    step = max(1, len(graphs) // max(1, args.plain_sample))
    idx = list(range(0, len(graphs), step))
    plain, plain_s = plain_loop(ctx, [graphs[i] for i in idx])
    mismatch = sum(int(not (p == res[i].totals).all()) for p, i in zip(plain, idx))
    k = len(idx)
    line = {
        "mode": "batch", "graphs": len(graphs), "pairs": pairs, "seconds": best, "graphs_per_s": len(graphs) / best,
        "kernel_ms": float(res[0].kernel_ms) if res else 0.0,
        "plain_graphs": k, "plain_seconds": plain_s, "plain_graphs_per_s": k / plain_s,
        "speedup_vs_plain": (len(graphs) / best) / (k / plain_s), "mismatches_vs_plain": mismatch,
        "thresholds": {"anchor_hub": a, "cache_hub": c, "dense_max": dm},
        "workload": "4096 graphs, n~U[16,2048], half G(n,p) p~U[0.01,0.5], half BA m~U{2..8}, seed %d" % args.seed,
    }
    print(json.dumps(line), flush=True)


def serve_requests(count, seed):
    rng = np.random.default_rng(seed)
    sizes = np.minimum(np.exp(rng.normal(math.log(5000.0), 1.2, count)), 50e6).astype(np.int64)
    sizes = np.maximum(sizes, 16)
    specs = []
    for i, m in enumerate(sizes):
        if i % 2 == 0:
            scale = max(4, int(math.ceil(math.log2(m / 16.0))))
            ef = max(1, int(round(m / float(1 << scale))))
            specs.append(("rmat", scale, ef, seed * 7919 + i))
        else:
            n = max(8, int(m // 8))
            specs.append(("er", n, min(1.0, 16.0 / n), seed * 7919 + i))

    def make(spec):
        kind, a, b, s = spec
        if kind == "rmat":
            return pgd.rmat(a, b, seed=s)
        return pgd.erdos_renyi(a, b, seed=s)

    with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        return list(ex.map(make, specs))


def run_serve(args):
    t0 = time.perf_counter()
    reqs = serve_requests(args.requests, args.seed)
    pairs = sum(len(s) for s, _ in reqs)
    log("generated %d requests, %d pairs in %.1fs" % (len(reqs), pairs, time.perf_counter() - t0))
    rng = np.random.default_rng(args.seed + 1)
    gaps = rng.exponential(1.0 / args.rate, len(reqs))
    # plain loop first (also the expected counts)
    ctx = pgd.Context()
    plain_loop(ctx, reqs[:16])
    expect, plain_s = plain_loop(ctx, reqs)
    ctx.close()
    log("plain loop: %.1f graphs/s" % (len(reqs) / plain_s))
    sv = pgd.Server(workers=args.workers)
    # warm-up
    for s, d in reqs[:8]:
        sv.wait(sv.submit(s, d), 60000)
    sv.close()
    sv = pgd.Server(workers=args.workers)
    tickets = []
    t_start = time.perf_counter()
    next_t = t_start
    for (s, d), gap in zip(reqs, gaps):
        next_t += gap
        while True:
            now = time.perf_counter()
            if now >= next_t:
                break
            time.sleep(min(0.0005, next_t - now))
        tickets.append(sv.submit(s, d))
    mismatch = 0
    for tk, e in zip(tickets, expect):
        st, r = sv.wait(tk, 600000)
        mismatch += int(st != 0 or not (r.totals == e).all())
    wall = time.perf_counter() - t_start
    stats = sv.stats()
    sv.close()
    line = {
        "mode": "serve", "requests": len(reqs), "pairs": pairs, "offered_rate": args.rate,
        "graphs_per_s": stats["graphs_per_s"], "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"],
        "mean_ms": stats["mean_ms"], "batches": stats["batches"], "wall_s": wall,
        "plain_graphs_per_s": len(reqs) / plain_s,
        "speedup_vs_plain": stats["graphs_per_s"] / (len(reqs) / plain_s), "mismatches_vs_plain": mismatch,
        "workers": args.workers,
        "workload": "Poisson arrivals; m ~ lognormal(median 5000, sigma 1.2, <= 50M); half RMAT, half G(n,p) "
                    "mean degree 16; seed %d" % args.seed,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["batch", "serve"])
    ap.add_argument("--graphs", type=int, default=4096)
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=4000.0)
    ap.add_argument("--workers", type=int, default=2)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--plain-sample", type=int, default=128)
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args()
    if args.mode == "batch":
        run_batch(args)
    else:
        run_serve(args)


if __name__ == "__main__":
    main()
