"""Benchmarks of the batched, served, large and small configurations.

    python -m benchmarks.suite batch [--graphs 4096] [--seed 1]
    python -m benchmarks.suite serve [--requests 2000] [--rate 4000 | --rates 1000,4000,...] [--seed 1]
    python -m benchmarks.suite large [--workloads rmat24,rgg24] [--samples 1000]
    python -m benchmarks.suite profile [--scale 18] [--order kcore] [--reps 1]
    python -m benchmarks.suite small [--reps 50]
    python -m benchmarks.suite profile_batch [--graphs 256]
    python -m benchmarks.suite shard [--scale 20]

batch: 4096 independent graphs, n uniform in [16, 2048]; half G(n, p) with p
uniform in [0.01, 0.5], half Barabasi-Albert with m uniform in {2..8}; all
from one seed.  The thresholds are autotuned on a sample, then the whole set
is decomposed in one call (one device build, one pass of the persistent
kernels) and compared with plain loops over a stratified sample, one graph
per call: the single-graph API (pgd_graph_from_edges + pgd_decompose) with
the default and with the tuned thresholds, and the batch kernels on a batch
of one.  graphs/s for all; the speed-up is against the fastest plain loop.

serve: requests arrive as a Poisson process of `rate` per second; each
request's edge count is lognormal (median 5000, sigma 1.2, clipped at 50 M),
half RMAT (scale ceil(log2(m/16)), edge factor chosen to hit m) and half
G(n, p) with mean degree 16.  They go to the continuous-batching server;
reported per offered rate: graphs/s, p50/p99 latency (submit to result),
and the same request list through the plain one-graph-per-call loops (the
single-graph API, and the batch kernels on a batch of one).

large: RMAT scale 24 (edge factor 16, (a,b,c,d) = (0.57,0.19,0.19,0.05),
seed 1) and the 3-D random geometric graph with n = 2^24 in the unit cube,
radius (3*24 / (4 pi n))^(1/3) (seed 1), each with degeneracy order and
per-edge counts.  Timed: sort_edges + decomposition of the resident graph
(the reference's "graphlet decomposition time"); the CSR build is reported
separately.  Checked: the per-edge columns against the global sums, the
closing identities, and a seeded random sample of rows plus the heaviest rows
against the oracle's marking procedure on those edges.

small: G(n=250, p=0.9), seed 1 (the small dense configuration), degree
order, per-edge counts; decomposition timed over `reps` runs on the resident
graph, and end to end (host pairs in, host rows out) likewise.  edges/s.

profile: one RMAT graph of the given scale, k-core order, decomposed `reps`
times with per-edge counts; prints the kernel time of each run.  This is the
command the ncu captures of the decomposition kernels are taken on.

Every batch/serve result is checked against the plain path's counts, and a
stratified sample of the graphs (spread over sizes, up to 20,000 edges each)
against the oracle (tests/oracle_lib.py, outside every timed region).
Prints one JSON line per mode (per workload for `large`).
"""
import argparse
import concurrent.futures as cf
import json
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import pgd_gb300 as pgd  # noqa: E402


def oracle_check(graphs, results, cap_edges=20000, count=32):
    """Compare results[i].totals with the oracle on a sample of the graphs of
    at most cap_edges pairs, spread evenly over their sizes.  Returns
    (graphs checked, mismatches)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol

    small = [i for i, (s, _) in enumerate(graphs) if len(s) <= cap_edges]
    small.sort(key=lambda i: len(graphs[i][0]))
    pick = [small[int(j * (len(small) - 1) / max(1, count - 1))] for j in range(min(count, len(small)))]
    pick = sorted(set(pick))
    bad = 0
    for i in pick:
        s, d = graphs[i]
        want = ol.OracleGraph.from_pairs(s, d, dedup=True).run(micro=False).totals()
        bad += int(not (np.asarray(results[i]) == want).all())
    return len(pick), bad


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


def page_locked(a):
    """A page-locked copy of a numpy array (torch's pinned allocator), or None
    without torch."""
    try:
        import torch
    except ImportError:
        return None
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


def plain_loop(ctx, graphs):
    """One graph per call: upload, build, decompose."""
    out = []
    t0 = time.perf_counter()
    for s, d in graphs:
        g = ctx.graph_from_edges(s, d)
        out.append(g.decompose(micro=False).totals)
        g.destroy()
    return out, time.perf_counter() - t0


def plain_batch1(ctx, graphs):
    """One graph per call through the batch kernels (a batch of one)."""
    out = []
    t0 = time.perf_counter()
    for s, d in graphs:
        out.append(ctx.decompose_pairs_batch_flat(np.array([0, len(s)], np.int64), s, d)[0].totals)
    return out, time.perf_counter() - t0


def run_batch(args, emit=True):
    t0 = time.perf_counter()
    graphs, specs = batch_graphs(args.graphs, args.seed)
    pairs = sum(len(s) for s, _ in graphs)
    log("generated %d graphs, %d pairs in %.1fs" % (len(graphs), pairs, time.perf_counter() - t0))
    ctx = pgd.Context()
    default_thr = ctx.thresholds()
    # autotune on a stratified sample (every 16th graph)
    sample = [ctx.graph_from_edges(s, d) for s, d in graphs[:: max(1, len(graphs) // 256)]]
    a, c, dm, ms = ctx.autotune(sample, reps=1)
    tmd = ctx.tensor_min_degree()
    for g in sample:
        g.destroy()
    log("autotuned thresholds: anchor_hub=%d cache_hub=%d dense_max=%d" % (a, c, dm))
    # warm-up, then timed runs of the whole set in one call, from host pair
    # arrays in the call's own input format, concatenated (and page-locked,
    # where torch is present) outside the timing
    ctx.decompose_pairs_batch(graphs[:64])
    off, src, dst = pgd.concat_pairs(graphs)
    src, dst, pinned = page_locked(src), page_locked(dst), True
    if src is None or dst is None:
        off, src, dst = pgd.concat_pairs(graphs)
        pinned = False
    times = []
    res = None
    for _ in range(args.reps):
        t0 = time.perf_counter()
        res = ctx.decompose_pairs_batch_flat(off, src, dst)
        times.append(time.perf_counter() - t0)
    best = min(times)
    # plain baselines over an evenly spaced sample of the same graphs, one graph
    # per call: the single-graph API (with the default and with the tuned
    # thresholds) and the batch kernels on a batch of one; the speed-up is
    # quoted against the fastest of the three.  They read the same host
    # memory: views into the batch's arrays.
    step = max(1, len(graphs) // max(1, args.plain_sample))
    idx = list(range(0, len(graphs), step))
    sub = [(src[off[i]:off[i + 1]], dst[off[i]:off[i + 1]]) for i in idx]
    k = len(idx)
    plain = {}
    tuned_rate = None
    p_t, s_t = plain_loop(ctx, sub)
    plain["single_graph_api_tuned"] = k / s_t
    ctx.set_thresholds(*default_thr)
    p_d, s_d = plain_loop(ctx, sub)
    plain["single_graph_api_default"] = k / s_d
    ctx.set_thresholds(a, c, dm)
    p_b, s_b = plain_batch1(ctx, sub)
    plain["batch_of_one"] = k / s_b
    mismatch = 0
    for lst in (p_t, p_d, p_b):
        mismatch += sum(int(not (p == res[i].totals).all()) for p, i in zip(lst, idx))
    best_plain = max(plain.values())
    checked, oracle_bad = oracle_check(graphs, [r.totals for r in res])
    line = {
        "mode": "batch", "graphs": len(graphs), "pairs": pairs, "seconds": best, "graphs_per_s": len(graphs) / best,
        "kernel_ms": float(res[0].kernel_ms) if res else 0.0,
        "plain_graphs": k, "plain_graphs_per_s": plain, "speedup_vs_best_plain": (len(graphs) / best) / best_plain,
        "mismatches_vs_plain": mismatch, "oracle_checked": checked, "oracle_mismatches": oracle_bad,
        "speedup_vs_single_graph_api": (len(graphs) / best) / max(plain["single_graph_api_default"],
                                                                  plain["single_graph_api_tuned"]),
        "speedup_vs_batch_of_one": (len(graphs) / best) / plain["batch_of_one"],
        "thresholds": {"anchor_hub": a, "cache_hub": c, "dense_max": dm, "tensor_min_degree": tmd},
        "host_pairs": "page-locked" if pinned else "pageable",
        "workload": "%d graphs, n~U[16,2048], half G(n,p) p~U[0.01,0.5], half BA m~U{2..8}, seed %d"
                    % (len(graphs), args.seed),
    }
    ctx.close()
    if emit:
        print(json.dumps(line), flush=True)
    return line


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


def serve_once(reqs, expect, gaps, workers):
    """Submit reqs on the Poisson schedule gaps; wait for all; check them."""
    sv = pgd.Server(workers=workers)
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
    return stats, wall, mismatch


def run_serve(args, emit=True):
    t0 = time.perf_counter()
    reqs = serve_requests(args.requests, args.seed)
    pairs = sum(len(s) for s, _ in reqs)
    log("generated %d requests, %d pairs in %.1fs" % (len(reqs), pairs, time.perf_counter() - t0))
    # plain loops first (also the expected counts): one graph per call through
    # the single-graph API and through the batch kernels (a batch of one)
    ctx = pgd.Context()
    plain_loop(ctx, reqs[:16])
    expect, plain_s = plain_loop(ctx, reqs)
    plain_batch1(ctx, reqs[:16])
    expect1, plain1_s = plain_batch1(ctx, reqs)
    ctx.close()
    assert all((x == y).all() for x, y in zip(expect, expect1))
    plain_rates = {"single_graph_api": len(reqs) / plain_s, "batch_of_one": len(reqs) / plain1_s}
    plain_rate = max(plain_rates.values())
    checked, oracle_bad = oracle_check(reqs, expect)
    log("plain loops: %s graphs/s" % plain_rates)
    # warm-up
    sv = pgd.Server(workers=args.workers)
    for s, d in reqs[:8]:
        sv.wait(sv.submit(s, d), 60000)
    sv.close()
    rates = [float(r) for r in args.rates.split(",")] if args.rates else [args.rate]
    lines = []
    for rate in rates:
        rng = np.random.default_rng(args.seed + 1)
        gaps = rng.exponential(1.0 / rate, len(reqs))
        stats, wall, mismatch = serve_once(reqs, expect, gaps, args.workers)
        line = {
            "mode": "serve", "requests": len(reqs), "pairs": pairs, "offered_rate": rate,
            "graphs_per_s": stats["graphs_per_s"], "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"],
            "mean_ms": stats["mean_ms"], "queue_p50_ms": stats["queue_p50_ms"], "queue_p99_ms": stats["queue_p99_ms"],
            "service_p50_ms": stats["service_p50_ms"], "service_p99_ms": stats["service_p99_ms"],
            "skipped_ahead": stats["skipped_ahead"], "batches": stats["batches"], "wall_s": wall,
            "plain_graphs_per_s": plain_rates, "speedup_vs_best_plain": stats["graphs_per_s"] / plain_rate,
            "mismatches_vs_plain": mismatch, "oracle_checked": checked, "oracle_mismatches": oracle_bad,
            "workers": args.workers,
            "workload": "Poisson arrivals; m ~ lognormal(median 5000, sigma 1.2, <= 50M); half RMAT, half G(n,p) "
                        "mean degree 16; seed %d" % args.seed,
        }
        lines.append(line)
        if emit:
            print(json.dumps(line), flush=True)
    return lines


RMAT = dict(a=0.57, b=0.19, c=0.19)


def run_profile_batch(args):
    """The batched workload on its first `graphs` graphs (ncu captures of the
    batch kernels on a small case)."""
    graphs, _ = batch_graphs(args.graphs, args.seed)
    ctx = pgd.Context()
    ctx.set_thresholds(64, 128, 2048)
    if args.tensor_min_degree >= 0:
        ctx.set_tensor_min_degree(args.tensor_min_degree)
    res = None
    for _ in range(max(1, args.reps)):
        res = ctx.decompose_pairs_batch(graphs)
    print(json.dumps({"mode": "profile_batch", "graphs": len(graphs), "pairs": sum(len(s) for s, _ in graphs),
                      "tensor_min_degree": ctx.tensor_min_degree(), "kernel_ms": float(res[0].kernel_ms)}),
          flush=True)


def run_profile(args):
    s, d = pgd.rmat(args.scale, 16, seed=1, **RMAT)
    ctx = pgd.Context()
    g = ctx.graph_from_edges(s, d)
    g.preprocess("deg")
    g.compute_cores()
    g.sort_edges(args.order)
    for _ in range(args.reps):
        res = g.decompose(micro=True)
        print(json.dumps({"mode": "profile", "scale": args.scale, "order": args.order, "n": int(res.n),
                          "m": int(res.m), "kernel_ms": float(res.kernel_ms), "hub_ms": float(res.hub_ms)}),
              flush=True)
    g.micro()   # the per-edge ids of the output rows (k_micro_ids)


def run_shard(args):
    """The edge-span split of one RMAT graph (pgd_gb300/shard.py) measured
    span by span on one GPU: each span's sort + decomposition time, their
    imbalance (max / mean), and the whole graph's time for comparison.  The
    spans' partial sums must add up to the whole graph's."""
    from pgd_gb300 import shard

    s, d = pgd.rmat(args.scale, 16, seed=1, **RMAT)
    ctx = pgd.Context()
    g = ctx.graph_from_edges(s, d)
    g.preprocess("deg")
    g.compute_cores()
    g.sort_edges(args.order)
    full = g.decompose(micro=True)
    full = g.decompose(micro=True)
    ev, eu, ids = g.edges()
    deg = np.bincount(ev, minlength=g.n) + np.bincount(eu, minlength=g.n)
    out = {"mode": "shard", "scale": args.scale, "n": g.n, "m": g.m, "full_kernel_ms": full.kernel_ms, "worlds": {}}
    for world in (2, 4, 8):
        for name, cost in (("cost_model", shard.edge_cost(ev, eu, deg, ids, ctx.thresholds()[1])),
                           ("edge_count", np.ones(len(ids)))):
            spans = shard.edge_spans(cost, world)
            times, hub, total = [], [], np.zeros(pgd.NSUMS, np.uint64)
            for lo, hi in spans:
                g.sort_edges_sample(ids[lo:hi].astype(np.int64), "natural", s2l=True)
                r = g.decompose(micro=True)
                times.append(r.kernel_ms)
                hub.append(r.hub_ms)
                total += r.sums
            assert (total == full.sums).all(), "span sums do not add up"
            out["worlds"]["%d_%s" % (world, name)] = {
                "span_kernel_ms": [round(t, 1) for t in times], "max_over_mean": max(times) / np.mean(times),
                "max_ms": max(times), "speedup_vs_full": full.kernel_ms / max(times)}
    print(json.dumps(out), flush=True)


def run_small(args):
    s, d = pgd.erdos_renyi(250, 0.9, seed=1)
    ctx = pgd.Context()
    g = ctx.graph_from_edges(s, d)
    g.preprocess("deg")
    g.sort_edges("deg")
    for _ in range(5):
        g.decompose(micro=True)
    t0 = time.perf_counter()
    kern = []
    for _ in range(args.reps):
        r = g.decompose(micro=True)
        kern.append(r.kernel_ms)
    dt = (time.perf_counter() - t0) / args.reps
    m = int(r.m)
    cols = np.empty((m, pgd.NMICRO), np.uint64)
    s1 = np.empty(m, np.int64)
    d1 = np.empty(m, np.int64)
    t0 = time.perf_counter()
    for _ in range(args.reps):
        ge = ctx.graph_from_edges(s, d)
        ge.preprocess("deg")
        ge.sort_edges("deg")
        ge.decompose(micro=True)
        pgd.lib().pgd_get_micro(ge.h, pgd._ptr(s1), pgd._ptr(d1), pgd._ptr(cols))
        ge.destroy()
    e2e = (time.perf_counter() - t0) / args.reps
    print(json.dumps({"mode": "small", "graph": "G(250, 0.9) seed 1", "n": int(r.n), "m": m,
                      "decompose_ms": dt * 1000, "kernel_ms": float(np.median(kern)), "edges_per_s": m / dt,
                      "e2e_ms": e2e * 1000, "e2e_edges_per_s": m / e2e}), flush=True)


def large_pairs(name, seed):
    if name == "rmat24":
        return pgd.rmat(24, 16, seed=seed, **RMAT), "RMAT scale 24, edge factor 16, (0.57,0.19,0.19,0.05)"
    if name == "rgg24":
        n = 1 << 24
        r = (3 * 24 / (4 * math.pi * n)) ** (1.0 / 3.0)
        return pgd.rgg3d(n, r, seed=seed), "3-D RGG n=2^24 in the unit cube, r=%.6f" % r
    raise ValueError(name)


def run_large(args):
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests"))
    for name in args.workloads.split(","):
        t0 = time.perf_counter()
        (src, dst), desc = large_pairs(name, args.seed)
        gen_s = time.perf_counter() - t0
        ctx = pgd.Context()
        t0 = time.perf_counter()
        g = ctx.graph_from_edges(src, dst)
        g.preprocess("deg")
        g.compute_cores()
        build_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        g.sort_edges("kcore")
        res = g.decompose(micro=True)
        step_s = time.perf_counter() - t0
        m = int(res.m)
        log("%s: n=%d m=%d build %.1fs, sort+decompose %.2fs (kernels %.1f ms)"
            % (name, res.n, m, build_s, step_s, res.kernel_ms))
        s1, d1, cols = g.micro()
        M64 = (1 << 64) - 1
        tot = dict(zip(pgd.TOTAL_NAMES, (int(x) for x in res.totals)))
        N = {i: int(res.sums[4 + i]) for i in range(1, 11)}
        checks = {
            "sum_t": bool(res.sums[0] == cols[:, 0].sum(dtype=np.uint64)),
            "sum_k4": bool(res.sums[3] == cols[:, 2].sum(dtype=np.uint64)),
            "sum_c4": bool(res.sums[4] == cols[:, 5].sum(dtype=np.uint64)),
            "chord_clique": (tot["total_4_chordcycle"] + 6 * tot["total_4_clique"]) & M64 == N[3],
            "path_cycle": (tot["total_4_path"] + 4 * tot["total_4_cycle"]) & M64 == N[5],
        }
        # sampled rows against the oracle (host CSR of the same pairs)
        import oracle_lib as ol

        t0 = time.perf_counter()
        o = ol.OracleGraph.from_pairs(src, dst, dedup=True)
        rng = np.random.default_rng(args.seed)
        pos = np.concatenate([rng.choice(m, size=min(args.samples, m), replace=False),
                              np.arange(min(args.heavy, m))])
        t_o, k_o, c_o = o.edge_sample(s1[pos] - 1, d1[pos] - 1)
        checks["sampled_rows"] = int(len(pos))
        checks["sampled_rows_equal"] = bool((t_o == cols[pos, 0]).all() and (k_o == cols[pos, 2]).all()
                                            and (c_o == cols[pos, 5]).all())
        oracle_s = time.perf_counter() - t0
        line = {
            "mode": "large", "workload": name, "graph": desc, "n": int(res.n), "m": m,
            "edges_per_s": m / step_s, "seconds": step_s, "kernel_ms": float(res.kernel_ms),
            "build_seconds": build_s, "generate_seconds": gen_s, "oracle_check_seconds": oracle_s,
            "checks": checks, "totals": tot,
        }
        print(json.dumps(line), flush=True)
        del o, cols, s1, d1
        g.destroy()
        ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["batch", "serve", "large", "profile", "small", "profile_batch", "shard"])
    ap.add_argument("--workloads", default="rmat24,rgg24")
    ap.add_argument("--samples", type=int, default=1000)
    ap.add_argument("--heavy", type=int, default=10)
    ap.add_argument("--scale", type=int, default=18)
    ap.add_argument("--order", default="kcore")
    ap.add_argument("--graphs", type=int, default=4096)
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=4000.0)
    ap.add_argument("--rates", default="", help="comma-separated offered rates to sweep (overrides --rate)")
    ap.add_argument("--workers", type=int, default=2)
    ap.add_argument("--reps", type=int, default=3)  # batch: timed repetitions; profile: decompositions
    ap.add_argument("--plain-sample", type=int, default=256)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--tensor-min-degree", type=int, default=-1, help="profile_batch: -1 keeps the default")
    args = ap.parse_args()
    if args.mode == "batch":
        run_batch(args)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "large":
        run_large(args)
    elif args.mode == "small":
        run_small(args)
    elif args.mode == "profile_batch":
        run_profile_batch(args)
    elif args.mode == "shard":
        run_shard(args)
    else:
        run_profile(args)


if __name__ == "__main__":
    main()
