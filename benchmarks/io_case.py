"""A small case for capturing the host-I/O and run-list kernels: an RMAT
graph uploaded from page-locked pairs (k_copy_mapped), decomposed with
per-edge rows that go to page-locked host buffers (k_micro_out), then a
pairs batch of dense graphs (k_tc_run_flags, k_tc_run_fill, k_gram_tiles).

    python -m benchmarks.io_case [--scale 18] [--graphs 32]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import pgd_gb300 as pgd  # noqa: E402
from benchmarks.suite import batch_graphs, page_locked  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=18)
    ap.add_argument("--graphs", type=int, default=32)
    args = ap.parse_args()
    s, d = pgd.rmat(args.scale, 16, seed=1)
    ps, pd = page_locked(s), page_locked(d)
    if ps is None:
        raise SystemExit("needs torch for page-locked buffers")
    ctx = pgd.Context()
    g = ctx.graph_from_edges(ps, pd)
    g.preprocess("deg")
    g.compute_cores()
    g.sort_edges("kcore")
    g.decompose(micro=True)
    m = g.order_length
    cols = page_locked(np.zeros((m, pgd.NMICRO), np.uint64))
    s1 = page_locked(np.zeros(m, np.int64))
    d1 = page_locked(np.zeros(m, np.int64))
    t0 = time.perf_counter()
    assert pgd.lib().pgd_get_micro(g.h, pgd._ptr(s1), pgd._ptr(d1), pgd._ptr(cols)) == 0
    t_rows = time.perf_counter() - t0
    graphs, _ = batch_graphs(args.graphs, 1)
    res = ctx.decompose_pairs_batch(graphs)
    print(json.dumps({"n": g.n, "m": g.m, "rows_bytes": int(m * (pgd.NMICRO * 8 + 16)),
                      "rows_ms": round(t_rows * 1000, 2), "batch_graphs": len(res)}), flush=True)
    g.destroy()
    ctx.close()


if __name__ == "__main__":
    main()
