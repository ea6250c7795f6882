"""Sharding one graph's ordered edge list over ranks: the span logic and the
one exchange (a wrapping sum of the 15 uint64 partials), as two gloo ranks on
the CPU.  Each rank decomposes its span with the oracle's sampled order; the
closed totals must equal the whole graph's."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

import oracle_lib as ol
from pgd_gb300 import shard


def test_edge_spans_cover_and_balance():
    rng = np.random.default_rng(1)
    for world in (1, 2, 3, 7):
        cost = rng.integers(1, 100, 1000).astype(np.float64)
        spans = shard.edge_spans(cost, world)
        assert spans[0][0] == 0 and spans[-1][1] == len(cost)
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
        loads = [cost[lo:hi].sum() for lo, hi in spans]
        assert max(loads) <= cost.sum() / world + cost.max()
    assert shard.edge_spans(np.zeros(0), 3) == [(0, 0), (0, 0), (0, 0)]
    assert shard.edge_spans(np.ones(2), 4)[-1][1] == 2


def _graph():
    rng = np.random.default_rng(7)
    n = 150
    src = rng.integers(0, n, 900).astype(np.int32)
    dst = rng.integers(0, n, 900).astype(np.int32)
    return src, dst


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    import pgd_gb300 as pgd

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    src, dst = _graph()
    full = ol.OracleGraph.from_pairs(src, dst, dedup=True).run(order="kcore", micro=False)
    ev, eu = full.edges()
    ids = full.order()
    deg = np.bincount(ev, minlength=full.n) + np.bincount(eu, minlength=full.n)
    lo, hi = shard.edge_spans(shard.edge_cost(ev, eu, deg, ids), world)[rank]
    part = ol.OracleGraph.from_pairs(src, dst, dedup=True).run_sample(ids[lo:hi], order="natural", s2l=True,
                                                                      micro=False)
    totals, sums = shard.sharded_totals(part.sums(), full.n, full.m, pgd.close_counts)
    out.put((rank, hi - lo, bool((totals == full.totals()).all()), bool((sums == full.sums()).all())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_whole_graph():
    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    env_path = os.pathsep.join([os.path.dirname(__file__), os.path.dirname(os.path.dirname(__file__))])
    old = os.environ.get("PYTHONPATH")
    os.environ["PYTHONPATH"] = env_path + (os.pathsep + old if old else "")
    try:
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        results = [out.get(timeout=120) for _ in procs]
        for p in procs:
            p.join(timeout=60)
    finally:
        if old is None:
            os.environ.pop("PYTHONPATH", None)
        else:
            os.environ["PYTHONPATH"] = old
    assert all(p.exitcode == 0 for p in procs)
    results.sort()
    assert sum(r[1] for r in results) > 0 and all(r[1] > 0 for r in results)
    assert all(r[2] and r[3] for r in results)
