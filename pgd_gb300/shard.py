"""Decomposition of one graph sharded over ranks.

Edges are independent given the CSR, so every rank holds the whole graph and
decomposes a contiguous span of the ordered edge list (E_ordered).  The spans
are weighted by an estimate of each edge's work in the decomposition kernels:
the scan of the non-anchor endpoint q's list plus the lists of its
low-degree neighbours, which are scanned per edge (see edge_cost).  Every
rank also computes the triangle count of every edge (the c4 identity reads
t of edges outside the span) and the graph's per-vertex structures: that
O(m) part is repeated on each rank and bounds strong scaling.  Each rank orders and decomposes its span with the sampled edge
order (`Graph.sort_edges_sample`, the reference's sort_edges with E_s,
graphlet_core.cpp:836-851).  The only exchange is a sum of the 15 uint64
partial sums, which wraps mod 2^64 exactly like the device sums.  The 17
totals are then closed on every rank from the summed partials
(graphlet_core.cpp:1449-1472).  Per-edge rows stay on the rank that owns the
span.

The span logic and the reduction are plain functions of arrays, so that they
can be exercised with any per-span decomposer (the tests use CPU processes
with the gloo backend).
"""
import numpy as np


def edge_spans(cost, world):
    """Contiguous spans [lo, hi) of the ordered edges, one per rank, with about
    equal total cost (the span of rank r ends where the prefix cost first
    reaches (r + 1) / world of the total)."""
    cost = np.asarray(cost, dtype=np.float64)
    m = len(cost)
    if world < 1:
        raise ValueError("world must be >= 1")
    c = np.cumsum(cost)
    total = c[-1] if m else 0.0
    bounds = [0]
    for r in range(1, world):
        b = int(np.searchsorted(c, total * r / world, side="left")) + 1 if m else 0
        bounds.append(min(max(b, bounds[-1]), m))
    bounds.append(m)
    return [(bounds[i], bounds[i + 1]) for i in range(world)]


def edge_cost(ev, eu, deg, order, cache_hub=40):
    """Work estimate of each ordered edge (p, q), p the endpoint of higher
    (degree, id): deg(q) slot records, plus the lists of q's neighbours of
    degree below cache_hub (their W(w, p) is counted per edge, the higher
    ones come from the anchor's histogram), plus one."""
    ev = np.asarray(ev, np.int64)
    eu = np.asarray(eu, np.int64)
    deg = np.asarray(deg, np.int64)
    n = len(deg)
    dv, du = deg[ev], deg[eu]
    small = np.bincount(ev, weights=np.where(du < cache_hub, du, 0), minlength=n) + \
        np.bincount(eu, weights=np.where(dv < cache_hub, dv, 0), minlength=n)
    a, b = ev[order], eu[order]
    da, db = deg[a], deg[b]
    q = np.where((da > db) | ((da == db) & (a > b)), b, a)
    return deg[q].astype(np.float64) + small[q] + 1.0


def reduce_sums(sums, group=None):
    """Sum of every rank's 15 uint64 partials (two's-complement int64 sums wrap
    exactly like uint64 ones)."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(sums, dtype=np.uint64).view(np.int64).copy())
    if dist.is_available() and dist.is_initialized():
        if dist.get_backend(group) == "nccl":   # NCCL reduces device tensors
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy().view(np.uint64).copy()


def sharded_totals(span_sums, n, m, close_counts, group=None):
    """Totals of the whole graph from this rank's partial sums."""
    sums = reduce_sums(span_sums, group)
    return close_counts(sums, n, m), sums


def decompose_sharded(ctx, src, dst, rank, world, order="kcore", micro=False, group=None):
    """Decompose the graph given by host pairs, this rank's span only, and
    return (totals, summed partials, this rank's Counts, its Graph).  With
    world == 1 the result equals an ordinary decomposition."""
    import pgd_gb300 as pgd

    g = ctx.graph_from_edges(src, dst)
    g.preprocess("deg")
    g.sort_edges(order)
    ev, eu, ids = g.edges()
    deg = np.bincount(ev, minlength=g.n) + np.bincount(eu, minlength=g.n)
    lo, hi = edge_spans(edge_cost(ev, eu, deg, ids), world)[rank]
    # natural key = position in the sample, ascending: the span keeps its order
    g.sort_edges_sample(ids[lo:hi], "natural", s2l=True)
    r = g.decompose(micro=micro)
    totals, sums = sharded_totals(r.sums, g.n, g.m, pgd.close_counts, group)
    return totals, sums, r, g
