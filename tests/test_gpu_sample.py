"""Sampled decomposition: sort_edges over a sample of edge ids (the E_s
overload, graphlet_core.cpp:836-851) followed by the decomposition of those
edges only.  Totals, raw sums, the order and every per-edge row equal the
oracle's sampled run, whose own parity with the reference is checked in
test_oracle.py."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu


def sample_ids(kind, m, rng):
    if kind == "subset":
        return rng.choice(m, max(1, m // 3), replace=False)
    if kind == "repeats":
        return rng.integers(0, m, max(1, m // 2))
    if kind == "all":
        return rng.permutation(m)
    return np.zeros(0, np.int64)


@pytest.mark.parametrize("graph", ["rmat", "er", "ba"])
@pytest.mark.parametrize("order,s2l,kind", [("natural", False, "subset"), ("deg", False, "repeats"),
                                             ("kcore", False, "subset"), ("kcore", True, "all"),
                                             ("deg", False, "empty")])
def test_sampled_decomposition_matches_oracle(ctx, graph, order, s2l, kind):
    s, d = {"rmat": lambda: pgd.rmat(12, 16, seed=21), "er": lambda: pgd.erdos_renyi(300, 0.2, seed=22),
            "ba": lambda: pgd.barabasi_albert(3000, 6, seed=23)}[graph]()
    rng = np.random.default_rng(5)
    g = ctx.graph_from_edges(s, d)
    g.preprocess("deg")
    ids = sample_ids(kind, g.m, rng)
    g.sort_edges_sample(ids, order, s2l)
    assert g.order_length == len(ids)
    r = g.decompose(micro=True)
    o = ol.OracleGraph.from_pairs(s, d, dedup=True).run_sample(ids, order=order, s2l=s2l)
    assert (r.totals == o.totals()).all()
    assert (r.sums == o.sums()).all()
    assert (g.edges()[2] == o.order()).all()
    a, b, c = g.micro()
    x, y, z = o.micro()
    assert len(c) == len(ids)
    assert (a == x).all() and (b == y).all() and (c == z).all()
    # back to the full order: the full decomposition again
    g.sort_edges(order, s2l)
    assert g.order_length == g.m
    full = g.decompose(micro=False)
    assert (full.totals == ol.OracleGraph.from_pairs(s, d, dedup=True).run(order=order, s2l=s2l,
                                                                          micro=False).totals()).all()


def test_sampled_edge_ids_are_checked(ctx):
    s, d = pgd.erdos_renyi(50, 0.3, seed=2)
    g = ctx.graph_from_edges(s, d)
    with pytest.raises(pgd.PGDError):
        g.sort_edges_sample([0, g.m], "deg")
    with pytest.raises(pgd.PGDError):
        g.sort_edges_sample(np.arange(g.m + 1) % g.m, "deg")


def test_batches_reject_sampled_orders(ctx):
    s, d = pgd.erdos_renyi(60, 0.3, seed=3)
    g1 = ctx.graph_from_edges(s, d)
    g2 = ctx.graph_from_edges(s, d)
    g1.sort_edges_sample([0, 1, 2], "deg")
    with pytest.raises(pgd.PGDError):
        ctx.decompose_batch([g1, g2])
