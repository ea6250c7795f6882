"""Sharded decomposition on the GPU: every rank's span decomposed through
the sampled edge order; the summed partials close to the whole graph's
totals, and the spans' per-edge rows are the whole graph's rows."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd
from pgd_gb300 import shard

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [1, 3])
def test_spans_sum_to_the_whole_graph(ctx, world):
    s, d = pgd.rmat(13, 16, seed=31)
    full = ol.OracleGraph.from_pairs(s, d, dedup=True).run(order="kcore", micro=True)
    fs, fd, fc = full.micro()
    acc = np.zeros(pgd.NSUMS, np.uint64)
    rows = 0
    for rank in range(world):
        totals, sums, r, g = shard.decompose_sharded(ctx, s, d, rank, world, order="kcore", micro=True)
        acc += r.sums                      # wraps mod 2^64 like the device sums
        a, b, c = g.micro()
        # the span's rows are the whole graph's rows at the span's positions
        assert (a == fs[rows:rows + len(a)]).all() and (c == fc[rows:rows + len(c)]).all()
        rows += len(a)
        if world == 1:
            assert (totals == full.totals()).all()
        g.destroy()
    assert rows == full.m
    assert (acc == full.sums()).all()
    assert (pgd.close_counts(acc, full.n, full.m) == full.totals()).all()
