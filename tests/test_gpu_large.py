"""Large graphs, where a full oracle run is too slow: sampled per-edge rows
against the oracle (the reference's marking procedure on each sampled edge)
and size-independent identities of the full result."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def check_large(ctx, src, dst, order, samples=3000, seed=0):
    g = ctx.graph_from_edges(src, dst)
    g.preprocess("deg")
    g.compute_cores()
    g.sort_edges(order)
    res = g.decompose(micro=True)
    s1, d1, cols = g.micro()
    m = len(cols)
    # per-edge columns agree with the global sums (mod 2^64)
    # numpy's uint64 sums wrap mod 2^64 exactly like the device sums
    assert res.sums[0] == cols[:, 0].sum(dtype=np.uint64)
    assert res.sums[3] == cols[:, 2].sum(dtype=np.uint64)
    assert res.sums[4] == cols[:, 5].sum(dtype=np.uint64)
    tot = dict(zip(pgd.TOTAL_NAMES, (int(x) for x in res.totals)))
    N = {i: int(res.sums[4 + i]) for i in range(1, 11)}
    assert (tot["total_4_chordcycle"] + 6 * tot["total_4_clique"]) & M64 == N[3]
    assert (tot["total_4_path"] + 4 * tot["total_4_cycle"]) & M64 == N[5]
    assert (2 * tot["total_4_2edge"] + tot["total_4_1edge"]) & M64 == N[8]
    # sampled rows, all 8 columns, by the reference's own procedure on each edge
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    deg = np.diff(o.csr()[0])

    def oracle_rows(v1, u1):
        v, u = v1 - 1, u1 - 1
        t_o, k_o, c_o = o.edge_sample(v, u)
        return ol.micro_rows(deg[v], deg[u], t_o, k_o, c_o)

    rng = np.random.default_rng(seed)
    pos = rng.choice(m, size=min(samples, m), replace=False)
    assert (oracle_rows(s1[pos], d1[pos]) == cols[pos]).all()
    # the heaviest rows too (first positions of the degree order)
    g.sort_edges("deg")
    r2 = g.decompose(micro=True)
    assert (r2.totals == res.totals).all()
    s2, d2, cols2 = g.micro()
    head = np.arange(min(200, m))
    assert (oracle_rows(s2[head], d2[head]) == cols2[head]).all()
    g.destroy()
    return res


def test_rmat21(ctx):
    src, dst = pgd.rmat(21, 16, seed=1)
    check_large(ctx, src, dst, "kcore")


def test_rgg3d_2p20(ctx):
    n = 1 << 20
    r = (3 * 24 / (4 * np.pi * n)) ** (1.0 / 3.0)
    src, dst = pgd.rgg3d(n, r, seed=1)
    res = check_large(ctx, src, dst, "kcore")
    assert res.m > 10 * n
