"""Batched decomposition (many uneven graphs in one pass) and the work-split
thresholds: per-graph results identical to single-graph decomposition and to
the oracle, whatever the thresholds."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu


def mixed_graphs(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(16, 400))
        kind = i % 4
        if kind == 0:
            out.append(pgd.erdos_renyi(n, float(rng.uniform(0.01, 0.5)), seed=seed * 1000 + i))
        elif kind == 1:
            out.append(pgd.barabasi_albert(n, int(rng.integers(2, 9)), seed=seed * 1000 + i))
        elif kind == 2:
            out.append(pgd.rmat(int(rng.integers(6, 10)), 8, seed=seed * 1000 + i))
        else:
            k = int(rng.integers(0, 3 * n))
            out.append((rng.integers(0, n, k).astype(np.int32), rng.integers(0, n, k).astype(np.int32)))
    return out


@pytest.mark.parametrize("dense_max", [0, 128, 2048])
def test_batch_matches_single_and_oracle(dense_max):
    ctx = pgd.Context()
    ctx.set_thresholds(128, 64, dense_max)
    pairs = mixed_graphs(40, 1) + [(np.zeros(0, np.int32), np.zeros(0, np.int32)),
                                   (np.array([0], np.int32), np.array([1], np.int32))]
    graphs = [ctx.graph_from_edges(s, d) for s, d in pairs]
    for i, g in enumerate(graphs):
        g.preprocess("deg")
        g.sort_edges("kcore" if i % 2 else "deg")
    res = ctx.decompose_batch(graphs, micro=True)
    for i, ((s, d), g, r) in enumerate(zip(pairs, graphs, res)):
        o = ol.OracleGraph.from_pairs(s, d, dedup=True).run(order="kcore" if i % 2 else "deg")
        assert (r.totals == o.totals()).all(), i
        assert (r.sums == o.sums()).all(), i
        a, b, c = g.micro()
        x, y, z = o.micro()
        assert (a == x).all() and (b == y).all() and (c == z).all(), i
        single = g.decompose(micro=False)
        assert (single.totals == r.totals).all()
    ctx.close()


@pytest.mark.parametrize("anchor,cache", [(2, 2), (32, 512), (256, 32), (64, 64), (128, 1 << 30)])
def test_thresholds_never_change_counts(anchor, cache):
    c = pgd.Context()
    c.set_thresholds(anchor, cache)
    assert c.thresholds() == (anchor, cache, 2048)
    for s, d in [pgd.rmat(12, 16, seed=3), pgd.erdos_renyi(300, 0.3, seed=4), pgd.barabasi_albert(2000, 7, seed=5)]:
        g = c.graph_from_edges(s, d)
        r = g.decompose(micro=True)
        o = ol.OracleGraph.from_pairs(s, d, dedup=True).run()
        assert (r.totals == o.totals()).all()
        assert (g.micro()[2] == o.micro()[2]).all()
    c.close()


def test_thresholds_rejected_out_of_range(ctx):
    with pytest.raises(pgd.PGDError):
        ctx.set_thresholds(1, 64)
    with pytest.raises(pgd.PGDError):
        ctx.set_thresholds(300, 64)
    with pytest.raises(pgd.PGDError):
        ctx.set_thresholds(128, 64, 4096)


def test_autotune_keeps_counts():
    c = pgd.Context()
    pairs = mixed_graphs(12, 7)
    graphs = [c.graph_from_edges(s, d) for s, d in pairs]
    a, h, d, ms = c.autotune(graphs, reps=1)
    assert 2 <= a <= 256 and h >= 2 and 0 <= d <= 2048 and ms > 0
    assert c.thresholds() == (a, h, d)
    res = c.decompose_batch(graphs)
    for (s, d), r in zip(pairs, res):
        o = ol.OracleGraph.from_pairs(s, d, dedup=True).run(micro=False)
        assert (r.totals == o.totals()).all()
    c.close()


@pytest.mark.parametrize("case", ["hist16_global", "hist32_global", "bitmap_split", "bitmap_large_n"])
def test_hub_kernel_layouts(case):
    """k_hub keeps the W histogram (16-bit counters when the maximum degree is
    below 65536, else 32-bit) in shared memory when it fits, and the N(p)
    bitmap over degree ranks in the rest of shared memory, with per-CTA
    global slices for what does not fit; every layout gives the oracle's
    counts."""
    c = pgd.Context()
    n_min = 0
    smem = 156 * 1024
    if case == "hist16_global":
        # 120k hubs (every vertex) at 2 B each do not fit in shared memory
        c.set_thresholds(2, 2)
        s, d = pgd.barabasi_albert(120000, 6, seed=11)
    elif case == "hist32_global":
        # a vertex of degree 70000 forces 32-bit counters; 70k hubs at 4 B
        c.set_thresholds(2, 2)
        s0, d0 = pgd.barabasi_albert(70000, 2, seed=13)
        leaves = np.arange(70000, dtype=np.int32)
        s = np.concatenate([s0, leaves])
        d = np.concatenate([d0, np.full(70000, 70000, np.int32)])
    elif case == "bitmap_split":
        # 78k hubs fill shared memory with counters: only the ~30k highest
        # ranks of the bitmap stay shared, the rest are in global memory
        c.set_thresholds(2, 2)
        s, d = pgd.barabasi_albert(78000, 6, seed=14)
    else:
        # 2M vertices (mostly isolated): the bitmap's tail is in global memory
        s, d = pgd.rmat(12, 16, seed=12)
        n_min = 2_000_000
    g = c.graph_from_edges(s, d, n_min=n_min)
    og = ol.OracleGraph.from_pairs(s, d, n_min=n_min, dedup=True)
    deg = np.diff(og.csr()[0])
    n = len(deg)
    if case == "hist16_global":
        assert deg.max() < 65536 and (deg >= 2).sum() * 2 > smem
    elif case == "hist32_global":
        assert deg.max() >= 65536 and (deg >= 2).sum() * 4 > smem
    elif case == "bitmap_split":
        hist = ((deg >= 2).sum() + 1) // 2 * 4
        assert deg.max() < 65536 and hist <= smem and (smem - hist) * 8 < n // 2
    else:
        assert n / 8 > smem
    r = g.decompose(micro=True)
    o = og.run()
    assert (r.totals == o.totals()).all()
    assert (r.sums == o.sums()).all()
    a, b, cols = g.micro()
    x, y, z = o.micro()
    assert (cols == z).all()
    c.close()


def test_dense_graphs_common_neighbour_path():
    """Batched graphs of at most 2048 vertices and average degree >= n/16 are
    decomposed with a common-neighbour matrix (c4 from the identity over
    CN[p][w] and CN[q][x]); sparser ones in the same batch keep the plain
    row-bitset kernel.  Totals, raw sums and per-edge rows equal the
    single-graph kernels' (k_hub / k_light), and the oracle's on the small
    graphs."""
    c = pgd.Context()
    c.set_thresholds(128, 64, 2048)
    specs = [(2048, 0.5), (2000, 0.07), (1500, 0.3), (1025, 0.2), (700, 0.9), (64, 1.0), (65, 0.5),
             (300, 0.06), (129, 0.4), (33, 0.8), (1800, 0.01)]
    pairs = [pgd.erdos_renyi(n, p, seed=100 + i) for i, (n, p) in enumerate(specs)]
    pairs.append(pgd.barabasi_albert(900, 3, seed=8))
    graphs = [c.graph_from_edges(s, d) for s, d in pairs]
    cn_path = []
    for g, (s, d) in zip(graphs, pairs):
        g.preprocess("deg")
        g.sort_edges("kcore")
    res = c.decompose_batch(graphs, micro=True)
    batch_rows = [g.micro() for g in graphs]
    for i, (g, r) in enumerate(zip(graphs, res)):
        cn_path.append(32 * r.m >= r.n * r.n)
        single = g.decompose(micro=True)
        assert (single.totals == r.totals).all(), i
        assert (single.sums == r.sums).all(), i
        a, b, cols = g.micro()
        x, y, z = batch_rows[i]
        assert (a == x).all() and (b == y).all() and (cols == z).all(), i
    assert sum(cn_path) >= 7 and not all(cn_path)
    for i in (5, 6, 8, 9, 7):
        o = ol.OracleGraph.from_pairs(*pairs[i], dedup=True).run(order="kcore")
        assert (res[i].totals == o.totals()).all(), i
        assert (batch_rows[i][2] == o.micro()[2]).all(), i
    # the pairs batch (device CSR build of the union) agrees
    pr = c.decompose_pairs_batch(pairs)
    for i, r in enumerate(pr):
        assert (r.totals == res[i].totals).all(), i
    c.close()
