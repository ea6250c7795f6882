"""GPU parity: the CUDA path (through the C ABI) against the reference's
golden vectors and the CPU oracle, bit for bit: the 17 global counts, the
per-edge rows, their order, k-core numbers, the edge arrays."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd
from helpers import (bign_pairs, brute_force_counts, load_npz, load_toys, mtx_pairs, rows_digest,
                     write_pairs_mtx)

pytestmark = pytest.mark.gpu

SYNTH = ["er250", "rmat12", "ba2000", "er1500"]
ORDERS = [("deg", False), ("kcore", False), ("natural", False), ("deg", True)]


def run_gpu(g, order="deg", s2l=False, neigh="deg", s2l_neigh=False, micro=True):
    g.preprocess(neigh, s2l_neigh)
    K = g.compute_cores()
    g.sort_edges(order, s2l)
    res = g.decompose(micro=micro)
    return res, K


def assert_same_as_oracle(g, o, micro=True):
    res, K = run_gpu(g, micro=micro)
    assert (g.n, g.m) == (o.n, o.m)
    assert (res.totals == o.totals()).all(), (res.totals, o.totals())
    assert (res.sums == o.sums()).all()
    if micro:
        s, d, c = g.micro()
        x, y, z = o.micro()
        assert (s == x).all() and (d == y).all()
        assert (c == z).all()
    return res


@pytest.mark.parametrize("name", sorted(load_toys().keys()))
def test_toy_graphs(ctx, tmp_path, name):
    toy = load_toys()[name]
    p = tmp_path / name
    p.write_text(toy["text"])
    g = ctx.graph_from_file(str(p))
    res, K = run_gpu(g)
    assert (g.n, g.m, K) == (toy["n"], toy["m"], toy["K"])
    assert [int(x) for x in res.totals] == toy["totals"]
    s, d, c = g.micro()
    assert [[int(a), int(b)] + [int(x) for x in r] for a, b, r in zip(s, d, c)] == toy["rows"]


def test_sample_graph_rows_and_golden(ctx, tmp_path):
    z = load_npz("dd21.npz")
    p = tmp_path / "sample_graph.csv"
    with open(p, "w") as f:
        f.write(str(z["header"]) + "\n")
        for a, b in z["pairs"]:
            f.write("%d,%d\n" % (a, b))
    g = ctx.graph_from_file(str(p))
    res, K = run_gpu(g)
    assert K == int(z["K"])
    assert (res.totals == z["totals"]).all()
    s, d, c = g.micro()
    assert (s == z["src"]).all() and (d == z["dst"]).all() and (c == z["cols"]).all()
    res, _ = run_gpu(g, order="kcore")
    s, d, c = g.micro()
    assert (res.totals == z["kc_totals"]).all()
    assert (s == z["kc_src"]).all() and (d == z["kc_dst"]).all() and (c == z["kc_cols"]).all()


@pytest.mark.parametrize("name", SYNTH)
def test_synthetic_vs_reference_fixtures(ctx, name):
    z = load_npz("synth.npz")
    src, dst = mtx_pairs(z[name + "_u"], z[name + "_v"])
    g = ctx.graph_from_edges(src, dst, dedup=False)
    for order, s2l in ORDERS:
        tag = "%s_%s%s" % (name, order, "_s2l" if s2l else "")
        res, K = run_gpu(g, order=order, s2l=s2l)
        n, m, Kref = z[tag + "_meta"]
        assert (g.n, g.m, K) == (n, m, Kref)
        assert (res.totals == z[tag + "_totals"]).all(), tag
        s, d, c = g.micro()
        assert rows_digest(s, d, c) == str(z[tag + "_rows_sha256"]), tag
        r = g.assortativity()
        assert float("%.6g" % r) == float("%.6g" % float(z[tag + "_r"]))


def test_mtx_file_reader(ctx, tmp_path):
    z = load_npz("synth.npz")
    src, dst = mtx_pairs(z["rmat12_u"], z["rmat12_v"])
    p = tmp_path / "g.mtx"
    write_pairs_mtx(str(p), src, dst)
    g = ctx.graph_from_file(str(p))
    res, _ = run_gpu(g)
    assert (res.totals == z["rmat12_deg_totals"]).all()


def test_huge_n_closing_wraps(ctx):
    z = load_npz("bign.npz")
    src, dst = bign_pairs(z)
    g = ctx.graph_from_edges(src, dst, dedup=False)
    res, _ = run_gpu(g, micro=False)
    assert g.n == int(z["n"]) and g.m == int(z["m"])
    assert (res.totals == z["totals"]).all()


@pytest.mark.parametrize("seed", range(8))
def test_random_graphs_vs_oracle(ctx, seed):
    rng = np.random.default_rng(seed)
    kind = seed % 4
    if kind == 0:
        src, dst = pgd.erdos_renyi(int(rng.integers(50, 400)), float(rng.uniform(0.02, 0.6)), seed=seed)
    elif kind == 1:
        src, dst = pgd.barabasi_albert(int(rng.integers(100, 3000)), int(rng.integers(2, 9)), seed=seed)
    elif kind == 2:
        src, dst = pgd.rmat(int(rng.integers(8, 12)), 8, seed=seed)
    else:
        n = int(rng.integers(20, 300))
        k = int(rng.integers(n, 10 * n))
        src = rng.integers(0, n, k).astype(np.int32)
        dst = rng.integers(0, n, k).astype(np.int32)
    g = ctx.graph_from_edges(src, dst, dedup=True)
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True).run()
    assert_same_as_oracle(g, o)
    assert (g.kcore() == o.kcore()).all()
    ev, eu, order = g.edges()
    oev, oeu = o.edges()
    assert (ev == oev).all() and (eu == oeu).all() and (order == o.order()).all()


@pytest.mark.parametrize("order", ["kcore_deg", "deg_vol", "kcore_vol", "kcore_deg_vol", "triangles", "natural",
                                   "kcore"])
@pytest.mark.parametrize("s2l", [False, True])
def test_edge_orders_vs_oracle(ctx, order, s2l):
    src, dst = pgd.barabasi_albert(1500, 4, seed=9)
    g = ctx.graph_from_edges(src, dst, dedup=True)
    res, _ = run_gpu(g, order=order, s2l=s2l)
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True).run(order=order, s2l=s2l)
    assert (res.totals == o.totals()).all()
    s, d, c = g.micro()
    x, y, w = o.micro()
    assert (s == x).all() and (d == y).all() and (c == w).all()


@pytest.mark.parametrize("neigh,s2l", [("kcore", False), ("natural", False), ("deg", True), ("kcore", True)])
def test_neighbour_orders_vs_oracle(ctx, neigh, s2l):
    src, dst = pgd.rmat(11, 8, seed=4)
    g = ctx.graph_from_edges(src, dst, dedup=True)
    res, _ = run_gpu(g, neigh=neigh, s2l_neigh=s2l)
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True).run(neigh=neigh, s2l_neigh=s2l)
    s, d, c = g.micro()
    x, y, w = o.micro()
    assert (s == x).all() and (d == y).all() and (c == w).all()


def test_csr_input_vs_oracle(ctx):
    src, dst = pgd.barabasi_albert(800, 3, seed=5)
    o0 = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    off, adj = o0.csr()
    # shuffle each row: the row order is the insertion order the reference keeps
    rng = np.random.default_rng(0)
    adj = adj.copy()
    for v in range(len(off) - 1):
        seg = adj[off[v]:off[v + 1]]
        rng.shuffle(seg)
    g = ctx.graph_from_csr(off, adj)
    o = ol.OracleGraph.from_csr(off, adj).run()
    assert_same_as_oracle(g, o)


# ---------------------------------------------------------------------------
# edge cases


def test_empty_and_tiny_graphs(ctx):
    for src, dst, n_min in [([], [], 0), ([0], [1], 0), ([0], [1], 10), ([0, 1, 2], [1, 2, 0], 3),
                            ([0, 0, 0, 0, 0], [1, 2, 3, 4, 5], 0), ([3], [3], 5)]:
        src = np.array(src, np.int32)
        dst = np.array(dst, np.int32)
        g = ctx.graph_from_edges(src, dst, n_min=n_min, dedup=True)
        res, _ = run_gpu(g)
        o = ol.OracleGraph.from_pairs(src, dst, n_min=n_min, dedup=True).run()
        assert (g.n, g.m) == (o.n, o.m)
        assert (res.totals == o.totals()).all()


def test_isolated_vertices_change_disconnected_counts(ctx):
    src = np.array([0, 1, 2, 2], np.int32)
    dst = np.array([1, 2, 0, 3], np.int32)
    a, _ = run_gpu(ctx.graph_from_edges(src, dst, n_min=0))
    b, _ = run_gpu(ctx.graph_from_edges(src, dst, n_min=9))
    want = brute_force_counts(9, list(zip(src.tolist(), dst.tolist())))
    got = dict(zip(pgd.TOTAL_NAMES, (int(x) for x in b.totals)))
    assert got == want
    assert a.totals[6] == b.totals[6] and a.totals[16] != b.totals[16]


def test_all_graphs_on_five_vertices_vs_census(ctx):
    import itertools

    pairs = list(itertools.combinations(range(5), 2))
    for mask in range(1, 1 << len(pairs), 7):
        edges = [pairs[i] for i in range(len(pairs)) if mask >> i & 1]
        src = np.array([e[0] for e in edges], np.int32)
        dst = np.array([e[1] for e in edges], np.int32)
        res, _ = run_gpu(ctx.graph_from_edges(src, dst, n_min=5), micro=False)
        assert dict(zip(pgd.TOTAL_NAMES, (int(x) for x in res.totals))) == brute_force_counts(5, edges)


def test_duplicates_and_self_loops(ctx):
    src = np.array([0, 1, 1, 2, 0, 3, 3], np.int32)
    dst = np.array([1, 0, 2, 2, 2, 3, 0], np.int32)
    g = ctx.graph_from_edges(src, dst, dedup=True)
    info = g.info()
    assert (info.n, info.m, info.self_loops, info.duplicates) == (4, 4, 2, 1)
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_edges(src, dst, dedup=False)
    assert e.value.status == 1


def test_bad_inputs_are_rejected(ctx):
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_edges(np.array([-1], np.int32), np.array([2], np.int32))
    assert e.value.status == 1
    off = np.array([0, 1, 1], np.int64)
    adj = np.array([1], np.int32)  # 0->1 without 1->0
    with pytest.raises(pgd.PGDError):
        ctx.graph_from_csr(off, adj)
    off = np.array([0, 1], np.int64)
    with pytest.raises(pgd.PGDError):
        ctx.graph_from_csr(off, np.array([0], np.int32))  # self loop
    g = ctx.graph_from_edges(np.array([0, 1], np.int32), np.array([1, 2], np.int32))
    for bad in ("rand", "var"):
        with pytest.raises(pgd.PGDError) as e:
            g.sort_edges(bad)
        assert e.value.status == 6
    with pytest.raises(pgd.PGDError) as e:
        g.preprocess("rand")
    assert e.value.status == 6
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_file("/nonexistent/graph.mtx")
    assert e.value.status == 5


def test_mtx_duplicates_rejected(ctx, tmp_path):
    p = tmp_path / "dup.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n3 3 3\n2 1\n3 2\n2 1\n")
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_file(str(p))
    assert e.value.status == 1


def test_budget_refuses_graph(tmp_path):
    small = pgd.Context(hbm_budget=1 << 16)
    src, dst = pgd.rmat(12, 16, seed=1)
    with pytest.raises(pgd.PGDError) as e:
        small.graph_from_edges(src, dst)
    assert e.value.status == 2
    assert small.resident_bytes == 0
    small.close()


def test_repeat_decompositions_are_identical(ctx):
    src, dst = pgd.rmat(12, 16, seed=2)
    g = ctx.graph_from_edges(src, dst)
    a, _ = run_gpu(g)
    ca = g.micro(ids=False).copy()
    b = g.decompose(micro=True)
    cb = g.micro(ids=False)
    assert (a.totals == b.totals).all() and (ca == cb).all()


def test_large_graph_default_thresholds():
    """Graphs of more than 1.5·2^20 vertices take hub thresholds 128 / 40 while
    the caller has set none; counts must not change (against the oracle and
    against the 64 / 32 thresholds set explicitly), and the context's
    thresholds stay as they were."""
    s, d = pgd.rmat(14, 8, seed=6)
    n = (8 << 20) + 1000
    c = pgd.Context()
    before = c.thresholds()
    g = c.graph_from_edges(s, d, n_min=n)
    assert g.n == n
    g.preprocess("deg")
    g.compute_cores()
    g.sort_edges("kcore")
    r = g.decompose(micro=True)
    assert c.thresholds() == before
    rows = g.micro()
    c2 = pgd.Context()
    c2.set_thresholds(64, 32, 2048)
    g2 = c2.graph_from_edges(s, d, n_min=n)
    g2.preprocess("deg")
    g2.compute_cores()
    g2.sort_edges("kcore")
    r2 = g2.decompose(micro=True)
    assert (r.totals == r2.totals).all() and (r.sums == r2.sums).all()
    for a, b in zip(rows, g2.micro()):
        assert (a == b).all()
    o = ol.OracleGraph.from_pairs(s, d, n_min=n, dedup=True).run(order="kcore", micro=False)
    assert (r.totals == o.totals()).all()
    g.destroy()
    g2.destroy()
    c.close()
    c2.close()
