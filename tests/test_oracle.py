"""The oracle (oracle/pgd_oracle.c) pinned against the reference's golden
vectors and, where the reference was compiled here, against the reference
itself.  CPU only."""
import itertools
import os

import numpy as np
import pytest

import oracle_lib as ol
from helpers import (READER_QUIRKS, bign_pairs, brute_force_counts, load_npz, load_toys, mtx_pairs, rows_digest)

SYNTH = ["er250", "rmat12", "ba2000", "er1500"]
ORDERS = [("deg", False), ("kcore", False), ("natural", False), ("deg", True)]


def _rows(g):
    s, d, c = g.micro()
    return s, d, c


@pytest.mark.parametrize("name", sorted(load_toys().keys()))
def test_toy_graphs(tmp_path, name):
    toy = load_toys()[name]
    p = tmp_path / name
    p.write_text(toy["text"])
    g = ol.OracleGraph.from_file(str(p)).run()
    assert g.n == toy["n"] and g.m == toy["m"] and g.max_core == toy["K"]
    assert [int(x) for x in g.totals()] == toy["totals"]
    s, d, c = _rows(g)
    rows = [[int(a), int(b)] + [int(x) for x in r] for a, b, r in zip(s, d, c)]
    assert rows == toy["rows"]


def test_toy_known_answers(tmp_path):
    """The counts the reference's toy graphs are built to show."""
    toys = load_toys()
    names = ol.TOTAL_NAMES
    t = dict(zip(names, toys["4-clique.txt"]["totals"]))
    assert t["total_4_clique"] == 1 and t["total_3_tris"] == 4
    assert all(t[k] == 0 for k in names if k not in ("total_4_clique", "total_3_tris", "total_2_1edge"))
    t = dict(zip(names, toys["4-chordal-cycle.txt"]["totals"]))
    assert t["total_4_chordcycle"] == 1 and t["total_3_tris"] == 2 and t["total_2_star"] == 2


def _write_sample_graph(tmp_path, z):
    p = tmp_path / "sample_graph.csv"
    with open(p, "w") as f:
        f.write(str(z["header"]) + "\n")
        for a, b in z["pairs"]:
            f.write("%d,%d\n" % (a, b))
    return str(p)


def test_sample_graph_matches_reference_rows(tmp_path):
    z = load_npz("dd21.npz")
    path = _write_sample_graph(tmp_path, z)
    g = ol.OracleGraph.from_file(path).run(order="deg")
    assert g.n == int(z["n"]) and g.m == int(z["m"]) and g.max_core == int(z["K"])
    assert (g.totals() == z["totals"]).all()
    s, d, c = _rows(g)
    assert (s == z["src"]).all() and (d == z["dst"]).all() and (c == z["cols"]).all()
    g = ol.OracleGraph.from_file(path).run(order="kcore")
    s, d, c = _rows(g)
    assert (g.totals() == z["kc_totals"]).all()
    assert (s == z["kc_src"]).all() and (d == z["kc_dst"]).all() and (c == z["kc_cols"]).all()


def test_sample_graph_golden_columns(tmp_path):
    """sample_graph.csv ships per-edge counts keyed by its own vertex ids; the
    reader relabels ids by first appearance (graphlet_core.cpp:424-440)."""
    z = load_npz("dd21.npz")
    path = _write_sample_graph(tmp_path, z)
    g = ol.OracleGraph.from_file(path).run()
    s, d, c = _rows(g)
    lookup = {}
    for a, b in z["pairs"]:
        if a == b:
            continue
        for x in (int(a), int(b)):
            if x not in lookup:
                lookup[x] = len(lookup)
    mine = {}
    for a, b, r in zip(s - 1, d - 1, c):
        mine[(min(a, b), max(a, b))] = tuple(int(x) for x in r)
    assert len(mine) == len(z["pairs"])
    for (a, b), r in zip(z["pairs"], z["golden_cols"]):
        ia, ib = lookup[int(a)], lookup[int(b)]
        assert mine[(min(ia, ib), max(ia, ib))] == tuple(int(x) for x in r)


@pytest.mark.parametrize("name", SYNTH)
def test_synthetic_vs_reference(name):
    z = load_npz("synth.npz")
    src, dst = mtx_pairs(z[name + "_u"], z[name + "_v"])
    for order, s2l in ORDERS:
        tag = "%s_%s%s" % (name, order, "_s2l" if s2l else "")
        g = ol.OracleGraph.from_pairs(src, dst).run(order=order, s2l=s2l)
        n, m, K = z[tag + "_meta"]
        assert (g.n, g.m, g.max_core) == (n, m, K)
        assert (g.totals() == z[tag + "_totals"]).all(), tag
        s, d, c = _rows(g)
        assert rows_digest(s, d, c) == str(z[tag + "_rows_sha256"]), tag


def test_huge_n_wraps_like_reference():
    z = load_npz("bign.npz")
    src, dst = bign_pairs(z)
    g = ol.OracleGraph.from_pairs(src, dst).run(micro=False)
    assert g.n == int(z["n"]) and g.m == int(z["m"])
    assert (g.totals() == z["totals"]).all()


def _census_ok(n, edges, threads=1):
    if edges:
        src = np.array([e[0] for e in edges], np.int32)
        dst = np.array([e[1] for e in edges], np.int32)
    else:
        src = dst = np.zeros(0, np.int32)
    g = ol.OracleGraph.from_pairs(src, dst, n_min=n).run(micro=False, threads=threads)
    want = brute_force_counts(n, edges)
    got = dict(zip(ol.TOTAL_NAMES, (int(x) for x in g.totals())))
    return got == want, got, want


def test_brute_force_all_graphs_on_five_vertices():
    pairs = list(itertools.combinations(range(5), 2))
    for mask in range(1 << len(pairs)):
        edges = [pairs[i] for i in range(len(pairs)) if mask >> i & 1]
        if not edges:
            continue
        ok, got, want = _census_ok(5, edges)
        assert ok, (edges, got, want)


def test_brute_force_random_graphs():
    rng = np.random.default_rng(11)
    for trial in range(40):
        n = int(rng.integers(6, 12))
        p = float(rng.uniform(0.1, 0.9))
        edges = [(i, j) for i in range(n) for j in range(i + 1, n) if rng.random() < p]
        if not edges:
            continue
        ok, got, want = _census_ok(n, edges)
        assert ok, (n, edges, got, want)


def test_closing_identities_hold():
    """graphlet_core.cpp:1275-1305 checks these relations between the totals
    and the raw sums (dead code in the reference; used here as a check)."""
    z = load_npz("synth.npz")
    src, dst = mtx_pairs(z["rmat12_u"], z["rmat12_v"])
    g = ol.OracleGraph.from_pairs(src, dst).run(micro=False)
    t = dict(zip(ol.TOTAL_NAMES, (int(x) for x in g.totals())))
    s = [int(x) for x in g.sums()]
    N = {i: s[4 + i] for i in range(1, 11)}
    M = (1 << 64) - 1
    assert (t["total_4_chordcycle"] + 6 * t["total_4_clique"]) & M == N[3]
    assert (t["total_4_path"] + 4 * t["total_4_cycle"]) & M == N[5]
    assert (3 * t["total_3_star"] + t["total_4_tailed_tris"]) & M == N[6]
    assert (2 * t["total_4_tailed_tris"] + 4 * t["total_4_chordcycle"]) & M == N[4]
    assert (2 * t["total_4_2edge"] + t["total_4_1edge"]) & M == N[8]


# ---------------------------------------------------------------------------
# live reference (only where it was compiled: oracle/_ref)

needs_ref = pytest.mark.skipif(not ol.ref_available(), reason="reference not compiled here")

EDGE_LIST_CASES = {
    "a.csv": "1,2\n2,3\n3,1\n3,4\n4,5\n5,3\n1,2\n2,2\n",
    "b.txt": "% comment\n1 2\n2 3\n3 1\n3 4\n4 1\n7 8\n8 3\n",
    "c.edges": "0 1\n1 2\n2 0\n2 3\n3 0\n1 3\n",
    "d.tab": "5\t9\n9\t11\n11\t5\n5\t2\n2\t9\n",
    "e.csv": "src,dst,w\n10,20,1\n20,30,1\n30,10,1\n10,40,2\n",
    "f.txt": "# header\n1 2 0.5\n2 3 0.5\n1 3 0.5\n3 4 1.0\n4 5 1\n5 1 1\n",
}


@needs_ref
@pytest.mark.parametrize("fname", sorted(EDGE_LIST_CASES))
def test_reader_rules_vs_reference(tmp_path, fname):
    p = tmp_path / fname
    p.write_text(EDGE_LIST_CASES[fname])
    r = ol.RefGraph.from_file(str(p)).run(micro=True)
    g = ol.OracleGraph.from_file(str(p)).run(micro=True)
    assert (g.n, g.m) == (r.n, r.m)
    assert (g.totals() == r.totals()).all()
    a, b, c = g.micro()
    x, y, z = r.micro()
    assert (a == x).all() and (b == y).all() and (c == z).all()


@needs_ref
@pytest.mark.parametrize("fname", sorted(READER_QUIRKS))
def test_reader_quirks_vs_reference(tmp_path, fname):
    p = tmp_path / fname
    p.write_bytes(READER_QUIRKS[fname].encode())
    r = ol.RefGraph.from_file(str(p)).run(micro=True)
    g = ol.OracleGraph.from_file(str(p)).run(micro=True)
    assert (g.n, g.m) == (r.n, r.m)
    assert (g.totals() == r.totals()).all()
    a, b, c = g.micro()
    x, y, z = r.micro()
    assert (a == x).all() and (b == y).all() and (c == z).all()


@needs_ref
@pytest.mark.parametrize("seed", range(6))
def test_random_graphs_vs_reference(seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(30, 200))
    k = int(rng.integers(n, 6 * n))
    src = rng.integers(0, n, k).astype(np.int32)
    dst = rng.integers(0, n, k).astype(np.int32)
    g = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    off, adj = g.csr()
    order = ["deg", "kcore", "natural", "kcore_deg", "deg_vol", "triangles"][seed]
    r = ol.RefGraph.from_csr(off, adj).run(order=order, micro=True)
    o = ol.OracleGraph.from_csr(off, adj).run(order=order, micro=True)
    assert (o.totals() == r.totals()).all()
    a, b, c = o.micro()
    x, y, z = r.micro()
    assert (a == x).all() and (b == y).all() and (c == z).all()
    assert o.max_core == r.max_core


@needs_ref
@pytest.mark.parametrize("neigh,s2l", [("kcore", False), ("natural", False), ("deg", True)])
def test_neighbour_orders_vs_reference(neigh, s2l):
    z = load_npz("synth.npz")
    src, dst = mtx_pairs(z["ba2000_u"], z["ba2000_v"])
    g = ol.OracleGraph.from_pairs(src, dst)
    off, adj = g.csr()
    r = ol.RefGraph.from_csr(off, adj, neigh=neigh, s2l_neigh=s2l).run(micro=True)
    o = ol.OracleGraph.from_csr(off, adj).run(neigh=neigh, s2l_neigh=s2l, micro=True)
    a, b, c = o.micro()
    x, y, w = r.micro()
    assert (a == x).all() and (b == y).all() and (c == w).all()


def _sample_graph(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(60, 200))
    k = int(rng.integers(3 * n, 8 * n))
    src = rng.integers(0, n, k).astype(np.int32)
    dst = rng.integers(0, n, k).astype(np.int32)
    g = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    return g.csr(), rng


@needs_ref
@pytest.mark.parametrize("order,s2l", [("natural", False), ("deg", False), ("kcore", True), ("deg_vol", False)])
def test_sampled_order_vs_reference(order, s2l):
    """sort_edges with E_s (graphlet_core.cpp:836-851) then the decomposition:
    the oracle's sampled path against the reference's, repeats included."""
    (off, adj), rng = _sample_graph(31)
    m = len(adj) // 2
    ids = rng.integers(0, m, m // 3)
    r = ol.RefGraph.from_csr(off, adj).run_sample(ids, order=order, s2l=s2l, micro=True)
    o = ol.OracleGraph.from_csr(off, adj).run_sample(ids, order=order, s2l=s2l, micro=True)
    assert o.n_ord == len(ids)
    assert (o.totals() == r.totals()).all()
    a, b, c = o.micro()
    x, y, z = r.micro()
    assert (a == x).all() and (b == y).all() and (c == z).all()


def test_sampled_rows_equal_full_rows():
    """A sampled edge's row does not depend on the sample: it equals the
    edge's row in the full decomposition."""
    (off, adj), rng = _sample_graph(32)
    m = len(adj) // 2
    full = ol.OracleGraph.from_csr(off, adj).run(order="natural", micro=True)
    fs, fd, fc = full.micro()
    rows = {(int(a), int(b)): c for a, b, c in zip(fs, fd, fc)}
    ids = rng.choice(m, m // 2, replace=False)
    o = ol.OracleGraph.from_csr(off, adj).run_sample(ids, order="kcore", micro=True)
    s, d, c = o.micro()
    assert len(c) == len(ids)
    for a, b, row in zip(s, d, c):
        assert (rows[(int(a), int(b))] == row).all()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_c4_identity_used_by_the_kernels(seed):
    """The decomposition kernels do not scan S_q x S_p for c4; they use
      c4 = sum_{w in S_q} W(w,p) - |S_q| - sum_{x in T} t(x,q) + 2*k4 + t,
    W(a,b) = |N(a) & N(b)|, t(x,q) = W(x,q) for x in T (k_hub reads W from a
    histogram, k_dense_cn from a common-neighbour matrix).  The identity must
    reproduce the oracle's per-edge c4 (the reference's S_u x S_v count) for
    either choice of p and q, next to its t and k4."""
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(40, 160))
    p_edge = float(rng.uniform(0.05, 0.6))
    iu, ju = np.triu_indices(n, 1)
    keep = rng.random(len(iu)) < p_edge
    src, dst = iu[keep].astype(np.int32), ju[keep].astype(np.int32)
    og = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    og.run(order="deg", micro=True)
    s1, d1, cols = og.micro()
    off, adj = og.csr()
    nn = len(off) - 1
    A = np.zeros((nn, nn), bool)
    for v in range(nn):
        A[v, adj[off[v]:off[v + 1]]] = True
    W = A.astype(np.int64) @ A.astype(np.int64)
    assert len(cols) == og.m > 0
    for (a, b), row in zip(zip(s1 - 1, d1 - 1), cols):
        t, k4, c4 = int(row[0]), int(row[2]), int(row[5])
        T = A[a] & A[b]
        assert T.sum() == t and W[a, b] == t
        for p, q in ((a, b), (b, a)):
            Sq = A[q] & ~A[p]
            Sq[p] = False
            got = int(W[Sq, p].sum()) - int(Sq.sum()) - int(W[T, q].sum()) + 2 * k4 + t
            assert got == c4, (p, q, got, c4)


@pytest.mark.parametrize("seed", range(4))
def test_dense_tensor_core_identities(seed):
    """What the tensor-core kernels of dense batch graphs compute, restated in
    integer numpy and checked against the oracle's per-edge k4 and c4:
      2·k4(p, q) = sum_{y in N(q)} A_py · D[p][y], D = C_q C_q^T over the ego
        network of q compacted to N(q)'s columns (k_dense_tc, for the edges
        (p, q) of q's run);
      c4 = E[q][p] - d_p + 2·k4 + t - |S_q|, E = A·(CN - A∘CN) - (A∘CN)·A,
        CN = A², |S_q| = d_q - t - 1 (k_dense_gram + k_dense_close)."""
    rng = np.random.default_rng(300 + seed)
    n = int(rng.integers(30, 120))
    p_edge = float(rng.uniform(0.1, 0.8))
    iu, ju = np.triu_indices(n, 1)
    keep = rng.random(len(iu)) < p_edge
    src, dst = iu[keep].astype(np.int32), ju[keep].astype(np.int32)
    og = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    og.run(order="kcore", micro=True)
    s1, d1, cols = og.micro()
    off, adj = og.csr()
    nn = len(off) - 1
    A = np.zeros((nn, nn), np.int64)
    for v in range(nn):
        A[v, adj[off[v]:off[v + 1]]] = 1
    deg = A.sum(1)
    CN = A @ A
    TA = A * CN
    E = A @ (CN - TA) - TA @ A
    assert (E == E.T).all()
    assert len(cols) == og.m > 0
    for (a, b), row in zip(zip(s1 - 1, d1 - 1), cols):
        t, k4, c4 = int(row[0]), int(row[2]), int(row[5])
        for p, q in ((a, b), (b, a)):
            nq = np.flatnonzero(A[q])
            C = A[np.ix_(nq, nq)]          # ego network of q, compacted to N(q)'s columns
            j = int(np.searchsorted(nq, p))
            assert (C[j] @ (C @ C[j])) == 2 * k4
            assert CN[p, q] == t
            got = int(E[q, p]) - int(deg[p]) + 2 * k4 + t - (int(deg[q]) - t - 1)
            assert got == c4, (p, q, got, c4)
