"""4-cliques of dense batch graphs on the tensor cores (k_dense_tc): for the
runs of edges sharing q whose degree lies in [tensor_min_degree, 1088], k4
comes from an e4m3 product of q's ego network accumulated in TMEM.  Counts
must not depend on which runs take that path: every per-edge row and total
equals the integer path's (tensor_min_degree 0), the single-graph kernels',
an independent numpy count of k4, and the oracle's on the smaller graphs."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu

# d_q across the path's limits: below and above 128 (default threshold),
# runs of more than 128 edges (several M tiles), d_q above 256 (several N
# tiles), d_q not a multiple of 16 or 64, and d_q around 1088 (the largest
# ego network the kernel keeps in shared memory) in (1230, 0.885)
SPECS = [(1230, 0.885), (2048, 0.5), (600, 0.5), (257, 0.99), (1200, 0.11), (160, 0.85), (900, 0.3),
         (40, 0.9), (2000, 0.07)]


def k4_numpy(ev, eu, n):
    """k4 of every edge (v, u) = edges inside N(v) ∩ N(u), from dense matrix
    products of each vertex's ego network."""
    A = np.zeros((n, n), np.float32)
    A[ev, eu] = 1
    A[eu, ev] = 1
    k4 = {}
    for q in range(n):
        nq = np.flatnonzero(A[q])
        if len(nq) == 0:
            continue
        B = A[np.ix_(nq, nq)]
        s = ((B @ B) * B).sum(1)
        for p, v in zip(nq, s):
            k4[(int(min(p, q)), int(max(p, q)))] = int(round(v)) // 2
    return k4


def batch_rows(c, graphs):
    res = c.decompose_batch(graphs, micro=True)
    return res, [g.micro() for g in graphs]


def test_tensor_k4_equals_integer_path_and_single_graph():
    c = pgd.Context()
    pairs = [pgd.erdos_renyi(n, p, seed=300 + i) for i, (n, p) in enumerate(SPECS)]
    pairs.append(pgd.barabasi_albert(700, 4, seed=9))
    graphs = [c.graph_from_edges(s, d) for s, d in pairs]
    for g in graphs:
        g.preprocess("deg")
        g.sort_edges("kcore")
    degs = [g.info().max_degree for g in graphs]
    assert max(degs) > 1088 and any(128 <= d <= 1088 for d in degs)
    c.set_tensor_min_degree(0)
    assert c.tensor_min_degree() == 0
    base, base_rows = batch_rows(c, graphs)
    for tmin in (2, 128, 1088):
        c.set_tensor_min_degree(tmin)
        res, rows = batch_rows(c, graphs)
        for i in range(len(graphs)):
            assert (res[i].totals == base[i].totals).all(), (tmin, i)
            assert (res[i].sums == base[i].sums).all(), (tmin, i)
            for a, b in zip(rows[i], base_rows[i]):
                assert (a == b).all(), (tmin, i)
    c.set_tensor_min_degree(128)
    for i, g in enumerate(graphs):
        single = g.decompose(micro=True)
        assert (single.totals == base[i].totals).all(), i
        for a, b in zip(g.micro(), base_rows[i]):
            assert (a == b).all(), i
    # the pairs batch (device CSR build of the union) with the tensor path
    pr = c.decompose_pairs_batch(pairs)
    for i, r in enumerate(pr):
        assert (r.totals == base[i].totals).all(), i
    c.close()


@pytest.mark.parametrize("n,p,seed", [(600, 0.5, 11), (257, 0.99, 12), (1100, 0.2, 13)])
def test_tensor_k4_equals_numpy(n, p, seed):
    c = pgd.Context()
    c.set_tensor_min_degree(2)
    s, d = pgd.erdos_renyi(n, p, seed=seed)
    g = c.graph_from_edges(s, d)
    g.preprocess("deg")
    g.sort_edges("kcore")
    c.decompose_batch([g], micro=True)
    _, _, cols = g.micro()
    ev, eu, order = g.edges()
    k4 = k4_numpy(ev, eu, g.n)
    want = np.array([k4[(int(min(ev[e], eu[e])), int(max(ev[e], eu[e])))] for e in order], np.uint64)
    assert (cols[:, 2] == want).all()
    c.close()


@pytest.mark.parametrize("n,p,seed", [(160, 0.85, 21), (257, 0.99, 22)])
def test_tensor_k4_oracle(n, p, seed):
    c = pgd.Context()
    c.set_tensor_min_degree(2)
    s, d = pgd.erdos_renyi(n, p, seed=seed)
    g = c.graph_from_edges(s, d)
    g.preprocess("deg")
    g.sort_edges("kcore")
    r = c.decompose_batch([g], micro=True)[0]
    o = ol.OracleGraph.from_pairs(s, d, dedup=True).run(order="kcore")
    assert (r.totals == o.totals()).all()
    a, b, cols = g.micro()
    x, y, z = o.micro()
    assert (a == x).all() and (b == y).all() and (cols == z).all()
    c.close()


def test_tensor_min_degree_range():
    c = pgd.Context()
    for bad in (1, -1, 1089):
        with pytest.raises(pgd.PGDError) as e:
            c.set_tensor_min_degree(bad)
        assert e.value.status == 1
    c.set_tensor_min_degree(1088)
    assert c.tensor_min_degree() == 1088
    c.close()
