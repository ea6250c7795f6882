"""Per-edge rows into page-locked host memory: pgd_get_micro writes them with
one kernel through the device's mapping of the buffers; the rows and ids must
equal the ones the copy path gives (pageable buffers, and a page-locked view
that is not 16-byte aligned)."""
import numpy as np
import pytest

import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu


def test_micro_into_page_locked_memory():
    torch = pytest.importorskip("torch")
    c = pgd.Context()
    s, d = pgd.rmat(14, 8, seed=2)
    g = c.graph_from_edges(s, d)
    g.preprocess("deg")
    g.compute_cores()
    g.sort_edges("kcore")
    g.decompose(micro=True)
    a, b, cols = g.micro()   # pageable buffers: copies
    m = g.order_length
    hc = torch.empty((m, pgd.NMICRO), dtype=torch.int64).pin_memory().numpy().view(np.uint64)
    hs = torch.empty(m, dtype=torch.int64).pin_memory().numpy()
    hd = torch.empty(m, dtype=torch.int64).pin_memory().numpy()
    assert pgd.lib().pgd_get_micro(g.h, pgd._ptr(hs), pgd._ptr(hd), pgd._ptr(hc)) == 0
    assert (hc == cols).all() and (hs == a).all() and (hd == b).all()
    # rows only, and a view 8 bytes into a page-locked buffer (copy path)
    big = torch.empty(m * pgd.NMICRO + 2, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
    off = big[1:1 + m * pgd.NMICRO].reshape(m, pgd.NMICRO)
    assert pgd.lib().pgd_get_micro(g.h, None, None, pgd._ptr(off)) == 0
    assert (off == cols).all()
    g.destroy()
    c.close()


def test_page_locked_pair_inputs():
    """Pairs in page-locked memory are uploaded by a kernel reading through the
    mapping: the same CSR, counts and rows as from pageable arrays, for the
    single-graph intake and for a pairs batch (offset views included)."""
    torch = pytest.importorskip("torch")
    c = pgd.Context()
    s, d = pgd.rmat(13, 8, seed=4)
    ps = torch.from_numpy(np.ascontiguousarray(s)).pin_memory().numpy()
    pd = torch.from_numpy(np.ascontiguousarray(d)).pin_memory().numpy()
    g1 = c.graph_from_edges(s, d)
    g2 = c.graph_from_edges(ps, pd)
    assert (g1.n, g1.m) == (g2.n, g2.m)
    for g in (g1, g2):
        g.preprocess("deg")
        g.compute_cores()
        g.sort_edges("kcore")
    r1, r2 = g1.decompose(micro=True), g2.decompose(micro=True)
    assert (r1.totals == r2.totals).all()
    for a, b in zip(g1.micro(), g2.micro()):
        assert (a == b).all()
    graphs = [pgd.erdos_renyi(300 + 37 * i, 0.1 + 0.05 * i, seed=40 + i) for i in range(6)]
    graphs.append(pgd.barabasi_albert(2000, 3, seed=9))
    off, src, dst = pgd.concat_pairs(graphs)
    want = c.decompose_pairs_batch_flat(off, src, dst)
    psrc = torch.from_numpy(src).pin_memory().numpy()
    pdst = torch.from_numpy(dst).pin_memory().numpy()
    got = c.decompose_pairs_batch_flat(off, psrc, pdst)
    for a, b in zip(want, got):
        assert (a.totals == b.totals).all()
    # one graph from a view into the page-locked arrays (not 16-byte aligned in general)
    i = 3
    one = c.decompose_pairs_batch_flat(np.array([0, off[i + 1] - off[i]], np.int64),
                                       psrc[off[i]:off[i + 1]], pdst[off[i]:off[i + 1]])[0]
    assert (one.totals == want[i].totals).all()
    g1.destroy()
    g2.destroy()
    c.close()
