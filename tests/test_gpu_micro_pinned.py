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
