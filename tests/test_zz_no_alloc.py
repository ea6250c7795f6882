"""The allocation-free entry point, pgd_decompose_csr_noalloc.

It exists for callers that cannot allocate device memory when they need
counts (a fixed workspace handed out by a host framework, a CUDA stream
capture, a loop where cudaMalloc would synchronise the device).  This test
calls it through the C ABI on device CSRs held by torch, twice in a row on
different graphs and once more on the first, and checks every global count
against the regular entry point, pgd_decompose, exactly (integer counts:
tolerance zero).  It also checks that an oversized graph is refused.  This
file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu


def _sorted_csr(src, dst):
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    off, adj = o.csr()
    adj = adj.copy()
    for v in range(len(off) - 1):
        adj[off[v]:off[v + 1]].sort()
    return off.astype(np.int64), adj.astype(np.int32)


def _noalloc(torch, off, adj, stream):
    d_off = torch.from_numpy(off).cuda()
    d_adj = torch.from_numpy(adj if len(adj) else np.zeros(1, np.int32)).cuda()
    torch.cuda.synchronize()
    out = pgd.pgd_counts()
    err = ctypes.create_string_buffer(512)
    st = pgd.lib().pgd_decompose_csr_noalloc(ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_adj.data_ptr()),
                                             len(off) - 1, len(adj), torch.cuda.current_device(),
                                             ctypes.c_void_p(stream.cuda_stream), ctypes.byref(out), err, 512)
    return st, out, err.value.decode()


def test_noalloc_matches_decompose_twice_in_a_row():
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    ctx = pgd.Context(stream=stream.cuda_stream)
    graphs = [pgd.rmat(12, 16, seed=5), pgd.erdos_renyi(300, 0.4, seed=2), pgd.barabasi_albert(3000, 6, seed=4)]
    for i, (src, dst) in enumerate(graphs + graphs[:1]):
        off, adj = _sorted_csr(src, dst)
        st, out, msg = _noalloc(torch, off, adj, stream)
        assert st == 0, msg
        want = ctx.graph_from_csr(off, adj).decompose(micro=False)
        got = np.array(list(out.totals), dtype=np.uint64)
        assert (got == want.totals).all(), (i, got, want.totals)
        assert (np.array(list(out.sums), dtype=np.uint64) == want.sums).all()
        assert (out.n, out.m) == (want.n, want.m)
    ctx.close()


def test_noalloc_refuses_oversized_graph():
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    limit = pgd.lib().pgd_noalloc_scratch_bytes()
    assert limit == 64 << 20
    # a path 0-1-...-(n-1) whose scratch needs exceed the limit
    n = int(limit // 40) + 10
    deg = np.full(n, 2, np.int64)
    deg[0] = deg[-1] = 1
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int64)
    adj = np.empty(off[-1], np.int32)
    adj[0] = 1
    mid = np.arange(1, n - 1)
    adj[off[mid]] = mid - 1
    adj[off[mid] + 1] = mid + 1
    adj[off[n - 1]] = n - 2
    st, out, msg = _noalloc(torch, off, adj, stream)
    assert st == 2 and "scratch" in msg
