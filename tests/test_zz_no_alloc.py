"""The allocation-free entry point, pgd_decompose_csr_noalloc.

It exists for callers that cannot allocate device memory when they need
counts: a plugin handed a fixed device workspace by a host framework whose
memory manager forbids allocation, or a latency-critical loop where
cudaMalloc/cudaFree would synchronise the device.  This test calls it through
the C ABI on device CSRs held by torch, several times in a row on different
graphs and once more on the first, and checks every global count against the
regular entry point, pgd_decompose, and against the oracle, exactly (integer
counts: tolerance zero).  One graph has more than 16,384 vertices, so the
k4 membership test beyond the per-warp rank bitmap, which this entry point
does by searching N(q), runs.  It also checks that an oversized graph and
malformed CSRs are refused.  This file is collected last so a failure here
leaves every other test run.
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
    graphs = [pgd.rmat(12, 16, seed=5), pgd.erdos_renyi(300, 0.4, seed=2), pgd.barabasi_albert(3000, 6, seed=4),
              pgd.barabasi_albert(40000, 3, seed=9)]
    nmax = 0
    for i, (src, dst) in enumerate(graphs + graphs[:1]):
        off, adj = _sorted_csr(src, dst)
        nmax = max(nmax, len(off) - 1)
        st, out, msg = _noalloc(torch, off, adj, stream)
        assert st == 0, msg
        got = np.array(list(out.totals), dtype=np.uint64)
        g = ctx.graph_from_csr(off, adj)
        want = g.decompose(micro=False)
        g.destroy()
        assert (got == want.totals).all(), (i, got, want.totals)
        assert (np.array(list(out.sums), dtype=np.uint64) == want.sums).all()
        assert (out.n, out.m) == (want.n, want.m)
        o = ol.OracleGraph.from_csr(off, adj).run(micro=False)
        assert (got == o.totals()).all(), (i, got, o.totals())
        assert (np.array(list(out.sums), dtype=np.uint64) == o.sums()).all()
    assert nmax > 16384
    ctx.close()


def test_noalloc_rejects_malformed_csr():
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    # a 5-cycle 0-1-2-3-4-0, rows sorted
    off = np.array([0, 2, 4, 6, 8, 10], np.int64)
    adj = np.array([1, 4, 0, 2, 1, 3, 2, 4, 0, 3], np.int32)
    st, out, msg = _noalloc(torch, off, adj, stream)
    assert st == 0, msg
    assert out.m == 5 and out.totals[9] == 0   # no induced 4-cycle in a 5-cycle
    unsorted = adj.copy()
    unsorted[[0, 1]] = unsorted[[1, 0]]
    asym = adj.copy()
    asym[1] = 3                                 # 0-3 without 3-0
    bad_first = off.copy()
    bad_first[0] = 1
    decreasing = off.copy()
    decreasing[2] = 1
    cases = [(off, unsorted, "rows must be sorted"), (off, asym, "rows must be sorted"),
             (bad_first, adj, "offsets"), (decreasing, adj, "offsets")]
    for o_, a_, text in cases:
        st, _, msg = _noalloc(torch, o_, a_, stream)
        assert st == 1 and "device CSR rejected" in msg and text in msg, (st, msg)
    # a valid call right after the refusals still gives the right counts
    st, out, msg = _noalloc(torch, off, adj, stream)
    assert st == 0 and out.m == 5, msg


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
