"""Batched decomposition from host pair lists and the continuous-batching
request server: every request's counts equal the oracle's for that graph
alone, under concurrency, memory refusal and timeouts."""
import threading

import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

pytestmark = pytest.mark.gpu


def request_mix(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = i % 5
        if kind == 0:
            out.append(pgd.rmat(int(rng.integers(5, 11)), 8, seed=seed * 100 + i))
        elif kind == 1:
            out.append(pgd.erdos_renyi(int(rng.integers(10, 300)), float(rng.uniform(0.02, 0.5)), seed=seed * 100 + i))
        elif kind == 2:
            out.append(pgd.barabasi_albert(int(rng.integers(10, 1500)), int(rng.integers(2, 8)), seed=seed * 100 + i))
        elif kind == 3:
            n = int(rng.integers(2, 80))
            k = int(rng.integers(0, 4 * n))
            out.append((rng.integers(0, n, k).astype(np.int32), rng.integers(0, n, k).astype(np.int32)))
        else:
            out.append((np.zeros(0, np.int32), np.zeros(0, np.int32)))
    return out


def oracle_totals(s, d, n_min=0):
    return ol.OracleGraph.from_pairs(s, d, n_min=n_min, dedup=True).run(micro=False).totals()


@pytest.mark.parametrize("dense_max", [0, 2048])
def test_pairs_batch_matches_oracle(dense_max):
    ctx = pgd.Context()
    ctx.set_thresholds(128, 64, dense_max)
    graphs = request_mix(60, 3)
    n_min = [0] * len(graphs)
    n_min[3] = 500  # isolated vertices count in n
    res = ctx.decompose_pairs_batch(graphs, n_min=n_min)
    for i, ((s, d), r) in enumerate(zip(graphs, res)):
        assert (r.totals == oracle_totals(s, d, n_min[i])).all(), i
    ctx.close()


def test_server_results_and_stats():
    sv = pgd.Server(workers=2)
    graphs = request_mix(80, 5)
    tickets = [None] * len(graphs)

    def submit(lo, hi):
        for i in range(lo, hi):
            tickets[i] = sv.submit(*graphs[i])

    threads = [threading.Thread(target=submit, args=(j * 20, (j + 1) * 20)) for j in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i, tk in enumerate(tickets):
        st, r = sv.wait(tk, 120000)
        assert st == 0
        assert (r.totals == oracle_totals(*graphs[i])).all(), i
    s = sv.stats()
    assert s["completed"] == len(graphs) and s["rejected"] == 0
    assert s["batches"] >= 1 and s["p99_ms"] >= s["p50_ms"] > 0 and s["graphs_per_s"] > 0
    sv.close()


def test_server_refuses_what_cannot_fit():
    sv = pgd.Server(workers=1, hbm_budget=4 << 20)
    big = pgd.rmat(14, 16, seed=1)           # estimate far above 4 MiB
    small = pgd.erdos_renyi(40, 0.3, seed=2)
    tb = sv.submit(*big)
    ts = sv.submit(*small)
    st, _ = sv.wait(tb, 60000)
    assert st == 2  # PGD_ENOMEM
    st, r = sv.wait(ts, 60000)
    assert st == 0 and (r.totals == oracle_totals(*small)).all()
    assert sv.stats()["rejected"] == 1
    sv.close()


def test_server_poll_and_timeout():
    sv = pgd.Server(workers=1)
    s, d = pgd.rmat(12, 16, seed=9)
    t = sv.submit(s, d)
    st, _ = sv.wait(t, 0)
    assert st in (0, 3)  # done already, or PGD_ETIMEOUT with the request still running
    if st == 3:
        got = None
        for _ in range(10000):
            got = sv.poll(t)
            if got is not None:
                break
            threading.Event().wait(0.005)
        assert got is not None and got[0] == 0
        assert (got[1].totals == oracle_totals(s, d)).all()
    sv.close()


def test_server_admits_small_requests_past_a_large_one():
    """A request that does not fit the memory left is passed by later, smaller
    ones (until it has waited max_wait_ms); every result stays exact."""
    big1 = pgd.rmat(16, 16, seed=11)
    big2 = pgd.rmat(16, 16, seed=12)
    smalls = [pgd.erdos_renyi(40, 0.3, seed=20 + i) for i in range(40)]
    # two large requests cannot be in flight together under this budget
    sv = pgd.Server(workers=2, hbm_budget=300 << 20, max_wait_ms=60000)
    t1 = sv.submit(*big1)
    t2 = sv.submit(*big2)
    ts = [sv.submit(*g) for g in smalls]
    for tk, g in zip([t1, t2] + ts, [big1, big2] + smalls):
        st, r = sv.wait(tk, 120000)
        assert st == 0 and (r.totals == oracle_totals(*g)).all()
    s = sv.stats()
    assert s["completed"] == 42 and s["skipped_ahead"] >= 1
    assert s["queue_p50_ms"] <= s["queue_p99_ms"] and s["service_p50_ms"] <= s["service_p99_ms"]
    assert s["p99_ms"] >= s["p50_ms"] > 0
    sv.close()


def test_server_dense_requests_on_both_workers():
    """Dense requests take the tensor-core kernels inside the server's batches,
    on both workers' streams at once: every result equals the single-graph
    kernels' (which never use the tensor cores) and, for the smaller graphs,
    the oracle's."""
    rng = np.random.default_rng(11)
    graphs = []
    for i in range(24):
        n = int(rng.integers(150, 900)) if i % 3 else int(rng.integers(40, 120))
        graphs.append(pgd.erdos_renyi(n, float(rng.uniform(0.3, 0.8)), seed=700 + i))
    ctx = pgd.Context()
    want = []
    for s, d in graphs:
        g = ctx.graph_from_edges(s, d)
        want.append(g.decompose(micro=False).totals)
        g.destroy()
    ctx.close()
    sv = pgd.Server(workers=2)
    tickets = [sv.submit(s, d) for s, d in graphs]
    for i, tk in enumerate(tickets):
        st, r = sv.wait(tk, 120000)
        assert st == 0
        assert (r.totals == want[i]).all(), i
        if i % 3 == 0:
            assert (r.totals == oracle_totals(*graphs[i])).all(), i
    assert sv.stats()["completed"] == len(graphs)
    sv.close()
