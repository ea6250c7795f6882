"""Full-size pins: the RMAT scale-20 graph in k-core order (the benchmark's
workload) and the 3-D random geometric graphs with n = 2^20 and n = 2^24
(200 M edges), decomposed on the GPU and compared bit for bit with the
oracle's full runs (every per-edge row,
in E_ordered order, through its SHA-256; the 17 totals; the 15 raw sums).
The fixtures come from tests/golden/make_large_golden.py."""
import json
import os

import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd
from helpers import GOLDEN, rows_digest

pytestmark = pytest.mark.gpu


def load(name):
    return json.load(open(os.path.join(GOLDEN, name + ".json")))


def pairs_of(case):
    if case["kind"] == "rmat":
        return ol.rmat(case["scale"], case["edge_factor"], seed=case["seed"], a=case["a"], b=case["b"], c=case["c"])
    n = case["n"]
    r = (3.0 * case["mean_degree"] / (4.0 * np.pi * n)) ** (1.0 / 3.0)
    return pgd.rgg3d(n, r, seed=case["seed"])


@pytest.mark.parametrize("name", ["rmat20_kcore", "rgg20_kcore", "rgg24_kcore"])
def test_full_graph_bit_exact(ctx, name):
    gold = load(name)
    src, dst = pairs_of(gold["case"])
    g = ctx.graph_from_edges(src, dst, dedup=True)
    g.preprocess("deg")
    K = g.compute_cores()
    g.sort_edges(gold["case"]["order"])
    res = g.decompose(micro=True)
    assert (int(res.n), int(res.m), int(K)) == (gold["n"], gold["m"], gold["K"])
    assert {k: int(v) for k, v in zip(pgd.TOTAL_NAMES, res.totals)} == gold["totals"]
    assert [int(x) for x in res.sums] == gold["sums"]
    s1, d1, cols = g.micro()
    assert [int(x) for x in cols.sum(axis=0, dtype=np.uint64)] == gold["col_sums"]
    pos = np.array(gold["sample_pos"])
    want = np.array(gold["sample_rows"], dtype=np.uint64)
    got = np.concatenate([s1[pos, None].astype(np.uint64), d1[pos, None].astype(np.uint64), cols[pos]], axis=1)
    assert (got == want).all()
    assert rows_digest(s1, d1, cols) == gold["rows_sha256"]
    g.destroy()
