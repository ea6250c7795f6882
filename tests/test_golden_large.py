"""CPU checks of the full-size fixtures (tests/golden/rmat20_kcore.json,
rgg20_kcore.json) and of the input generators they rest on.

The fixtures hold the oracle's full per-edge loop on the two graphs.  Here
their sampled rows are re-derived by a second procedure of the oracle (the
reference's marking procedure run on each sampled edge alone, then the micro
stores), their totals by the closing identities from their raw sums, and
their input by the generators."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd
from helpers import GOLDEN


def load(name):
    return json.load(open(os.path.join(GOLDEN, name + ".json")))


def test_oracle_rmat_matches_product_generator():
    for scale, seed in ((10, 1), (14, 3), (16, 1)):
        a = ol.rmat(scale, 16, seed=seed)
        b = pgd.rmat(scale, 16, seed=seed)
        assert (a[0] == b[0]).all() and (a[1] == b[1]).all()


@pytest.mark.parametrize("name", ["rmat20_kcore", "rgg20_kcore"])
def test_large_fixture_is_consistent(name):
    gold = load(name)
    case = gold["case"]
    if case["kind"] == "rmat":
        src, dst = ol.rmat(case["scale"], case["edge_factor"], seed=case["seed"], a=case["a"], b=case["b"],
                           c=case["c"])
    else:
        n = case["n"]
        r = (3.0 * case["mean_degree"] / (4.0 * np.pi * n)) ** (1.0 / 3.0)
        src, dst = pgd.rgg3d(n, r, seed=case["seed"])
    digest = hashlib.sha256(np.ascontiguousarray(src, "<i4").tobytes() +
                            np.ascontiguousarray(dst, "<i4").tobytes()).hexdigest()
    assert digest == gold["pairs_sha256"]
    # totals from the raw sums by the closing identities
    tot = ol.close(np.array(gold["sums"], np.uint64), gold["n"], gold["m"])
    assert {k: int(v) for k, v in zip(ol.TOTAL_NAMES, tot)} == gold["totals"]
    # sampled rows by the marking procedure on each edge alone
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    assert (o.n, o.m) == (gold["n"], gold["m"])
    rows = np.array(gold["sample_rows"], dtype=np.uint64)
    v = rows[:, 0].astype(np.int64) - 1
    u = rows[:, 1].astype(np.int64) - 1
    t, k4, c4 = o.edge_sample(v, u)
    off, _ = o.csr()
    deg = np.diff(off)
    want = ol.micro_rows(deg[v], deg[u], t, k4, c4)
    assert (want == rows[:, 2:]).all()
