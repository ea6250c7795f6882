"""Full-size fixtures for the large benchmark graphs, made by the oracle.

The reference itself needs hours for these graphs (RMAT scale 20 in k-core
order: about 6.7 h on 8 cores), so the fixture comes from the oracle
(oracle/pgd_oracle.c), whose parity with the reference is pinned by
tests/test_oracle.py on every graph the reference finishes, including the
reference's RMAT-18 totals.  One run of the oracle's full per-edge loop per
graph, all host threads (about 20 minutes for RMAT-20 and 6 for the 3-D RGG
with n = 2^24 on 8 cores; the latter needs about 45 GB of host memory).

Writes, per graph, tests/golden/<name>.json:
  generator arguments and the SHA-256 of the raw input pairs,
  n, m, K (max core), the 17 totals and the 15 raw sums,
  the SHA-256 of the ordered per-edge rows (src+1, dst+1 and the 8 columns,
  little-endian uint64, in E_ordered order: the `-m` file's rows),
  the wrapped uint64 sum of every per-edge column,
  and 256 rows in full (the first 64 positions and 192 seeded random ones),
  so that a digest mismatch can be localised.

Run:  python tests/golden/make_large_golden.py [rmat20_kcore] [rgg20_kcore] [rgg24_kcore]
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)

import oracle_lib as ol  # noqa: E402
from helpers import rows_digest  # noqa: E402


def rgg_radius(n, mean_degree=24):
    return (3.0 * mean_degree / (4.0 * np.pi * n)) ** (1.0 / 3.0)


CASES = {
    "rmat20_kcore": {"kind": "rmat", "scale": 20, "edge_factor": 16, "a": 0.57, "b": 0.19, "c": 0.19, "seed": 1,
                     "order": "kcore"},
    "rgg20_kcore": {"kind": "rgg3d", "n": 1 << 20, "mean_degree": 24, "seed": 1, "order": "kcore"},
    "rgg24_kcore": {"kind": "rgg3d", "n": 1 << 24, "mean_degree": 24, "seed": 1, "order": "kcore"},
}


def make_pairs(case):
    """The case's raw input pairs (before symmetrising and dedup)."""
    if case["kind"] == "rmat":
        return ol.rmat(case["scale"], case["edge_factor"], seed=case["seed"], a=case["a"], b=case["b"], c=case["c"])
    import pgd_gb300 as pgd  # the RGG generator is host code of the product library

    return pgd.rgg3d(case["n"], rgg_radius(case["n"], case["mean_degree"]), seed=case["seed"])


def pairs_digest(src, dst):
    return hashlib.sha256(np.ascontiguousarray(src, "<i4").tobytes() +
                          np.ascontiguousarray(dst, "<i4").tobytes()).hexdigest()


def sample_positions(m, seed=20):
    rng = np.random.default_rng(seed)
    head = np.arange(min(64, m))
    rest = rng.choice(m, size=min(192, m), replace=False)
    return np.unique(np.concatenate([head, rest]))


def make(name):
    case = CASES[name]
    t0 = time.time()
    src, dst = make_pairs(case)
    o = ol.OracleGraph.from_pairs(src, dst, dedup=True)
    o.run(order=case["order"], micro=True, cheap_side=True)
    s1, d1, cols = o.micro()
    pos = sample_positions(len(cols))
    out = {
        "case": case,
        "made_by": "oracle/pgd_oracle.c (po_decompose, full per-edge loop, micro rows)",
        "pairs_sha256": pairs_digest(src, dst),
        "n": int(o.n), "m": int(o.m), "K": int(o.max_core),
        "totals": {k: int(v) for k, v in zip(ol.TOTAL_NAMES, o.totals())},
        "sums": [int(x) for x in o.sums()],
        "rows_sha256": rows_digest(s1, d1, cols),
        "col_sums": [int(x) for x in cols.sum(axis=0, dtype=np.uint64)],
        "sample_pos": [int(p) for p in pos],
        "sample_rows": [[int(s1[p]), int(d1[p])] + [int(x) for x in cols[p]] for p in pos],
        "seconds": round(time.time() - t0, 1),
    }
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(out, f, indent=1)
    print("%s: n=%d m=%d K=%d in %.0f s" % (name, out["n"], out["m"], out["K"], out["seconds"]), flush=True)


if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        make(name)
