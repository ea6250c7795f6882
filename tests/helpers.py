"""Shared helpers for the tests: fixtures loading, brute-force census, digests."""
import hashlib
import itertools
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_toys():
    return json.load(open(os.path.join(GOLDEN, "toy.json")))


def load_npz(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def rows_digest(src, dst, cols, chunk=1 << 20):
    """SHA-256 of the rows (src, dst, 8 columns) as little-endian uint64,
    hashed a chunk of rows at a time (the same digest as one pass over the
    whole table, without building it)."""
    h = hashlib.sha256()
    for i in range(0, len(cols), chunk):
        rows = np.concatenate([np.asarray(src[i:i + chunk], np.uint64)[:, None],
                               np.asarray(dst[i:i + chunk], np.uint64)[:, None],
                               np.asarray(cols[i:i + chunk], np.uint64)], axis=1)
        h.update(np.ascontiguousarray(rows, "<u8").tobytes())
    return h.hexdigest()


def mtx_pairs(u, v):
    """The pair sequence a reader sees for an mtx file that lists (max+1, min+1)
    per line in the given order: 0-based (larger, smaller)."""
    u = np.asarray(u, np.int32)
    v = np.asarray(v, np.int32)
    return np.maximum(u, v), np.minimum(u, v)


def bign_pairs(z):
    n = int(z["n_path"])
    extra = z["extra"].astype(np.int64)
    i = np.arange(0, n - 1, dtype=np.int64)
    src = np.concatenate([i + 1, extra + 1]).astype(np.int32)
    dst = np.concatenate([i, extra - 1]).astype(np.int32)
    return src, dst


def write_pairs_mtx(path, src, dst):
    n = int(max(src.max(), dst.max())) + 1 if len(src) else 0
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, len(src)))
        np.savetxt(f, np.stack([np.asarray(src) + 1, np.asarray(dst) + 1], 1), fmt="%d")


# Brute-force census of the 4-node graphlets (pure Python; tiny graphs only).
# Classes by (edge count, sorted degree sequence) of the induced subgraph.
_FOUR = {
    (6, (3, 3, 3, 3)): "total_4_clique",
    (5, (2, 2, 3, 3)): "total_4_chordcycle",
    (4, (1, 2, 2, 3)): "total_4_tailed_tris",
    (4, (2, 2, 2, 2)): "total_4_cycle",
    (3, (1, 1, 1, 3)): "total_3_star",
    (3, (1, 1, 2, 2)): "total_4_path",
    (3, (0, 2, 2, 2)): "total_4_tri",
    (2, (0, 1, 1, 2)): "total_4_2star",
    (2, (1, 1, 1, 1)): "total_4_2edge",
    (1, (0, 0, 1, 1)): "total_4_1edge",
    (0, (0, 0, 0, 0)): "total_4_indep",
}


def brute_force_counts(n, edges):
    adj = [set() for _ in range(n)]
    for a, b in edges:
        adj[a].add(b)
        adj[b].add(a)
    out = {k: 0 for k in _FOUR.values()}
    for q in itertools.combinations(range(n), 4):
        deg = [sum(1 for y in q if y in adj[x]) for x in q]
        ne = sum(deg) // 2
        out[_FOUR[(ne, tuple(sorted(deg)))]] += 1
    three = {"total_3_tris": 0, "total_2_star": 0, "total_3_1edge": 0, "total_3_indep": 0}
    for q in itertools.combinations(range(n), 3):
        ne = sum(1 for x, y in itertools.combinations(q, 2) if y in adj[x])
        three[["total_3_indep", "total_3_1edge", "total_2_star", "total_3_tris"][ne]] += 1
    out.update(three)
    m = len(set(tuple(sorted(e)) for e in edges))
    out["total_2_1edge"] = m
    out["total_2_indep"] = n * (n - 1) // 2 - m
    return out


# Reader quirks: files whose ids, delimiters, line endings, comments and
# missing fields exercise the reference reader's rules (graphlet_core.cpp:
# 196-241 tokens, 291-457 edge lists, 459-522 mtx).  Each was run through the
# reference's own ./pgd (built from source) without a crash or a hang.
READER_QUIRKS = {
    "crlf.txt": "1 2\r\n2 3\r\n3 1\r\n3 4\r\n",
    "three_spaces.txt": "1   2\n2   3\n3   1\n1   4\n",
    "banner.txt": "%%MatrixMarket matrix coordinate pattern symmetric\n% c\n4 4 3\n1 2\n2 3\n3 1\n",
    "comments_between.txt": "1 2\n\n# mid\n2 3\n% x\n3 1\n\n",
    "no_final_newline.txt": "1 2\n2 3\n3 1",
    "missing_first_id.txt": "0 1\n 2\n1 2\n2 0\n3 4\n",
    "single_token.txt": "1 2\n5\n2 3\n3 1\n",
    "trailing_junk.csv": "1,2\n2,3\n3,1x\n4,1\n",
    "leading_spaces.txt": "  1 2\n2 3\n3 1\n",
    "zero_late.edges": "1 2\n2 3\n0 1\n3 0\n",
    "empty_first_line.txt": "% c\n\n1 2\n2 3\n3 1\n",
    "header_and_empty_field.csv": "a,b\n1,2\n2,3\n,4\n3,1\n",
    "empty_middle_field.tab": "1\t2\t9\n2\t3\t9\n3\t\t9\n3\t1\t9\n",
    "comments.mtx": "%%MatrixMarket matrix coordinate pattern symmetric\n% comment\n5 5 4\n2 1\n3 2\n% mid\n3 1\n5 4\n",
    "zero_size_line.mtx": "0 0 0\n1 2\n",
    "missing_second_id.mtx": "6 6 4\n3 2\n5 \n6 1\n4 2\n",
    "single_id.mtx": "6 6 4\n2 3\n5\n6 1\n",
    "crlf.mtx": "3 3 2\r\n2 1\r\n3 2\r\n",
    "self_loop_no_final_newline.mtx": "3 3 3\n1 1\n2 1\n3 2",
}

# Files on which the reference indexes its relabel table out of bounds (an id
# carried over from the previous line, already relabelled, then decremented
# to -1): undefined there, refused with PGD_EINVAL here and by the oracle.
READER_REFUSED = {
    "carried_id_below_zero.txt": "1 2\n 3\n2 3\n4 5\n3 1\n",
    "negative_id.txt": "1 2\n2 -3\n",
}
