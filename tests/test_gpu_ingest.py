"""Graph files parsed on the device (pgd_graph_from_file) against the oracle's
restatement of the reference reader: the reader's quirks (delimiters, line
endings, comments, 0/1-based ids, missing fields, mtx size lines), seeded
larger files in varied formats, and the refusals."""
import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd
from helpers import READER_QUIRKS, READER_REFUSED

pytestmark = pytest.mark.gpu


def same_as_oracle(ctx, path, orders=("deg", "kcore")):
    """n, m, the edge arrays (which fix the relabelled ids and the insertion
    order), totals and per-edge rows equal the oracle's."""
    o = ol.OracleGraph.from_file(path)
    g = ctx.graph_from_file(path)
    assert (g.n, g.m) == (o.n, o.m)
    for order in orders:
        o = ol.OracleGraph.from_file(path).run(order=order, micro=True)
        g.preprocess("deg")
        ev, eu, _ = g.edges(with_order=False)
        oev, oeu = o.edges()
        assert (ev == oev).all() and (eu == oeu).all()
        g.compute_cores()
        g.sort_edges(order)
        res = g.decompose(micro=True)
        assert (res.totals == o.totals()).all()
        s, d, c = g.micro()
        x, y, z = o.micro()
        assert (s == x).all() and (d == y).all() and (c == z).all()
    g.destroy()


@pytest.mark.parametrize("fname", sorted(READER_QUIRKS))
def test_reader_quirks_on_device(ctx, tmp_path, fname):
    p = tmp_path / fname
    p.write_bytes(READER_QUIRKS[fname].encode())
    same_as_oracle(ctx, str(p))


@pytest.mark.parametrize("fname", sorted(READER_REFUSED))
def test_reader_refusals_on_device(ctx, tmp_path, fname):
    p = tmp_path / fname
    p.write_bytes(READER_REFUSED[fname].encode())
    with pytest.raises(ValueError):
        ol.OracleGraph.from_file(str(p))
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_file(str(p))
    assert e.value.status == 1


def test_missing_file_and_repeated_mtx_edge(ctx, tmp_path):
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_file(str(tmp_path / "absent.txt"))
    assert e.value.status == 5
    p = tmp_path / "twice.mtx"
    p.write_text("3 3 3\n2 1\n3 2\n2 1\n")
    with pytest.raises(pgd.PGDError) as e:
        ctx.graph_from_file(str(p))
    assert e.value.status == 1 and "twice" in str(e.value)


def write_variant(path, src, dst, style, rng):
    """The pairs in one of several textual forms the reader accepts."""
    lines = []
    if style == "csv_weights":
        lines.append("source,target,weight")
        lines += ["%d,%d,%.3f" % (a, b, rng.random()) for a, b in zip(src, dst)]
    elif style == "tabs_comments_crlf":
        lines.append("# tab separated")
        for i, (a, b) in enumerate(zip(src, dst)):
            if i % 97 == 0:
                lines.append("% a comment")
            lines.append("%d\t%d" % (a, b))
        text = "\r\n".join(lines)
        path.write_bytes(text.encode())
        return
    elif style == "zero_based_spaces":
        lines += ["%d %d" % (a - 1, b - 1) for a, b in zip(src, dst)]
    elif style == "mtx":
        lines.append("%%MatrixMarket matrix coordinate pattern symmetric")
        n = int(max(src.max(), dst.max()))
        lines.append("%d %d %d" % (n, n, len(src)))
        lines += ["%d %d" % (max(a, b), min(a, b)) for a, b in zip(src, dst)]
    path.write_text("\n".join(lines) + "\n")


@pytest.mark.parametrize("style", ["csv_weights", "tabs_comments_crlf", "zero_based_spaces", "mtx"])
def test_seeded_files_on_device(ctx, tmp_path, style):
    rng = np.random.default_rng(7)
    s, d = pgd.rmat(11, 8, seed=3)
    keep = s != d
    u = np.minimum(s, d)[keep].astype(np.int64)
    v = np.maximum(s, d)[keep].astype(np.int64)
    key = np.unique(u * (1 << 32) + v)
    order = rng.permutation(len(key))          # file order is not id order
    a = (key[order] >> 32) + 1
    b = (key[order] & 0xFFFFFFFF) + 1
    if style != "mtx":                          # edge lists may repeat a pair
        a = np.concatenate([a, b[:50]])
        b = np.concatenate([b, a[:50]])
    p = tmp_path / ("g." + {"csv_weights": "csv", "tabs_comments_crlf": "tab", "zero_based_spaces": "txt",
                            "mtx": "mtx"}[style])
    write_variant(p, a, b, style, rng)
    same_as_oracle(ctx, str(p), orders=("kcore",))


def test_large_mtx_file_matches_pairs(ctx, tmp_path):
    """RMAT scale 16 as an mtx file: the device reader gives the graph the
    pair intake gives (same n, m, CSR and counts)."""
    s, d = pgd.rmat(16, 16, seed=1)
    keep = s != d
    u = np.minimum(s, d)[keep].astype(np.int64)
    v = np.maximum(s, d)[keep].astype(np.int64)
    key = np.unique(u * (1 << 32) + v)
    a = (key >> 32).astype(np.int32)
    b = (key & 0xFFFFFFFF).astype(np.int32)
    n = int(b.max()) + 1
    p = tmp_path / "rmat16.mtx"
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, len(a)))
        np.savetxt(f, np.stack([b + 1, a + 1], 1), fmt="%d")
    g1 = ctx.graph_from_file(str(p))
    g2 = ctx.graph_from_edges(b, a, dedup=False)
    assert (g1.n, g1.m) == (g2.n, g2.m)
    for g in (g1, g2):
        g.preprocess("deg")
    e1 = g1.edges(with_order=False)
    e2 = g2.edges(with_order=False)
    assert (e1[0] == e2[0]).all() and (e1[1] == e2[1]).all()
    r1 = g1.decompose(micro=False)
    r2 = g2.decompose(micro=False)
    assert (r1.totals == r2.totals).all()
