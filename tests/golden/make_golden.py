"""Regenerate the golden fixtures in tests/golden/ from the reference.

Needs the reference tree (default /root/reference, or $PGD_REFERENCE) and
the reference built from its sources (`make -C oracle ref`).  Writes:

  toy.json        the reference's toy graphs (data/4-clique*.txt, data/4-chordal-cycle.txt,
                  data/4-clique.edges): file text, the reference's 17 totals and micro rows
  dd21.npz        sample_graph.csv: its input pairs, the golden per-edge rows it ships,
                  and the reference's totals and micro rows (row order included)
  synth.npz       seeded synthetic graphs (G(250,0.9) seed 1, RMAT scale 12, BA, ER mix)
                  with the reference's totals and micro rows for several orderings
  bign.npz        a 2.3M-vertex sparse graph whose n(n-1)(n-2) overflows int64:
                  pairs and the reference's totals
  cli/*.txt.gz    stdout, -c and -m files of the reference's ./pgd on small inputs

Run:  python tests/golden/make_golden.py
"""
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)

import oracle_lib as ol  # noqa: E402
import pgd_gb300 as pgd  # noqa: E402

REF = os.environ.get("PGD_REFERENCE", "/root/reference")
TOYS = ["data/4-clique.txt", "data/4-chordal-cycle.txt", "data/4-clique-and-edge.txt", "data/4-clique.edges"]


def ref_run_file(path, order="deg", s2l=False, neigh="deg", s2l_neigh=False, micro=True):
    g = ol.RefGraph.from_file(path, neigh=neigh, s2l_neigh=s2l_neigh).run(order=order, s2l=s2l, micro=micro,
                                                                          workers=8)
    out = {"n": g.n, "m": g.m, "K": g.max_core, "r": g.r, "totals": g.totals()}
    if micro:
        out["src"], out["dst"], out["cols"] = g.micro()
    return out


def write_mtx(path, src, dst, n):
    """Each undirected edge once, 1-based, larger id first (as the RMAT sketch did)."""
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, len(src)))
        a = np.maximum(src, dst) + 1
        b = np.minimum(src, dst) + 1
        np.savetxt(f, np.stack([a, b], 1), fmt="%d")


def rows_digest(src, dst, cols):
    """SHA-256 of the ordered micro rows (src, dst, 8 columns as little-endian uint64)."""
    rows = np.concatenate([np.asarray(src, np.uint64)[:, None], np.asarray(dst, np.uint64)[:, None],
                           np.asarray(cols, np.uint64)], axis=1)
    return hashlib.sha256(np.ascontiguousarray(rows, "<u8").tobytes()).hexdigest()


def simple_pairs(src, dst):
    """Symmetrised, deduplicated, self-loop-free pairs (u < v), sorted."""
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    keep = src != dst
    u = np.minimum(src, dst)[keep]
    v = np.maximum(src, dst)[keep]
    key = np.unique(u * (1 << 32) + v)
    return (key >> 32).astype(np.int32), (key & 0xFFFFFFFF).astype(np.int32)


def main():
    if not ol.ref_available():
        subprocess.run(["make", "-s", "-C", ol.ORACLE_DIR, "ref", "REF=" + REF], check=True)
    tmp = tempfile.mkdtemp()
    try:
        # ---- toy graphs ----------------------------------------------------
        toys = {}
        for rel in TOYS:
            src = os.path.join(REF, rel)
            text = open(src).read()
            path = os.path.join(tmp, os.path.basename(rel))
            open(path, "w").write(text)
            r = ref_run_file(path)
            toys[os.path.basename(rel)] = {
                "text": text, "n": r["n"], "m": r["m"], "K": r["K"],
                "totals": [int(x) for x in r["totals"]],
                "rows": [[int(a), int(b)] + [int(x) for x in c] for a, b, c in zip(r["src"], r["dst"], r["cols"])],
            }
        json.dump(toys, open(os.path.join(HERE, "toy.json"), "w"), indent=1)

        # ---- sample_graph.csv (DD21) ---------------------------------------
        lines = open(os.path.join(REF, "sample_graph.csv")).read().splitlines()
        header = lines[0]
        body = np.array([[int(x) for x in ln.split(",")] for ln in lines[1:] if ln.strip()], np.int64)
        path = os.path.join(tmp, "sample_graph.csv")
        shutil.copy(os.path.join(REF, "sample_graph.csv"), path)
        r = ref_run_file(path)
        r_kc = ref_run_file(path, order="kcore")
        np.savez_compressed(
            os.path.join(HERE, "dd21.npz"),
            header=np.array(header), pairs=body[:, :2].astype(np.int32), golden_cols=body[:, 2:].astype(np.uint64),
            totals=r["totals"], src=r["src"], dst=r["dst"], cols=r["cols"], n=r["n"], m=r["m"], K=r["K"],
            kc_totals=r_kc["totals"], kc_src=r_kc["src"], kc_dst=r_kc["dst"], kc_cols=r_kc["cols"],
        )

        # ---- seeded synthetic graphs ---------------------------------------
        synth = {}
        cases = {
            "er250": pgd.erdos_renyi(250, 0.9, seed=1),
            "rmat12": pgd.rmat(12, 16, seed=1),
            "ba2000": pgd.barabasi_albert(2000, 5, seed=3),
            "er1500": pgd.erdos_renyi(1500, 0.02, seed=7),
        }
        for name, (s, d) in cases.items():
            u, v = simple_pairs(s, d)
            n = int(max(u.max(), v.max())) + 1
            path = os.path.join(tmp, name + ".mtx")
            write_mtx(path, u, v, n)
            synth[name + "_u"] = u
            synth[name + "_v"] = v
            for order, s2l in (("deg", False), ("kcore", False), ("natural", False), ("deg", True)):
                tag = "%s_%s%s" % (name, order, "_s2l" if s2l else "")
                r = ref_run_file(path, order=order, s2l=s2l)
                synth[tag + "_totals"] = r["totals"]
                synth[tag + "_rows_sha256"] = np.array(rows_digest(r["src"], r["dst"], r["cols"]))
                if order == "deg" and not s2l:
                    # per-edge values once, keyed by (src, dst); other orders by digest
                    synth[tag + "_src"] = r["src"].astype(np.int32)
                    synth[tag + "_dst"] = r["dst"].astype(np.int32)
                    synth[tag + "_cols"] = r["cols"]
                synth[tag + "_meta"] = np.array([r["n"], r["m"], r["K"]], np.int64)
                synth[tag + "_r"] = np.array(r["r"])
        np.savez_compressed(os.path.join(HERE, "synth.npz"), **synth)

        # ---- huge n, sparse (int64 overflow of n(n-1)(n-2)) -----------------
        n = 2_300_000
        rng = np.random.default_rng(5)
        extra = np.unique(rng.integers(1, n - 2, size=2000))
        a = np.concatenate([np.arange(1, n), extra])
        b = np.concatenate([np.arange(2, n + 1), extra + 2])
        path = os.path.join(tmp, "bign.mtx")
        with open(path, "w") as f:
            f.write("%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, len(a)))
            np.savetxt(f, np.stack([b, a], 1), fmt="%d")
        r = ref_run_file(path, micro=False)
        # pairs = the path 0-1-...-(n-1) (as (i+1, i)) followed by (x+1, x-1) for x in extra
        np.savez_compressed(os.path.join(HERE, "bign.npz"), n_path=n, extra=extra.astype(np.int32),
                            totals=r["totals"], n=r["n"], m=r["m"])

        # ---- CLI transcripts ----------------------------------------------
        cli = os.path.join(HERE, "cli")
        os.makedirs(cli, exist_ok=True)
        runs = {
            "clique_micro": (os.path.join(tmp, "4-clique.txt"), ["-m", "{out}.micro", "-c", "{out}.macro"]),
            "chordal": (os.path.join(tmp, "4-chordal-cycle.txt"), []),
            "sample_global": (os.path.join(tmp, "sample_graph.csv"), ["-c", "{out}.macro"]),
            "sample_micro_kcore": (os.path.join(tmp, "sample_graph.csv"), ["-o", "kcore", "-m", "{out}.micro"]),
            "er250_micro": (os.path.join(tmp, "er250.mtx"), ["-m", "{out}.micro"]),
        }
        meta = {}
        for name, (inp, extra_args) in runs.items():
            outbase = os.path.join(tmp, name)
            args = [ol.REF_BIN, "-f", inp] + [x.format(out=outbase) for x in extra_args]
            res = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, cwd=tmp)
            files = {}
            for suffix in (".micro", ".macro"):
                if os.path.exists(outbase + suffix):
                    files[suffix] = name + suffix + ".gz"
                    with open(outbase + suffix, "rb") as fi, gzip.open(os.path.join(cli, name + suffix + ".gz"), "wb") as fo:
                        fo.write(fi.read())
            with gzip.open(os.path.join(cli, name + ".stdout.gz"), "wt") as fo:
                fo.write(res.stdout.replace(tmp + "/", "{dir}/"))
            meta[name] = {"input": os.path.basename(inp), "args": extra_args, "files": files,
                          "returncode": res.returncode}
        json.dump(meta, open(os.path.join(cli, "runs.json"), "w"), indent=1)
        print("golden fixtures written to", HERE)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
