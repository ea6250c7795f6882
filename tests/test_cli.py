"""The drop-in `pgd` command line tool against transcripts of the
reference's own ./pgd (tests/golden/cli/, made by make_golden.py): the same
stdout line for line (the wall-clock timing line aside) and the same -c/-m
files byte for byte."""
import gzip
import json
import os
import subprocess

import numpy as np
import pytest

import pgd_gb300 as pgd
from helpers import GOLDEN, load_npz, load_toys

pytestmark = pytest.mark.gpu

CLI_DIR = os.path.join(GOLDEN, "cli")


def _inputs(tmp):
    toys = load_toys()
    for name in ("4-clique.txt", "4-chordal-cycle.txt"):
        open(os.path.join(tmp, name), "w").write(toys[name]["text"])
    z = load_npz("dd21.npz")
    with open(os.path.join(tmp, "sample_graph.csv"), "w") as f:
        f.write(str(z["header"]) + "\n")
        for a, b in z["pairs"]:
            f.write("%d,%d\n" % (a, b))
    s = load_npz("synth.npz")
    u, v = s["er250_u"], s["er250_v"]
    n = int(max(u.max(), v.max())) + 1
    with open(os.path.join(tmp, "er250.mtx"), "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, len(u)))
        np.savetxt(f, np.stack([np.maximum(u, v) + 1, np.minimum(u, v) + 1], 1), fmt="%d")


def _strip(text):
    return [ln for ln in text.splitlines() if not ln.startswith("graphlet decomposition time")]


RUNS = json.load(open(os.path.join(CLI_DIR, "runs.json")))


@pytest.mark.parametrize("name", sorted(RUNS))
def test_cli_transcript(tmp_path, name):
    tmp = str(tmp_path)
    _inputs(tmp)
    run = RUNS[name]
    outbase = os.path.join(tmp, name)
    args = [pgd.CLI_PATH, "-f", os.path.join(tmp, run["input"])] + [a.format(out=outbase) for a in run["args"]]
    res = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, cwd=tmp, timeout=300)
    assert res.returncode == run["returncode"], res.stderr
    want = gzip.open(os.path.join(CLI_DIR, name + ".stdout.gz"), "rt").read().replace("{dir}/", tmp + "/")
    assert _strip(res.stdout) == _strip(want)
    for suffix, fname in run["files"].items():
        got = open(outbase + suffix, "rb").read()
        assert got == gzip.open(os.path.join(CLI_DIR, fname), "rb").read(), suffix
