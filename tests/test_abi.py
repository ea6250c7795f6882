"""The C-ABI library: it loads, exports every symbol include/*.h declares,
and its host-only pieces (closing identities, generators, status strings)
behave.  No compute call needs a GPU here."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle_lib as ol
import pgd_gb300 as pgd

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            text = open(os.path.join(INCLUDE, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names.update(re.findall(r"\b(pgd_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    L = ctypes.CDLL(pgd.LIB_PATH)
    decl = declared_functions()
    assert len(decl) >= 20
    missing = [n for n in decl if not hasattr(L, n)]
    assert not missing, missing
    assert set(decl) <= set(pgd.EXPORTS) | set(decl)


def test_python_binding_lists_every_declared_symbol():
    assert set(declared_functions()) <= set(pgd.EXPORTS)


def test_status_strings():
    L = pgd.lib()
    for s in range(7):
        assert L.pgd_status_string(s)


def test_no_device_is_an_error_not_a_fallback():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(pgd.PGDError) as e:
        pgd.Context()
    assert e.value.status == 4  # PGD_ECUDA


def test_host_closing_matches_oracle():
    rng = np.random.default_rng(3)
    for trial in range(200):
        sums = rng.integers(0, 2 ** 63, size=15, dtype=np.uint64) * np.uint64(rng.integers(1, 3))
        if trial % 3 == 0:
            sums = rng.integers(0, 10 ** 9, size=15, dtype=np.uint64)
        n = int(rng.integers(0, 5_000_000))
        m = int(rng.integers(0, 10 ** 8))
        assert (pgd.close_counts(sums, n, m) == ol.close(sums, n, m)).all()


def _u01_numpy(seed, stream, idx):
    M = (1 << 64) - 1

    def mix(z):
        z = (z + 0x9E3779B97F4A7C15) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    key = mix(seed ^ mix(stream))
    return (mix((key + idx) & M) >> 11) * (1.0 / 9007199254740992.0)


def test_generator_counter_rng_is_splitmix():
    L = pgd.lib()
    for seed, stream, idx in [(1, 0x524D4154, 0), (1, 0x524D4154, 12345), (7, 0x4552, 2 ** 40), (0, 0, 0)]:
        assert L.pgd_gen_u01(seed, stream, idx) == _u01_numpy(seed, stream, idx)


def test_generators_are_deterministic_and_shaped():
    a = pgd.rmat(10, 16, seed=3)
    b = pgd.rmat(10, 16, seed=3)
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    assert len(a[0]) == 16 << 10 and a[0].max() < 1024
    c = pgd.rmat(10, 16, seed=4)
    assert not (a[0] == c[0]).all()
    s, d = pgd.erdos_renyi(250, 0.9, seed=1)
    assert 0.88 < len(s) / (250 * 249 / 2) < 0.92 and (s < d).all()
    s, d = pgd.barabasi_albert(500, 4, seed=2)
    assert len(s) == 10 + (500 - 5) * 4
    s, d = pgd.rgg3d(2000, 0.1, seed=5)
    assert len(s) > 0 and (s < d).all()


def test_concat_pairs_layout():
    """The flat batch format of pgd_decompose_pairs_batch: graph i's pairs are
    src/dst[off[i]:off[i + 1]], int32 ids, int64 offsets (no device needed)."""
    import numpy as np

    import pgd_gb300 as pgd

    graphs = [(np.array([0, 1, 2], np.int64), np.array([1, 2, 0], np.int64)),
              (np.zeros(0, np.int32), np.zeros(0, np.int32)),
              (np.array([5], np.int32), np.array([7], np.int32))]
    off, src, dst = pgd.concat_pairs(graphs)
    assert off.dtype == np.int64 and src.dtype == np.int32 and dst.dtype == np.int32
    assert off.tolist() == [0, 3, 3, 4]
    assert src.tolist() == [0, 1, 2, 5] and dst.tolist() == [1, 2, 0, 7]
    off0, src0, dst0 = pgd.concat_pairs([])
    assert off0.tolist() == [0] and len(src0) == 0 and len(dst0) == 0
