"""Design invariants of the tensor-core kernels of dense batch graphs
(decompose.cu: k_dense_tc, k_dense_gram), restated on the CPU:

* the operand-tile addressing: a builder item (16 bytes of one row) at byte
  16·i of a tile is exactly where the no-swizzle K-major core-matrix layout
  (8-row x 16-byte core matrices, LBO 128 B along K, SBO 512 B between 8-row
  groups) puts that row's 16 bytes;
* the nibble spread: (nib · 0x01020408) & 0x08080808 puts e4m3 2^-6 (0x08) in
  byte i exactly when bit i of nib is set;
* the bit-compress of Hacker's Delight §7-4 with its masks computed once per
  mask word, against a bit-by-bit compress;
* the warp's segmented OR-scan that assembles a compacted row from the 32
  lanes' compressed words, against a bit-by-bit compaction.
"""
import numpy as np

M64 = (1 << 64) - 1


def core_matrix_offset(row, kbyte, lbo=128, sbo=512):
    return (row >> 3) * sbo + (kbyte >> 4) * lbo + (row & 7) * 16 + (kbyte & 15)


def test_tile_item_addressing():
    # k_dense_tc / k_dense_gram: 64 bytes of K per row; item i2 -> row, 16-byte block
    for i2 in range(256 * 4):
        row = ((i2 >> 5) << 3) | (i2 & 7)
        blk = (i2 >> 3) & 3
        for b in range(16):
            assert core_matrix_offset(row, 16 * blk + b) == 16 * i2 + b
    # every (row, byte) of a 256-row tile is covered exactly once
    seen = set()
    for i2 in range(256 * 4):
        row = ((i2 >> 5) << 3) | (i2 & 7)
        blk = (i2 >> 3) & 3
        seen.add((row, blk))
    assert len(seen) == 256 * 4
    # an MMA's K step of 32 bytes starts 256 bytes further: two core matrices along K
    assert core_matrix_offset(0, 32) == 256 and core_matrix_offset(0, 16) == 128


def test_nibble_spread_to_e4m3():
    for nib in range(16):
        w = (nib * 0x01020408) & 0x08080808
        for b in range(4):
            assert (w >> (8 * b)) & 0xFF == (0x08 if (nib >> b) & 1 else 0)


def compress_masks(m):
    mk = (~m << 1) & M64
    mv = []
    for i in range(6):
        mp = (mk ^ (mk << 1)) & M64
        for sh in (2, 4, 8, 16, 32):
            mp = (mp ^ (mp << sh)) & M64
        v = mp & m
        mv.append(v)
        m = ((m ^ v) | (v >> (1 << i))) & M64
        mk = mk & ~mp & M64
    return mv


def compress(x, m, mv):
    x &= m
    for i in range(6):
        t = x & mv[i]
        x = ((x ^ t) | (t >> (1 << i))) & M64
    return x


def compress_naive(x, m):
    r, k = 0, 0
    for b in range(64):
        if (m >> b) & 1:
            r |= ((x >> b) & 1) << k
            k += 1
    return r


def test_bit_compress():
    rng = np.random.default_rng(3)
    for it in range(3000):
        m = int(rng.integers(0, 1 << 63)) * 2 + int(rng.integers(0, 2))
        if it % 4 == 1:
            m &= int(rng.integers(0, 1 << 63))
        if it % 4 == 2:
            m = M64 if it % 8 == 2 else 0
        x = int(rng.integers(0, 1 << 63)) * 2 + int(rng.integers(0, 2))
        assert compress(x, m, compress_masks(m)) == compress_naive(x, m)


def test_segmented_scan_compaction():
    rng = np.random.default_rng(5)
    for trial in range(400):
        W = int(rng.integers(1, 33))
        dens = float(rng.choice([0.03, 0.2, 0.5, 0.9, 1.0]))
        masks = [0] * 32
        for w in range(W):
            masks[w] = sum(1 << b for b in range(64) if rng.random() < dens)
        cnt = [bin(x).count("1") for x in masks]
        d = sum(cnt)
        if d == 0:
            continue
        o = [sum(cnt[:w]) for w in range(32)]
        KW = (d + 63) >> 6
        row = [int(rng.integers(0, 1 << 63)) * 2 + 1 if w < W else 0 for w in range(32)]
        bits = []
        for w in range(32):
            v = compress_naive(row[w], masks[w])
            bits += [(v >> i) & 1 for i in range(cnt[w])]
        want = [sum(bits[64 * k + i] << i for i in range(64) if 64 * k + i < d) for k in range(KW)]
        # the kernel's lanes
        w0 = [x >> 6 for x in o]
        sh = [x & 63 for x in o]
        v = [compress_naive(row[w], masks[w]) for w in range(32)]
        hi = [(v[w] >> (64 - sh[w])) if (sh[w] and sh[w] + cnt[w] > 64) else 0 for w in range(32)]
        first = [w == 0 or w0[w - 1] != w0[w] for w in range(32)]
        last = [w == 31 or w0[w + 1] != w0[w] for w in range(32)]
        val = [((v[w] << sh[w]) & M64) | (hi[w - 1] if first[w] and w > 0 else 0) for w in range(32)]
        for i in range(5):
            dl = 1 << i
            val = [val[w] | (val[w - dl] if w >= dl and w0[w - dl] == w0[w] else 0) for w in range(32)]
        C = [0] * (KW + 1)
        for w in range(32):
            if last[w] and w0[w] < KW:
                C[w0[w]] = val[w]
        if hi[31]:
            C[w0[31] + 1] = hi[31]
        assert C[:KW] == want and C[KW] == 0
