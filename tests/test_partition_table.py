"""The committed partition pattern tables (csrc/astc_partition_table.h) are
what the generator computes, and what the oracle's spec decoder does: a
two-partition block with partition 0 black and partition 1 white (all weights
zero) decodes to exactly the table's mask, for every partition index and
both block sizes; the three-partition class lists equal the oracle's, are
distinct splits into three non-empty sets, and a three-partition block with
partitions black / grey / white decodes to exactly each class's sets."""
import os
import re
import sys

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "astc_encoder_gb300", "csrc")


def _header_tables():
    text = open(os.path.join(CSRC, "astc_partition_table.h")).read()
    out = {}
    for name in ("kPartition2Mask4x4", "kPartition2Mask6x6"):
        body = re.search(name + r"\[1024\] = \{(.*?)\};", text, re.S).group(1)
        out[name] = [int(v.rstrip("ul"), 16) for v in re.findall(r"0x[0-9A-Fa-f]+u?l*", body)]
        assert len(out[name]) == 1024
    return out["kPartition2Mask4x4"], out["kPartition2Mask6x6"]


def _header_classes():
    text = open(os.path.join(CSRC, "astc_partition_table.h")).read()
    out = []
    for name, shift, mbits in (("kPartition2Classes4x4", 16, 16), ("kPartition2Classes6x6", 54, 36)):
        body = re.search(name + r"\[\d+\] = \{(.*?)\};", text, re.S).group(1)
        vals = [int(v.rstrip("ul"), 16) for v in re.findall(r"0x[0-9A-Fa-f]+u?l*", body)]
        out.append([(v >> shift, v & ((1 << mbits) - 1)) for v in vals])
    return out


def test_classes_pick_the_same_index_as_a_full_scan():
    """The class lists scanned in order give the full scan's choice for any split."""
    m4, m6 = _header_tables()
    c4, c6 = _header_classes()
    rng = np.random.default_rng(3)
    for dim, table, cls in ((4, m4, c4), (6, m6, c6)):
        n = dim * dim
        full = (1 << n) - 1
        for s, m in cls:
            assert table[s] == m and m not in (0, full)
        for _ in range(300):
            ideal = int(rng.integers(1, full))
            best = (n + 1, -1)
            for s, m in enumerate(table):
                if m in (0, full):
                    continue
                d = bin(m ^ ideal).count("1")
                d = min(d, n - d)
                if d < best[0]:
                    best = (d, s)
            got = (n + 1, -1)
            for s, m in cls:
                d = bin(m ^ ideal).count("1")
                d = min(d, n - d)
                if d < got[0]:
                    got = (d, s)
            assert got == best


def test_header_matches_generator():
    sys.path.insert(0, CSRC)
    try:
        import gen_partition_table as gen
    finally:
        sys.path.remove(CSRC)
    m4, m6 = _header_tables()
    assert m4 == gen.masks(4)
    assert m6 == gen.masks(6)
    assert _header_classes() == [gen.classes(4), gen.classes(6)]


def _two_partition_block(seed: int) -> np.ndarray:
    # 4x4 weight grid, QUANT_3 weights (26 bits, all zero), 2 partitions, CEM 8
    # for both; 12 endpoint values of QUANT_64 (6 bits each) from bit 29:
    # partition 0 all 0 (black), partition 1 all 63 (white)
    r = 3  # QUANT_3: R = 3 -> bits [1:0] = 1, bit 4 = 1; A = 2 at bits 5-6
    mode = ((r >> 1) & 3) | ((r & 1) << 4) | (2 << 5)
    v = mode | (1 << 11) | (seed << 13) | ((8 << 2) << 23)
    for i in range(6, 12):
        v |= 63 << (29 + 6 * i)
    return np.frombuffer(v.to_bytes(16, "little"), np.uint8).copy()


@pytest.mark.parametrize("dim", [4, 6])
def test_table_matches_spec_decoder(oracle, dim):
    m4, m6 = _header_tables()
    table = m4 if dim == 4 else m6
    for seed in range(1024):
        rgba, err = oracle.decode_block(_two_partition_block(seed), dim, dim)
        assert err == 0
        rgba = rgba.reshape(-1, 4)
        assert set(np.unique(rgba[:, 0]).tolist()) <= {0, 255}
        mask = sum(1 << i for i in range(dim * dim) if rgba[i, 0] == 255)
        assert mask == table[seed], seed


def _header_three_classes():
    text = open(os.path.join(CSRC, "astc_partition_table.h")).read()

    def arr(name):
        body = re.search(name + r"\[\d+\] = \{(.*?)\};", text, re.S).group(1)
        return [int(v.rstrip("ul"), 16) for v in re.findall(r"0x[0-9A-Fa-f]+u?l*", body)]

    c4 = [(v >> 32, v & 0xFFFF, (v >> 16) & 0xFFFF) for v in arr("kPartition3Classes4x4")]
    a, b = arr("kPartition3Classes6x6A"), arr("kPartition3Classes6x6B")
    c6 = [(x >> 54, x & ((1 << 36) - 1), y) for x, y in zip(a, b)]
    return c4, c6


def test_three_partition_classes_match_generator_and_oracle(oracle):
    sys.path.insert(0, CSRC)
    try:
        import gen_partition_table as gen
    finally:
        sys.path.remove(CSRC)
    c4, c6 = _header_three_classes()
    assert c4 == gen.classes3(4) and c6 == gen.classes3(6)
    assert c4 == oracle.three_classes(4) and c6 == oracle.three_classes(6)
    for dim, cls in ((4, c4), (6, c6)):
        full = (1 << (dim * dim)) - 1
        seeds = [s for s, _, _ in cls]
        assert seeds == sorted(seeds)
        for s, m1, m2 in cls:
            assert m1 and m2 and not (m1 & m2) and (full & ~(m1 | m2))
        # distinct as splits: no two classes are the same three sets
        keys = {frozenset([m1, m2, full & ~(m1 | m2)]) for _, m1, m2 in cls}
        assert len(keys) == len(cls)


def _three_partition_block(seed: int) -> np.ndarray:
    # 4x4 weight grid, QUANT_3 weights (26 bits, all zero), 3 partitions, CEM 8
    # for all; 18 endpoint values of QUANT_16 (4 bits each) from bit 29:
    # partition 0 all 0 (black), partition 1 all 8 (136), partition 2 all 15 (255)
    r = 3
    mode = ((r >> 1) & 3) | ((r & 1) << 4) | (2 << 5)
    v = mode | (2 << 11) | (seed << 13) | ((8 << 2) << 23)
    for i in range(6, 18):
        v |= (8 if i < 12 else 15) << (29 + 4 * i)
    return np.frombuffer(v.to_bytes(16, "little"), np.uint8).copy()


@pytest.mark.parametrize("dim", [4, 6])
def test_three_partition_classes_match_spec_decoder(oracle, dim):
    c4, c6 = _header_three_classes()
    for seed, m1, m2 in (c4 if dim == 4 else c6):
        rgba, err = oracle.decode_block(_three_partition_block(seed), dim, dim)
        assert err == 0
        r = rgba.reshape(-1, 4)[:, 0]
        assert set(np.unique(r).tolist()) <= {0, 136, 255}
        got1 = sum(1 << i for i in range(dim * dim) if r[i] == 136)
        got2 = sum(1 << i for i in range(dim * dim) if r[i] == 255)
        assert (got1, got2) == (m1, m2), seed
