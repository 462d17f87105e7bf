"""The oracle's spec-generated tables against the reference's literal arrays.

The reference ships its ISE and scramble tables as literals
(ASTC_IntegerSequenceEncoding.hlsl:5-71, ASTC_Table.hlsl:4-66) and the 6x6
bilinear taps as idx_grids / wt_grids (ASTC_Encode.hlsl:268-304); the golden
file tests/golden/reference_tables.json holds them, parsed from the sources
by tests/golden/make_golden.py.  The oracle generates every table from the
ASTC specification, so element-wise equality pins both.
"""
import json
import os

import numpy as np

from conftest import GOLDEN

REF = json.load(open(os.path.join(GOLDEN, "reference_tables.json")))


def test_bits_trits_quints(oracle):
    got = oracle.table("oracle_table_btq", 63)
    assert got.tolist() == REF["bits_trits_quints_table"]


def test_integer_from_trits(oracle):
    got = oracle.table("oracle_table_trits", 243)
    assert got.tolist() == REF["integer_from_trits"]


def test_integer_from_quints(oracle):
    got = oracle.table("oracle_table_quints", 125)
    assert got.tolist() == REF["integer_from_quints"]


def test_scramble_table(oracle):
    got = oracle.table("oracle_table_scramble", 384)
    assert got.tolist() == REF["scramble_table"]


def test_scramble_orders_by_unquantised_weight(oracle):
    # for every weight range: symbol scramble[i] unquantises to the i-th
    # smallest weight -- the property the table encodes
    sc = oracle.table("oracle_table_scramble", 384).reshape(12, 32)
    levels = [2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32]
    for q, n in enumerate(levels):
        vals = [oracle.unquant_weight(q, int(sc[q, i])) for i in range(n)]
        assert vals == sorted(vals), q
        assert vals[0] == 0 and vals[-1] == 64
        assert sorted(sc[q, :n].tolist()) == list(range(n))


def test_6x6_grid_taps(oracle):
    for g in range(16):
        idx, wt = oracle.grid_taps(g)
        assert idx.tolist() == REF["idx_grids"][g]
        want = np.array([np.float32(float(s)) for s in REF["wt_grids"][g]], np.float32)
        assert np.array_equal(wt, want), g


def test_blockmode_words(oracle):
    # assemble_blockmode (ASTC_Encode.hlsl:446-473) for QUANT_12 / QUANT_6 on a
    # 4x4 grid; 0x043 is the mode of every block of the reference's leaf.astc
    for alpha, mode, cem in ((False, 0x251, 8), (True, 0x043, 12)):
        blk = oracle.assemble_symbolic(np.zeros(8), np.zeros(16), alpha)
        word = int.from_bytes(bytes(blk[:4]), "little")
        assert word & 0x7FF == mode
        assert (word >> 11) & 3 == 0
        assert (word >> 13) & 0xF == cem


def test_srgb_lut(oracle):
    lut = oracle.srgb_lut()
    for c in (0, 1, 10, 11, 128, 200, 255):
        x = c / 255.0
        lin = x / 12.92 if x <= 0.04045 else ((x + 0.055) / 1.055) ** 2.4
        assert lut[c] == np.float32(np.float32(lin) * np.float32(255.0))
    assert lut[0] == 0.0 and lut[255] == 255.0
    assert np.all(np.diff(lut) > 0)


def test_unorm8_fetch_is_exact():
    # the D3D11 UNORM8 -> float -> x255 chain of MainCS (ASTC_Encode.hlsl:574-579)
    # returns the integer code exactly for every byte value
    c = np.arange(256, dtype=np.float32)
    assert np.array_equal((c / np.float32(255.0)) * np.float32(255.0), c)


def test_product_srgb_values_match_oracle(oracle):
    import astc_encoder_gb300 as astc
    assert np.array_equal(astc.srgb_texel_values(), oracle.srgb_lut())
