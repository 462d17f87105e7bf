"""Integer stages of the oracle: ISE, unquantisation, block assembly, decoder.

Property tests written from the ASTC specification: every one of the 21
ranges round-trips through encode -> spec decode; the bit counts follow
compute_ise_bitcount (ASTC_IntegerSequenceEncoding.hlsl:76-93); symbolic
blocks decode back to their endpoints.
"""
import numpy as np
import pytest

LEVELS = [2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32, 40, 48, 64, 80, 96, 128, 160, 192, 256]


def _ise_bits_formula(q, n):
    lv = LEVELS[q]
    b = 0
    while lv % 2 == 0:
        lv //= 2
        b += 1
    if lv == 3:
        return ((8 + 5 * b) * n + 4) // 5
    if lv == 5:
        return ((7 + 3 * b) * n + 2) // 3
    return n * b


@pytest.mark.parametrize("quant", range(21))
def test_ise_round_trip_all_ranges(oracle, quant):
    rng = np.random.default_rng(quant)
    for count in (1, 2, 3, 4, 5, 6, 7, 8, 11, 16, 17):
        bits = oracle.ise_bits(quant, count)
        assert bits == _ise_bits_formula(quant, count)
        if bits > 128:
            continue
        for _ in range(20):
            v = rng.integers(0, LEVELS[quant], count).astype(np.uint32)
            enc = oracle.ise_encode(quant, v)
            dec = oracle.ise_decode(quant, count, enc)
            assert np.array_equal(dec, v)
            # nothing is written past the spec's bit count
            tail = int.from_bytes(bytes(enc), "little") >> bits
            assert tail == 0


def test_ise_extremes(oracle):
    for quant in range(21):
        top = LEVELS[quant] - 1
        n = 1
        while oracle.ise_bits(quant, n + 1) <= 128 and n < 64:
            n += 1
        v = np.full(n, top, np.uint32)
        assert np.array_equal(oracle.ise_decode(quant, n, oracle.ise_encode(quant, v)), v)
        z = np.zeros(n, np.uint32)
        assert int.from_bytes(bytes(oracle.ise_encode(quant, z)), "little") == 0


def test_unquant_ranges(oracle):
    for q in range(12):
        vals = sorted(oracle.unquant_weight(q, v) for v in range(LEVELS[q]))
        assert vals[0] == 0 and vals[-1] == 64
        assert len(set(vals)) == LEVELS[q]
    for q in range(4, 21):                  # colour ranges start at QUANT_6
        vals = sorted(oracle.unquant_color(q, v) for v in range(LEVELS[q]))
        assert vals[0] == 0 and vals[-1] == 255
        assert len(set(vals)) == LEVELS[q]
    # QUANT_256 endpoints are stored verbatim
    assert [oracle.unquant_color(20, v) for v in range(256)] == list(range(256))


@pytest.mark.parametrize("alpha", [False, True])
def test_symbolic_block_decodes_to_endpoints(oracle, alpha):
    rng = np.random.default_rng(7 + alpha)
    rmax = 5 if alpha else 11
    for _ in range(200):
        ep = rng.integers(0, 256, 8).astype(np.uint32)
        # the encoder orders endpoints dark -> light by their RGB sum
        if ep[0] + ep[2] + ep[4] > ep[1] + ep[3] + ep[5]:
            ep = ep.reshape(4, 2)[:, ::-1].reshape(-1).copy()
        if not alpha:
            ep[6], ep[7] = 255, 255
        qw = rng.integers(0, rmax + 1, 16).astype(np.uint32)
        qw[0], qw[1] = 0, rmax
        blk = oracle.assemble_symbolic(ep, qw, alpha)
        dec, rc = oracle.decode_block(blk, 4, 4)
        assert rc == 0
        e0 = ep[0::2].astype(int)
        e1 = ep[1::2].astype(int)
        assert np.array_equal(dec[0, 0], e0)       # weight 0 -> e0 exactly
        assert np.array_equal(dec[0, 1], e1)       # full weight -> e1 exactly
        # every texel lies between the endpoints
        lo, hi = np.minimum(e0, e1), np.maximum(e0, e1)
        assert np.all(dec.reshape(-1, 4) >= lo) and np.all(dec.reshape(-1, 4) <= hi)


def test_constant_block_layout(oracle):
    # a constant block: e0 == e1 == colour, every weight bit zero
    for alpha in (False, True):
        tex = np.tile(np.array([[10, 200, 30, 77]], np.float32), (16, 1))
        ep, qw, blk = oracle.encode_block(tex, 4, alpha)
        assert ep[:6].tolist() == [10, 10, 200, 200, 30, 30]
        assert np.all(qw == 0)
        v = int.from_bytes(bytes(blk), "little")
        eps = [(v >> (17 + 8 * i)) & 0xFF for i in range(8 if alpha else 6)]
        assert eps[:6] == [10, 10, 200, 200, 30, 30]
        if alpha:
            assert eps[6:] == [77, 77]
        wbits = 42 if alpha else 58
        assert v >> (128 - wbits) == 0


def test_decoder_void_extent_and_errors(oracle):
    # void-extent LDR block: mode bits 0x1FC, 16-bit RGBA at bits 64..127
    v = 0x1FC | (0x1FFF << 12) | (0x1FFF << 25) | (0x1FFF << 38) | (0x1FFF << 51)
    v |= (0x1234 << 64) | (0xABCD << 80) | (0x00FF << 96) | (0xFF00 << 112)
    blk = np.frombuffer(v.to_bytes(16, "little"), np.uint8)
    dec, rc = oracle.decode_block(blk, 4, 4)
    assert rc == 0 and dec[0, 0].tolist() == [0x12, 0xAB, 0x00, 0xFF]
    # reserved block mode (low 4 bits zero) -> error colour magenta
    dec, rc = oracle.decode_block(np.zeros(16, np.uint8), 4, 4)
    assert rc == 1 and dec[0, 0].tolist() == [255, 0, 255, 255]


def test_flops_constants(oracle):
    f4 = oracle.flops_per_block(4, False)
    f6 = oracle.flops_per_block(6, True)
    assert 1500 < f4 < 2200 and 2800 < f6 < 3800
