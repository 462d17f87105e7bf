"""Explains, block by block, every block of the reference's own output
textures/leaf.astc that the FP32 oracle does not reproduce bit for bit.

leaf.astc was written by the reference shader (niepp/astc_encoder,
ASTC_Encode.hlsl) on unknown D3D11 hardware with -alpha -4x4 from the
vertically flipped leaf.png.  The oracle reproduces 64,332 of its 65,536
blocks exactly.  Each of the other 1,204 (tests/golden/leaf_differing_blocks.npz,
made by tests/golden/make_golden.py) falls in one of four classes, every one a
decision that the exact FP32 arithmetic and the reference's GPU arithmetic can
take differently:

A  weight tie (1,085 blocks): the endpoints are identical, and every weight
   that differs differs by one step where the oracle's scaled weight w * R
   lies within 2 ulp of .5 (collinear texels put it exactly on .5 in exact
   arithmetic; quantize_weight, ASTC_Encode.hlsl:256-260, rounds it).
B  endpoint rounding tie (15 blocks): every endpoint value that differs
   differs by one where the oracle's float endpoint lies within 2 ulp of .5
   (encode_color's round, ASTC_Encode.hlsl:233-245); weights that differ are
   ties as in A.
C  decoupled alpha axis (101 blocks): the block's RGB-alpha covariance is
   exactly zero and its alpha variance exceeds the RGB part's principal one.
   The power iteration's start vector has no alpha (ASTC_Encode.hlsl:96), so
   exact FP32 never leaves RGB, while any rounding noise on the reference's
   GPU grows by (lambda_alpha / lambda_rgb)^16 over the 16 products and the
   reference converges (fully or partly) to the alpha axis.
D  early exit at noise level (3 blocks): the covariance maps the start vector
   (0.26726, 0.80178, 0.53452), whose digits make r - g + b = 0, to a vector
   of length below 1e-5 (ASTC_Encode.hlsl:100) that is rounding noise; the
   oracle returns early and collapses the block to its mean, the reference
   did not.

For C and D the test exhibits the noise: seeding the start vector's alpha
with one value of magnitude at most 2^-20 (sixteen ulp of its largest
component, 0.80178) makes the oracle assemble exactly the reference's block.
"""
import json
import os

import numpy as np

from conftest import GOLDEN

FIX = np.load(os.path.join(GOLDEN, "leaf_differing_blocks.npz"))
STATS = json.load(open(os.path.join(GOLDEN, "leaf_full_stats.json")))

# tolerances of the classes, in ulp of the value rounded
TIE_ULP = 2
SEED_MAX = 2.0 ** -20
EXPECTED = {"A": 1085, "B": 15, "C": 101, "D": 3}


def _seeds() -> np.ndarray:
    """Powers of two first, then a fine geometric grid, both signs, all
    within SEED_MAX."""
    pw = [s * 2.0 ** -k for k in range(20, 41) for s in (1, -1)]
    fine = np.geomspace(1e-12, SEED_MAX, 3000)
    return np.array(pw + [s * g for g in fine for s in (1, -1)], np.float32)


def _symbolic(block: np.ndarray, oracle):
    """Endpoints r0 r1 g0 g1 b0 b1 a0 a1 and unscrambled QUANT_6 weights of a
    mode-0x043 CEM-12 block (the only mode in leaf.astc)."""
    q = block.view("<u8")
    v = int(q[0]) | (int(q[1]) << 64)
    ep = np.array([(v >> (17 + 8 * i)) & 0xFF for i in range(8)])
    rev = np.array([int(f"{int(block[15 - i]):08b}"[::-1], 2) for i in range(16)], np.uint8)
    sc6 = oracle.table("oracle_table_scramble", 384)[4 * 32:4 * 32 + 6]     # QUANT_6 row
    inv = np.argsort(sc6)
    qw = np.array([int(inv[x]) for x in oracle.ise_decode(4, 16, rev, 0)])
    return ep, qw


def _ties(vals, q_oracle, q_ref) -> bool:
    for i in np.where(q_oracle != q_ref)[0]:
        if abs(int(q_oracle[i]) - int(q_ref[i])) != 1:
            return False
        v = np.float32(vals[i])
        if abs(float(v) - np.floor(float(v)) - 0.5) > TIE_ULP * float(np.spacing(np.abs(v))):
            return False
    return True


def classify(texels: np.ndarray, ref: np.ndarray, oracle, seeds) -> str | None:
    tex = texels.astype(np.float32)
    tr = oracle.trace_block(tex, 4, True)
    ep_r, qw_r = _symbolic(ref, oracle)
    ep_o, qw_o = tr["ep"].astype(int), tr["qw"].astype(int)
    if np.array_equal(ep_o, ep_r) and _ties(tr["wR"], qw_o, qw_r):
        return "A"
    e_float = np.stack([tr["e0"], tr["e1"]], 1).reshape(-1)        # r0 r1 g0 g1 ...
    if _ties(e_float, ep_o, ep_r) and _ties(tr["wR"], qw_o, qw_r):
        return "B"
    seed = oracle.find_seed(tex, 4, True, ref, seeds)
    if seed is None or abs(seed) > SEED_MAX:
        return None
    cov = tr["cov"].reshape(4, 4).astype(np.float64)
    if np.all(cov[:3, 3] == 0) and np.all(cov[3, :3] == 0):
        if cov[3, 3] > np.linalg.eigvalsh(cov[:3, :3])[-1]:
            return "C"
        return None
    if tr["early_exit"] and tr["min_len"] < 1e-5:
        return "D"
    return None


def _encode_each(texels: np.ndarray, oracle) -> np.ndarray:
    return np.stack([oracle.encode(t.reshape(4, 4, 4), block_dim=4, has_alpha=True)[0] for t in texels])


def _sse(blocks: np.ndarray, texels: np.ndarray, oracle) -> float:
    """Squared error (RGBA, 8-bit) of the blocks' spec decode."""
    tot = 0.0
    for b, t in zip(blocks, texels):
        d, err = oracle.decode(b[None], 4, 4, 4)
        assert err == 0
        tot += float(np.sum((d.astype(np.float64) - t.reshape(4, 4, 4).astype(np.float64)) ** 2))
    return tot


def _psnr_gap_db(sse_a: float, sse_b: float) -> float:
    return 10 * np.log10(sse_a / sse_b)


def test_fixture_is_the_oracles_difference(oracle):
    """The fixture holds exactly the blocks the oracle gets wrong, and their
    error difference is the whole image's."""
    n = len(FIX["index"])
    assert n == STATS["blocks"] - STATS["oracle_identical_blocks"] == 1204
    got = _encode_each(FIX["texels"], oracle)
    assert not np.any(np.all(got == FIX["reference"], axis=1))
    # integer fields (mode 0x043, one partition, CEM 12) agree everywhere
    gw, rw = got.view("<u4")[:, 0], FIX["reference"].view("<u4")[:, 0]
    assert np.array_equal(gw & 0x1FFFF, rw & 0x1FFFF)
    # identical blocks decode identically, so the whole-image error
    # difference is the differing blocks' difference
    d_or = _sse(got, FIX["texels"], oracle)
    d_ref = _sse(FIX["reference"], FIX["texels"], oracle)
    assert STATS["oracle_sse"] - STATS["reference_sse"] == d_or - d_ref


def test_every_differing_block_is_explained(oracle):
    seeds = _seeds()
    classes = {}
    unexplained = []
    for i in range(len(FIX["index"])):
        c = classify(FIX["texels"][i], FIX["reference"][i], oracle, seeds)
        if c is None:
            unexplained.append(int(FIX["index"][i]))
        else:
            classes[c] = classes.get(c, 0) + 1
    assert not unexplained, f"blocks with no class: {unexplained[:20]}"
    assert classes == EXPECTED


def test_axis_classes_carry_the_psnr_gap(oracle):
    """The oracle decodes 0.0475 dB below leaf.astc over the whole image.
    Replacing only the C and D blocks by the seeded oracle's blocks (which are
    the reference's) leaves the ties, and the gap falls below 0.001 dB: the
    reference's better PSNR comes from the alpha axis its rounding noise
    found, not from its rounding of ties (measured: 0.0475 -> 0.0003 dB)."""
    seeds = _seeds()
    n = len(FIX["index"])
    ref = FIX["reference"]
    got = _encode_each(FIX["texels"], oracle)
    mixed = got.copy()
    replaced = 0
    for i in range(n):
        if classify(FIX["texels"][i], ref[i], oracle, seeds) in ("C", "D"):
            mixed[i] = ref[i]
            replaced += 1
    assert replaced == EXPECTED["C"] + EXPECTED["D"]
    d_ref = _sse(ref, FIX["texels"], oracle)
    gap_plain = _psnr_gap_db(STATS["oracle_sse"], STATS["reference_sse"])
    gap_mixed = _psnr_gap_db(STATS["reference_sse"] + _sse(mixed, FIX["texels"], oracle) - d_ref,
                             STATS["reference_sse"])
    assert 0.04 < gap_plain < 0.05, gap_plain
    assert abs(gap_mixed) < 0.001, gap_mixed
