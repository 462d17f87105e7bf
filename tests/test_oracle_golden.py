"""Pins the FP32 oracle against the reference's own output, textures/leaf.astc.

leaf.astc was produced by the reference shader on unknown D3D11 hardware with
-alpha -4x4 in linear space from the vertically flipped leaf.png.  Its integer
fields (block mode, partition bits, CEM, endpoint layout, ISE of constant
blocks) pin the integer stages exactly.  The float stages can only be pinned
statistically: the oracle reproduces 98.16% of the blocks bit for bit, and
tests/test_oracle_leaf_classes.py explains each of the others (weight and
endpoint ties, and the alpha axis that the reference's rounding noise finds
in RGB-alpha decoupled blocks).  The oracle is deterministic, so the counts
below are exact: any change of its arithmetic shows here.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

CROPS = np.load(os.path.join(GOLDEN, "leaf_crops.npz"))
STATS = json.load(open(os.path.join(GOLDEN, "leaf_full_stats.json")))


def _endpoint_field(blocks):
    q = blocks.view("<u8")
    return (q[:, 0] >> np.uint64(17)) | (q[:, 1] << np.uint64(47))


def _psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return 10 * np.log10(255.0 ** 2 / mse)


def test_header_of_reference_file():
    h = CROPS["header"]
    assert h[:4].tolist() == [0x13, 0xAB, 0xA1, 0x5C]
    assert h[4:7].tolist() == [4, 4, 1]
    assert int(h[7]) | int(h[8]) << 8 | int(h[9]) << 16 == 1024
    assert int(h[10]) | int(h[11]) << 8 | int(h[12]) << 16 == 1024
    assert h[13:16].tolist() == [1, 0, 0]
    assert STATS["mode_words"] == [0x043] and STATS["cem_values"] == [12]


# per crop: blocks that differ, blocks whose endpoint field differs, and the
# oracle's decoded PSNR minus the reference's (dB)
CROP_FIGURES = {0: (17, 7, -0.0765), 1: (10, 0, -0.0002)}


@pytest.mark.parametrize("crop", [0, 1])
def test_oracle_matches_leaf_crop(oracle, crop):
    rgba = CROPS[f"crop{crop}_rgba"]
    ref = CROPS[f"crop{crop}_blocks"]
    got = oracle.encode(rgba, block_dim=4, has_alpha=True)
    same = np.all(got == ref, axis=1)
    # integer fields of every block
    gw = got.view("<u4")[:, 0]
    rw = ref.view("<u4")[:, 0]
    assert np.array_equal(gw & 0x1FFFF, rw & 0x1FFFF)
    # constant blocks: e0 == e1 == the colour, all weights zero -> identical
    tex = rgba.reshape(32, 4, 32, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    const = np.all(tex == tex[:, :1, :], axis=(1, 2))
    assert const.sum() > 100
    assert same[const].all()
    # the float stages: exact counts of the deterministic oracle
    n_diff, n_ep, gap = CROP_FIGURES[crop]
    assert int((~same).sum()) == n_diff
    assert int((_endpoint_field(got) != _endpoint_field(ref)).sum()) == n_ep
    d_ref, e1 = oracle.decode(ref, 128, 128, 4)
    d_got, e2 = oracle.decode(got, 128, 128, 4)
    assert e1 == 0 and e2 == 0
    assert abs((_psnr(d_got, rgba) - _psnr(d_ref, rgba)) - gap) < 0.001


def test_oracle_matches_full_leaf(oracle, reference_dir):
    """Whole image (only where the reference tree is mounted)."""
    from astc_encoder_gb300 import image_io
    img = image_io.load_png(os.path.join(reference_dir, "textures", "leaf.png"))
    flipped = np.ascontiguousarray(img[::-1])
    raw = open(os.path.join(reference_dir, "textures", "leaf.astc"), "rb").read()
    ref = np.frombuffer(raw[16:], np.uint8).reshape(-1, 16)
    got = oracle.encode(flipped, block_dim=4, has_alpha=True)
    same = np.all(got == ref, axis=1)
    tex = flipped.reshape(256, 4, 256, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    const = np.all(tex == tex[:, :1, :], axis=(1, 2))
    assert const.sum() == STATS["constant_blocks"] == 18340
    assert same[const].all()
    assert int(same.sum()) == STATS["oracle_identical_blocks"] == 64332        # 98.16%
    ep_same = _endpoint_field(got) == _endpoint_field(ref)     # 64 bits from bit 17
    assert int((~ep_same).sum()) == 118                                        # 99.82%
    d_ref, _ = oracle.decode(ref, 1024, 1024, 4)
    d_got, _ = oracle.decode(got, 1024, 1024, 4)
    gap = _psnr(d_ref, flipped) - _psnr(d_got, flipped)
    assert 0.047 < gap < 0.048, gap
    # the reference's constant blocks decode back to their exact colour
    db = d_ref.reshape(256, 4, 256, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    assert np.array_equal(db[const], tex[const])
