"""Regenerates the golden fixtures in tests/golden/ from the reference tree.

Run in a checkout that has the reference tree (its path is the one required
argument).  Writes:

* reference_tables.json -- the reference's literal tables, parsed from its
  HLSL sources as text: bits_trits_quints_table, integer_from_trits,
  integer_from_quints (ASTC_IntegerSequenceEncoding.hlsl:5-71),
  scramble_table (ASTC_Table.hlsl:4-66), idx_grids / wt_grids
  (ASTC_Encode.hlsl:268-304, weights kept as their source literals).
* leaf_crops.npz -- two 128x128 crops of textures/leaf.png, decoded with
  astc_encoder_gb300.image_io and flipped vertically as the reference CLI
  does (main.cpp:24), plus the matching 32x32-block windows of the reference's
  own output textures/leaf.astc (produced with -alpha -4x4, linear).  Crops
  start on block boundaries so every block lies inside the image.
* leaf_full_stats.json -- whole-image facts of leaf.astc used by the
  fixture-only tests (block count, mode words, constant-block count).
* leaf_differing_blocks.npz -- every block of textures/leaf.astc that the
  FP32 oracle does not reproduce bit for bit: its block index, its 16 texels
  (flipped as above) and the reference's 16 bytes.  The tests explain each
  one by the decision that differs (tests/test_oracle_leaf_classes.py).

The reference's texture is 1024x1024; the crops keep the committed fixture
small (about 100 KB) while covering constant, opaque and cut-out blocks.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from astc_encoder_gb300 import image_io  # noqa: E402

# block-grid origins (block row, block column) of the two crops
CROPS = [(96, 176), (176, 0)]
CROP_BLOCKS = 32


def parse_int_table(src: str, name: str) -> list[int]:
    m = re.search(name + r"\s*\[[^\]]*\]\s*=\s*\{(.*?)\};", src, re.S)
    if not m:
        raise ValueError(f"table {name} not found")
    body = re.sub(r"//[^\n]*", "", m.group(1))
    return [int(x) for x in re.findall(r"-?\d+", body)]


def parse_vec_table(src: str, name: str, kind: str) -> list[list[str]]:
    m = re.search(name + r"\s*\[[^\]]*\]\s*=\s*\{(.*?)\};", src, re.S)
    if not m:
        raise ValueError(f"table {name} not found")
    return [[t.strip() for t in g.split(",")] for g in re.findall(kind + r"\(([^)]*)\)", m.group(1))]


def main(ref: str) -> None:
    ise = open(os.path.join(ref, "ASTC_IntegerSequenceEncoding.hlsl")).read()
    tab = open(os.path.join(ref, "ASTC_Table.hlsl")).read()
    enc = open(os.path.join(ref, "ASTC_Encode.hlsl")).read()
    tables = {
        "bits_trits_quints_table": parse_int_table(ise, "bits_trits_quints_table"),
        "integer_from_trits": parse_int_table(ise, "integer_from_trits"),
        "integer_from_quints": parse_int_table(ise, "integer_from_quints"),
        "scramble_table": parse_int_table(tab, "scramble_table"),
        "idx_grids": [[int(v) for v in g] for g in parse_vec_table(enc, "idx_grids", "uint4")],
        "wt_grids": parse_vec_table(enc, "wt_grids", "float4"),
        "source": "niepp/astc_encoder: ASTC_IntegerSequenceEncoding.hlsl:5-71, "
                  "ASTC_Table.hlsl:4-66, ASTC_Encode.hlsl:268-304",
    }
    assert len(tables["integer_from_trits"]) == 243
    assert len(tables["integer_from_quints"]) == 125
    assert len(tables["scramble_table"]) == 384
    assert len(tables["bits_trits_quints_table"]) == 63
    with open(os.path.join(HERE, "reference_tables.json"), "w") as fh:
        json.dump(tables, fh, indent=1)

    img = image_io.load_png(os.path.join(ref, "textures", "leaf.png"))
    flipped = np.ascontiguousarray(img[::-1])
    raw = open(os.path.join(ref, "textures", "leaf.astc"), "rb").read()
    header = np.frombuffer(raw[:16], np.uint8)
    blocks = np.frombuffer(raw[16:], np.uint8).reshape(256, 256, 16)
    arrays = {"header": header}
    for i, (by, bx) in enumerate(CROPS):
        n = CROP_BLOCKS
        arrays[f"crop{i}_rgba"] = flipped[by * 4:(by + n) * 4, bx * 4:(bx + n) * 4].copy()
        arrays[f"crop{i}_blocks"] = blocks[by:by + n, bx:bx + n].reshape(-1, 16).copy()
        arrays[f"crop{i}_origin"] = np.array([by, bx], np.int32)
    np.savez_compressed(os.path.join(HERE, "leaf_crops.npz"), **arrays)

    flat = blocks.reshape(-1, 16)
    words = flat.view("<u4")
    tex = flipped.reshape(256, 4, 256, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    const = np.all(tex == tex[:, :1, :], axis=(1, 2))
    stats = {
        "width": 1024, "height": 1024, "block": [4, 4], "blocks": int(flat.shape[0]),
        "mode_words": sorted(set(int(x) for x in (words[:, 0] & 0x7FF))),
        "cem_values": sorted(set(int(x) for x in ((words[:, 0] >> 13) & 0xF))),
        "constant_blocks": int(const.sum()),
        "source": "niepp/astc_encoder textures/leaf.png, textures/leaf.astc",
    }
    from oracle import oracle
    got = oracle.encode(flipped, block_dim=4, has_alpha=True)
    differ = np.where(~np.all(got == flat, axis=1))[0].astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "leaf_differing_blocks.npz"), index=differ,
                        texels=tex[differ].astype(np.uint8), reference=flat[differ].copy())
    stats["oracle_identical_blocks"] = int(flat.shape[0] - len(differ))
    # whole-image squared error (RGBA, 8-bit) of each decode against the source
    for key, blocks in (("reference_sse", flat), ("oracle_sse", got)):
        dec, errors = oracle.decode(blocks, 1024, 1024, 4)
        assert errors == 0
        stats[key] = float(np.sum((dec.astype(np.float64) - flipped.astype(np.float64)) ** 2))
    with open(os.path.join(HERE, "leaf_full_stats.json"), "w") as fh:
        json.dump(stats, fh, indent=1)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the niepp/astc_encoder tree>")
    main(sys.argv[1])
