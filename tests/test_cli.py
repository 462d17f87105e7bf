"""The drop-in command line tool astc_cs_enc (reference: main.cpp:140-258).

CPU tests exercise its image reader through --dump-rgba (no GPU): PNGs of
every colour type and all five row filters written here with zlib, PAM, TGA
(grey / BGR / BGRA, raw and run-length encoded, either row order) and BMP
(24-bit padded rows, 32-bit, bit fields, either row order).
GPU tests run the full encode and compare the written .astc with the
library's blocks for the flipped image, and the reference's own leaf.astc.
"""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

CLI = os.path.join(ROOT, "astc_encoder_gb300", "_lib", "astc_cs_enc")


def _png(path, arr, ctype, depth=8, palette=None, trns=None):
    """Writes a PNG, cycling the row filter through 0..4."""
    h, w = arr.shape[:2]
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bps = depth // 8
    data = arr.reshape(h, w * chans).astype(np.uint16 if depth == 16 else np.uint8)
    if depth == 16:
        rows = data.astype(">u2").view(np.uint8).reshape(h, w * chans * 2)
    else:
        rows = data
    bpp = chans * bps
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for y in range(h):
        f = y % 5
        cur = rows[y].astype(np.int32)
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if f == 0:
            enc = cur
        elif f == 1:
            enc = cur - left
        elif f == 2:
            enc = cur - prev
        elif f == 3:
            enc = cur - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = abs(p - left), abs(p - prev), abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            enc = cur - pred
        out.append(f)
        out += (enc & 255).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        png += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        png += chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    png += chunk(b"IDAT", zlib.compress(bytes(out), 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as fh:
        fh.write(png)


def _dump(native, path, tmp_path):
    out = str(tmp_path / "dump.pam")
    r = subprocess.run([CLI, path, "--dump-rgba", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    from astc_encoder_gb300 import image_io
    return image_io.load_image(out)


@pytest.mark.parametrize("ctype", [0, 2, 3, 4, 6])
def test_cli_reads_every_png_colour_type(native, tmp_path, ctype):
    rng = np.random.default_rng(ctype)
    h, w = 37, 53
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    arr = rng.integers(0, 256, (h, w, chans), dtype=np.uint8)
    arr[5:20, 7:30] = arr[0, 0]                       # runs, so deflate emits matches
    palette = trns = None
    if ctype == 3:
        palette = rng.integers(0, 256, (256, 3))
        trns = rng.integers(0, 256, 200)
    path = str(tmp_path / "in.png")
    _png(path, arr, ctype, palette=palette, trns=trns)
    want = np.empty((h, w, 4), np.uint8)
    if ctype == 3:
        idx = arr[..., 0]
        want[..., :3] = palette.astype(np.uint8)[idx]
        a = np.full(256, 255, np.uint8)
        a[:len(trns)] = trns
        want[..., 3] = a[idx]
    elif chans >= 3:
        want[..., :3] = arr[..., :3]
        want[..., 3] = arr[..., 3] if chans == 4 else 255
    else:
        want[..., :3] = arr[..., :1]
        want[..., 3] = arr[..., 1] if chans == 2 else 255
    got = _dump(native, path, tmp_path)
    assert np.array_equal(got, want[::-1])            # flipped like main.cpp:24


def test_cli_reads_16bit_png_and_pam(native, tmp_path):
    rng = np.random.default_rng(9)
    arr = rng.integers(0, 65536, (20, 30, 4), dtype=np.uint16)
    path = str(tmp_path / "in16.png")
    _png(path, arr, 6, depth=16)
    got = _dump(native, path, tmp_path)
    assert np.array_equal(got, (arr >> 8).astype(np.uint8)[::-1])
    pam = tmp_path / "in.pam"
    img = rng.integers(0, 256, (11, 13, 4), dtype=np.uint8)
    pam.write_bytes(b"P7\nWIDTH 13\nHEIGHT 11\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n" + img.tobytes())
    assert np.array_equal(_dump(native, str(pam), tmp_path), img[::-1])


def _tga(path, arr, rle=False, top_down=False):
    """Writes a TGA: (h, w) grey, (h, w, 3) BGR or (h, w, 4) BGRA from RGB(A)."""
    h, w = arr.shape[:2]
    grey = arr.ndim == 2
    px = arr if grey else arr[..., [2, 1, 0] + ([3] if arr.shape[2] == 4 else [])]
    bpp = 8 if grey else 8 * arr.shape[2]
    rows = px if top_down else px[::-1]
    flat = rows.reshape(h * w, -1).astype(np.uint8)
    body = bytearray()
    if not rle:
        body += flat.tobytes()
    else:
        i = 0
        while i < len(flat):
            run = 1
            while i + run < len(flat) and run < 128 and np.array_equal(flat[i + run], flat[i]):
                run += 1
            if run > 1:
                body.append(0x80 | (run - 1))
                body += flat[i].tobytes()
                i += run
                continue
            lit = 1
            while i + lit < len(flat) and lit < 128 and not (
                    i + lit + 1 < len(flat) and np.array_equal(flat[i + lit], flat[i + lit + 1])):
                lit += 1
            body.append(lit - 1)
            body += flat[i:i + lit].tobytes()
            i += lit
    itype = (11 if rle else 3) if grey else (10 if rle else 2)
    head = struct.pack("<BBBHHBHHHHBB", 3, 0, itype, 0, 0, 0, 0, 0, w, h, bpp, 0x20 if top_down else 0)
    with open(path, "wb") as fh:
        fh.write(head + b"abc" + bytes(body))


def _bmp(path, arr, top_down=False, bitfields=False):
    """Writes a BMP from (h, w, 3) RGB (24-bit) or (h, w, 4) RGBA (32-bit)."""
    h, w, c = arr.shape
    bpp = 8 * c
    stride = (w * c + 3) & ~3
    rows = arr if top_down else arr[::-1]
    data = bytearray()
    for r in rows:
        line = r[:, [2, 1, 0] + ([3] if c == 4 else [])].astype(np.uint8).tobytes()
        data += line + b"\0" * (stride - len(line))
    masks = struct.pack("<IIII", 0x00FF0000, 0x0000FF00, 0x000000FF, 0xFF000000) if bitfields else b""
    hdr_size = 56 if bitfields else 40
    off = 14 + hdr_size
    info = struct.pack("<IiiHHIIiiII", hdr_size, w, -h if top_down else h, 1, bpp, 3 if bitfields else 0,
                       len(data), 2835, 2835, 0, 0) + masks
    with open(path, "wb") as fh:
        fh.write(b"BM" + struct.pack("<IHHI", off + len(data), 0, 0, off) + info + bytes(data))


@pytest.mark.parametrize("channels", [1, 3, 4])
@pytest.mark.parametrize("rle", [False, True])
@pytest.mark.parametrize("top_down", [False, True])
def test_cli_reads_tga(native, tmp_path, channels, rle, top_down):
    rng = np.random.default_rng(17 + channels)
    shape = (19, 23) if channels == 1 else (19, 23, channels)
    arr = rng.integers(0, 256, shape, dtype=np.uint8)
    arr[3:9, 2:15] = arr[3, 2]                          # runs for the RLE encoder
    path = str(tmp_path / "in.tga")
    _tga(path, arr, rle=rle, top_down=top_down)
    want = np.full((19, 23, 4), 255, np.uint8)
    if channels == 1:
        want[..., :3] = arr[..., None]
    else:
        want[..., :channels] = arr
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    assert np.array_equal(image_io.load_image(path), want)


@pytest.mark.parametrize("channels,bitfields", [(3, False), (4, False), (4, True)])
@pytest.mark.parametrize("top_down", [False, True])
def test_cli_reads_bmp(native, tmp_path, channels, bitfields, top_down):
    rng = np.random.default_rng(29 + channels)
    arr = rng.integers(0, 256, (13, 21, channels), dtype=np.uint8)     # 21 * 3 rows need padding
    path = str(tmp_path / "in.bmp")
    _bmp(path, arr, top_down=top_down, bitfields=bitfields)
    want = np.full((13, 21, 4), 255, np.uint8)
    want[..., :channels] = arr
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    assert np.array_equal(image_io.load_image(path), want)


def test_cli_rejects_unknown_format(native, tmp_path):
    path = tmp_path / "in.xyz"
    path.write_bytes(b"\x00\x01garbage")
    r = subprocess.run([CLI, str(path)], capture_output=True, text=True)
    assert r.returncode != 0 and "unsupported image format" in r.stdout


def test_cli_argument_errors(native, tmp_path):
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode != 0 and "wrong args count" in r.stdout
    r = subprocess.run([CLI, str(tmp_path / "missing.png")], capture_output=True, text=True)
    assert r.returncode != 0 and "load source texture failed" in r.stdout
    bad = tmp_path / "bad.png"
    bad.write_bytes(b"\x89PNG\r\n\x1a\n" + b"\x00" * 40)
    r = subprocess.run([CLI, str(bad), "--dump-rgba", str(tmp_path / "x.pam")], capture_output=True, text=True)
    assert r.returncode != 0


def test_cli_reads_reference_leaf(native, tmp_path, reference_dir):
    from astc_encoder_gb300 import image_io
    leaf = os.path.join(reference_dir, "textures", "leaf.png")
    got = _dump(native, leaf, tmp_path)
    assert np.array_equal(got, image_io.load_png(leaf)[::-1])


@pytest.mark.gpu
@pytest.mark.parametrize("flags,opts", [
    ([], dict(block_dim=4)),
    (["-alpha", "-4x4"], dict(block_dim=4, has_alpha=True)),
    (["-6x6", "-alpha", "-srgb"], dict(block_dim=6, has_alpha=True, srgb=True)),
    (["-norm", "-srgb"], dict(block_dim=4, is_normal=True)),          # sRGB ignored for -norm
    (["-6x6", "--clamp"], dict(block_dim=6, border=1)),
    (["-6x6", "-alpha", "--search"], dict(block_dim=6, has_alpha=True, quality=1)),
    (["--max-accumulation", "--search"], dict(block_dim=4, axis=1, quality=1)),
    (["-6x6", "-alpha", "-srgb", "--thorough"], dict(block_dim=6, has_alpha=True, srgb=True, quality=2)),
    (["--partitions"], dict(block_dim=4, quality=3)),
    (["-6x6", "--three-partitions"], dict(block_dim=6, quality=4)),
    (["-alpha", "--best-fit"], dict(block_dim=4, has_alpha=True, axis=2)),
    (["-6x6", "-alpha", "-srgb", "--best-fit", "--search"], dict(block_dim=6, has_alpha=True, srgb=True, axis=2,
                                                               quality=1)),
])
def test_cli_encode_matches_library(native, oracle, tmp_path, flags, opts):
    rng = np.random.default_rng(len(flags))
    img = rng.integers(0, 256, (45, 67, 4), dtype=np.uint8)
    img[10:30, 5:40] = (12, 200, 99, 255)
    src = str(tmp_path / "tex.v1.png")
    _png(src, img, 6)
    r = subprocess.run([CLI, src, *flags], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    dst = str(tmp_path / "tex.v1.astc")                 # last extension stripped
    assert "save astc to:" + dst in r.stdout
    blocks, bx, by, w, h = native.load_astc(dst)
    assert (bx, by, w, h) == (opts["block_dim"], opts["block_dim"], 67, 45)
    flipped = np.ascontiguousarray(img[::-1])
    assert np.array_equal(blocks, oracle.encode(flipped, **opts))


@pytest.mark.gpu
def test_cli_on_the_reference_fixture_crop(native, tmp_path):
    crops = np.load(os.path.join(GOLDEN, "leaf_crops.npz"))
    rgba = crops["crop0_rgba"]                        # already in the flipped orientation
    src = str(tmp_path / "crop.png")
    _png(src, rgba[::-1], 6)                          # store unflipped; the CLI flips it back
    r = subprocess.run([CLI, src, "-alpha", "-4x4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    blocks, *_ = native.load_astc(str(tmp_path / "crop.astc"))
    assert np.all(blocks == crops["crop0_blocks"], axis=1).mean() >= 0.97
