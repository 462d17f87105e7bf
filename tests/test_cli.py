"""The drop-in command line tool astc_cs_enc (reference: main.cpp:140-258).

CPU tests exercise its image reader through --dump-rgba (no GPU): PNGs of
every colour type and all five row filters written here with zlib, PAM, TGA
(grey / BGR / BGRA / 16-bit / colour-mapped, raw and run-length encoded,
either row order) and BMP
(1/4/8-bit palettes, 16-bit 5:5:5 and bit fields, 24-bit padded rows, 32-bit,
bit fields, either row order), and baseline
JPEG (grey and YCbCr at 4:4:4 / 4:2:2 / 4:4:0 / 4:2:0, restart intervals,
8- and 16-bit quantisation tables; baseline with one interleaved scan or one
scan per component, and progressive with spectral selection, successive
approximation and EOB runs) written here with scipy's orthonormal DCT and
Huffman tables built from the data, plus a third-party JPEG where one is
installed, PSD merged images (grey / RGB, alpha, 8 / 16 bits, raw and
PackBits, extra channels) and GIF first images (palettes, transparency,
interlacing, offset frames, a full 12-bit LZW table) with an LZW encoder
written here, Radiance HDR (flat and run-length scanlines) and Softimage PIC
(uncompressed, pure and mixed run-length packets).
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


def _png(path, arr, ctype, depth=8, palette=None, trns=None, interlace=False):
    """Writes a PNG of sample values `arr` (in the image's bit depth), cycling
    the row filter through 0..4; Adam7 passes when `interlace`."""
    h, w = arr.shape[:2]
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    data = arr.reshape(h, w, chans).astype(np.int64)
    passes = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
              (0, 1, 1, 2)] if interlace else [(0, 0, 1, 1)]
    bpp = max(1, chans * depth // 8)
    out, nrow = bytearray(), 0
    for x0, y0, dx, dy in passes:
        sub = data[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        ph, pw = sub.shape[:2]
        flat = sub.reshape(ph, pw * chans)
        if depth == 16:
            rows = flat.astype(">u2").view(np.uint8).reshape(ph, pw * chans * 2).astype(np.int32)
        elif depth == 8:
            rows = flat.astype(np.int32)
        else:
            bits = ((flat[..., None] >> np.arange(depth - 1, -1, -1)) & 1).astype(np.uint8)
            rows = np.packbits(bits.reshape(ph, -1), axis=1).astype(np.int32)
        prev = np.zeros(rows.shape[1], np.int32)
        for y in range(ph):
            f = nrow % 5
            nrow += 1
            cur = rows[y]
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
                pp = left + prev - upleft
                pa, pb, pc = abs(pp - left), abs(pp - prev), abs(pp - upleft)
                pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
                enc = cur - pred
            out.append(f)
            out += (enc & 255).astype(np.uint8).tobytes()
            prev = cur

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0,
                                                               1 if interlace else 0))
    if palette is not None:
        png += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        png += chunk(b"tRNS", bytes(trns) if isinstance(trns, (bytes, bytearray)) else trns.astype(np.uint8).tobytes())
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


@pytest.mark.parametrize("ctype,depth", [(0, 1), (0, 2), (0, 4), (3, 1), (3, 2), (3, 4)])
@pytest.mark.parametrize("interlace", [False, True])
def test_cli_reads_low_depth_png(native, tmp_path, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 10 + depth + 100 * interlace)
    h, w = 13, 19                                           # rows end mid-byte
    vals = rng.integers(0, 1 << depth, (h, w))
    path = str(tmp_path / "in.png")
    want = np.full((h, w, 4), 255, np.uint8)
    if ctype == 3:
        pal = rng.integers(0, 256, ((1 << depth), 3))
        trns = rng.integers(0, 256, max(1, (1 << depth) - 1))   # the last entry stays opaque
        _png(path, vals, 3, depth, palette=pal, trns=trns, interlace=interlace)
        want[..., :3] = pal[vals]
        alpha = np.full(1 << depth, 255)
        alpha[:len(trns)] = trns
        want[..., 3] = alpha[vals]
    else:
        _png(path, vals, 0, depth, interlace=interlace)
        want[..., :3] = (vals * (255 // ((1 << depth) - 1)))[..., None]
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    assert np.array_equal(image_io.load_image(path), want)


@pytest.mark.parametrize("ctype,depth", [(0, 8), (2, 8), (3, 8), (4, 8), (6, 8), (2, 16), (6, 16)])
@pytest.mark.parametrize("h,w", [(13, 11), (1, 1), (3, 9), (8, 8)])
def test_cli_reads_interlaced_png(native, tmp_path, ctype, depth, h, w):
    rng = np.random.default_rng(ctype + depth + h * w)
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    vals = rng.integers(0, 256 if ctype == 3 else 1 << depth, (h, w, chans))
    path = str(tmp_path / "in.png")
    want = np.full((h, w, 4), 255, np.uint8)
    hi = vals >> 8 if depth == 16 else vals
    if ctype == 3:
        pal = rng.integers(0, 256, (256, 3))
        _png(path, vals, 3, 8, palette=pal, interlace=True)
        want[..., :3] = pal[vals[..., 0]]
    else:
        _png(path, vals, ctype, depth, interlace=True)
        want[..., :3] = hi[..., :3] if chans >= 3 else hi[..., :1]
        if chans in (2, 4):
            want[..., 3] = hi[..., -1]
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


@pytest.mark.parametrize("ctype,depth", [(0, 8), (0, 2), (2, 8), (2, 16)])
def test_cli_png_transparency_key(native, tmp_path, ctype, depth):
    """tRNS for grey and RGB images: pixels equal to the key colour (in the
    image's own bit depth) are transparent."""
    rng = np.random.default_rng(ctype + depth)
    h, w, chans = 11, 14, 1 if ctype == 0 else 3
    vals = rng.integers(0, 1 << depth, (h, w, chans))
    key = vals[3, 4].copy()
    vals[7, 2:9] = key
    path = str(tmp_path / "in.png")
    _png(path, vals, ctype, depth, trns=b"".join(struct.pack(">H", int(k)) for k in key))
    want = np.full((h, w, 4), 255, np.uint8)
    scale = (lambda v: v >> 8) if depth == 16 else (lambda v: v * (255 // ((1 << depth) - 1)))
    want[..., :3] = scale(vals) if chans == 3 else scale(vals[..., :1])
    want[..., 3] = np.where((vals == key).all(-1), 0, 255)
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


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


def _tga_mapped(path, idx, colours, cbits, first=0, rle=False):
    """Writes a colour-mapped TGA: 8-bit indices into a 15/16/24/32-bit colour
    map (`colours` holds the stored entries).  The first-entry field is
    `first`, written as that many bytes ahead of the entries: stb_image (the
    reference's loader) skips that many bytes and then uses the indices as
    stored."""
    h, w = idx.shape
    cb = (cbits + 7) // 8
    head = struct.pack("<BBBHHBHHHHBB", 0, 1, 9 if rle else 1, first, len(colours), cbits, 0, 0, w, h, 8, 0x20)
    cmap = b"\xee" * first + b"".join(bytes(int(x) for x in c[:cb]) for c in colours)
    body = bytearray()
    for r in idx.astype(np.uint8):
        if rle:
            for v in r:                                     # one-pixel packets: raw (count 1)
                body += bytes([0, int(v)])
        else:
            body += r.tobytes()
    with open(path, "wb") as fh:
        fh.write(head + cmap + bytes(body))


def _tga16(path, v):
    h, w = v.shape
    head = struct.pack("<BBBHHBHHHHBB", 0, 0, 2, 0, 0, 0, 0, 0, w, h, 16, 0x20)
    with open(path, "wb") as fh:
        fh.write(head + v.astype("<u2").tobytes())


@pytest.mark.parametrize("cbits,rle,first", [(24, False, 0), (32, True, 5), (16, False, 2), (15, True, 0)])
def test_cli_reads_colour_mapped_tga(native, tmp_path, cbits, rle, first):
    rng = np.random.default_rng(cbits + rle)
    h, w, n = 11, 17, 40
    cb = (cbits + 7) // 8
    stored = rng.integers(0, 256, (n, cb))
    idx = rng.integers(0, n, (h, w))
    path = str(tmp_path / "in.tga")
    _tga_mapped(path, idx, stored, cbits, first, rle)
    if cb == 2:
        v = stored[:, 0] | (stored[:, 1] << 8)
        table = np.stack([((v >> s) & 31) * 255 // 31 for s in (10, 5, 0)] + [np.full(n, 255)], -1)
    else:
        table = np.full((n, 4), 255)
        table[:, :3] = stored[:, [2, 1, 0]]
        if cb == 4:
            table[:, 3] = stored[:, 3]
    want = table[idx].astype(np.uint8)
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


def test_tga_colour_map_rules_of_the_reference_loader(native, tmp_path):
    """An index past the colour map takes entry 0; a colour map in an
    unmapped (true-colour) file is skipped."""
    from astc_encoder_gb300 import image_io
    colours = np.array([[10, 20, 30], [40, 50, 60], [70, 80, 90]])
    idx = np.array([[0, 1, 2, 3], [200, 2, 1, 0]])
    path = str(tmp_path / "m.tga")
    _tga_mapped(path, idx, colours, 24)
    table = colours[:, [2, 1, 0]]
    want = np.full((2, 4, 4), 255, np.uint8)
    want[..., :3] = table[np.where(idx < 3, idx, 0)]
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    assert np.array_equal(image_io.load_image(path), want)
    # true colour with a (useless) 2-entry 24-bit colour map before the pixels
    arr = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3)
    head = struct.pack("<BBBHHBHHHHBB", 0, 1, 2, 0, 2, 24, 0, 0, 3, 2, 24, 0x20)
    with open(path, "wb") as fh:
        fh.write(head + bytes(6) + arr[..., [2, 1, 0]].tobytes())
    want = np.full((2, 3, 4), 255, np.uint8)
    want[..., :3] = arr
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    assert np.array_equal(image_io.load_image(path), want)


def test_bmp_all_zero_alpha_reads_opaque(native, tmp_path):
    """32-bit BI_RGB (BGRX) files with every fourth byte 0 read as opaque, as
    stb_image reads them; one nonzero alpha byte keeps the alpha."""
    from astc_encoder_gb300 import image_io
    rng = np.random.default_rng(3)
    arr = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    arr[..., 3] = 0
    path = str(tmp_path / "x.bmp")
    _bmp(path, arr)
    want = arr.copy()
    want[..., 3] = 255
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    assert np.array_equal(image_io.load_image(path), want)
    arr[2, 3, 3] = 1
    _bmp(path, arr)
    assert np.array_equal(_dump(native, path, tmp_path), arr[::-1])
    assert np.array_equal(image_io.load_image(path), arr)


def test_pic_pure_runs_cut_at_the_row_end(native, tmp_path):
    """Pure run-length PIC packets: a run past the end of the row is cut to
    the row, an empty run reads its value and adds no pixels."""
    from astc_encoder_gb300 import image_io
    w, h = 5, 2
    head = b"\x53\x80\xf6\x34" + struct.pack(">f", 3.71) + b"".ljust(80, b"\0")
    head += b"PICT" + struct.pack(">HHfHH", w, h, 1.0, 3, 0) + bytes([0, 8, 1, 0xF0])
    body = bytes([0, 1, 2, 3, 4]) + bytes([3, 9, 9, 9, 9]) + bytes([200, 7, 7, 7, 7])   # row 0: 0 + 3 + 2
    body += bytes([255, 5, 6, 7, 8])                                                      # row 1: 255 -> 5
    path = str(tmp_path / "r.pic")
    with open(path, "wb") as fh:
        fh.write(head + body)
    want = np.zeros((h, w, 4), np.uint8)
    want[0, :3] = (9, 9, 9, 9)
    want[0, 3:] = (7, 7, 7, 7)
    want[1, :] = (5, 6, 7, 8)
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    assert np.array_equal(image_io.load_image(path), want)


def test_cli_reads_16bit_tga(native, tmp_path):
    v = np.random.default_rng(9).integers(0, 1 << 16, (7, 13))
    path = str(tmp_path / "in.tga")
    _tga16(path, v)
    want = np.full((7, 13, 4), 255, np.uint8)
    for c, sh in enumerate((10, 5, 0)):
        want[..., c] = ((v >> sh) & 31) * 255 // 31
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


def _pic(path, rgba, packets):
    """Writes a Softimage PIC; packets: (type, channel mask) with type 0
    uncompressed, 1 pure run-length, 2 mixed run-length."""
    h, w = rgba.shape[:2]
    head = b"\x53\x80\xf6\x34" + struct.pack(">f", 3.71) + b"written by the test suite".ljust(80, b"\0")
    head += b"PICT" + struct.pack(">HHfHH", w, h, 1.0, 3, 0)
    head += b"".join(bytes([1 if i + 1 < len(packets) else 0, 8, t, m]) for i, (t, m) in enumerate(packets))
    body = bytearray()
    for y in range(h):
        for t, m in packets:
            chans = [c for c in range(4) if m & (0x80 >> c)]
            px = [bytes(int(v) for v in rgba[y, x, chans]) for x in range(w)]
            x = 0
            while x < w:
                run = 1
                while x + run < w and px[x + run] == px[x] and run < 300:
                    run += 1
                if t == 0:
                    body += px[x]
                    x += 1
                elif t == 1:
                    run = min(run, 255)
                    body += bytes([run]) + px[x]
                    x += run
                elif run >= 2:
                    body += (bytes([128]) + struct.pack(">H", run) if run > 128 else bytes([run + 127])) + px[x]
                    x += run
                else:
                    k = x
                    while k < w and k - x < 128 and not (k + 1 < w and px[k + 1] == px[k]):
                        k += 1
                    k = max(k, x + 1)
                    body += bytes([k - x - 1]) + b"".join(px[x:k])
                    x = k
    with open(path, "wb") as fh:
        fh.write(head + bytes(body))


@pytest.mark.parametrize("packets", [[(0, 0xF0)], [(2, 0xE0), (1, 0x10)], [(1, 0xE0)], [(2, 0xF0)],
                                     [(0, 0x80), (2, 0x40), (1, 0x30)]])
def test_cli_reads_pic(native, tmp_path, packets):
    rng = np.random.default_rng(len(packets) * 7 + packets[0][0])
    h, w = 9, 310                                           # a run longer than 128 takes the 16-bit count
    rgba = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    rgba[2:6, 10:200] = rgba[2, 10]
    rgba[7, :] = (9, 8, 7, 6)
    path = str(tmp_path / "in.pic")
    _pic(path, rgba, packets)
    want = np.full((h, w, 4), 255, np.uint8)
    for _, m in packets:
        for c in range(4):
            if m & (0x80 >> c):
                want[..., c] = rgba[..., c]
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


def _bmp_indexed(path, idx, palette, bpp, used=0, top_down=False):
    """Writes a 1/4/8-bit palette BMP (indices MSB-first, rows padded to 4 bytes)."""
    h, w = idx.shape
    stride = ((w * bpp + 31) // 32) * 4
    rows = idx if top_down else idx[::-1]
    data = bytearray()
    for r in rows:
        bits = ((r[:, None] >> np.arange(bpp - 1, -1, -1)) & 1).astype(np.uint8).reshape(-1)
        line = np.packbits(bits).tobytes()
        data += line + b"\0" * (stride - len(line))
    n = used or (1 << bpp)
    pal = b"".join(bytes([int(c[2]), int(c[1]), int(c[0]), 0]) for c in palette[:n])
    off = 14 + 40 + len(pal)
    info = struct.pack("<IiiHHIIiiII", 40, w, -h if top_down else h, 1, bpp, 0, len(data), 2835, 2835, used, 0)
    with open(path, "wb") as fh:
        fh.write(b"BM" + struct.pack("<IHHI", off + len(data), 0, 0, off) + info + pal + bytes(data))


def _bmp16(path, v, masks=None):
    """Writes a 16-bit BMP of raw 16-bit pixel values (5:5:5, or bit fields)."""
    h, w = v.shape
    stride = ((w * 16 + 31) // 32) * 4
    data = bytearray()
    for r in v[::-1]:
        line = r.astype("<u2").tobytes()
        data += line + b"\0" * (stride - len(line))
    extra = struct.pack("<III", *masks) if masks else b""
    off = 14 + 40 + len(extra)
    info = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 16, 3 if masks else 0, len(data), 2835, 2835, 0, 0) + extra
    with open(path, "wb") as fh:
        fh.write(b"BM" + struct.pack("<IHHI", off + len(data), 0, 0, off) + info + bytes(data))


@pytest.mark.parametrize("bpp,used,top_down", [(1, 0, False), (4, 0, True), (4, 11, False), (8, 0, False),
                                               (8, 200, True)])
def test_cli_reads_palette_bmp(native, tmp_path, bpp, used, top_down):
    rng = np.random.default_rng(bpp * 7 + used)
    h, w = 13, 21                                           # odd widths: padded, partial bytes
    n = used or (1 << bpp)
    palette = rng.integers(0, 256, (n, 3))
    idx = rng.integers(0, n, (h, w))
    path = str(tmp_path / "in.bmp")
    _bmp_indexed(path, idx, palette, bpp, used, top_down)
    want = np.full((h, w, 4), 255, np.uint8)
    want[..., :3] = palette[idx]
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


@pytest.mark.parametrize("masks", [None, (0xF800, 0x07E0, 0x001F)])
def test_cli_reads_16bit_bmp(native, tmp_path, masks):
    rng = np.random.default_rng(16 + (masks is not None))
    h, w = 9, 15
    v = rng.integers(0, 1 << 16, (h, w))
    path = str(tmp_path / "in.bmp")
    _bmp16(path, v, masks)
    want = np.full((h, w, 4), 255, np.uint8)
    for c, m in enumerate(masks or (0x7C00, 0x03E0, 0x001F)):
        shift = (m & -m).bit_length() - 1
        n = bin(m >> shift).count("1")
        x = (v & m) >> shift
        # the field's bits repeated, cut to 8: the binary fraction x / (2^n - 1)
        want[..., c] = np.minimum(255, (x * 256) // ((1 << n) - 1))
    assert np.array_equal(_dump(native, path, tmp_path), want[::-1])
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(path), want)


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


# T.81 zig-zag: anti-diagonals in turn, odd ones walked down, even ones up
ZIGZAG = np.array(sorted(range(64), key=lambda i: (i // 8 + i % 8,
                                                    (i // 8) if (i // 8 + i % 8) % 2 else (i % 8))))


def _huffman_table(freq):
    """Canonical Huffman code (lengths <= 16) for {symbol: count}; a dummy
    symbol of count 0 takes the all-ones code, which T.81 reserves."""
    import heapq
    freq = dict(freq)
    while True:
        heap = [(f, i, [s]) for i, (s, f) in enumerate(sorted(freq.items()))] + [(0, -1, [256])]
        heapq.heapify(heap)
        length = {s: 0 for s in list(freq) + [256]}
        n = len(heap)
        while len(heap) > 1:
            fa, _, a = heapq.heappop(heap)
            fb, _, b = heapq.heappop(heap)
            for s in a + b:
                length[s] += 1
            heapq.heappush(heap, (fa + fb, n, a + b))
            n += 1
        if max(length.values()) <= 16:
            break
        freq = {s: f // 2 + 1 for s, f in freq.items()}
    order = sorted(length, key=lambda s: (length[s], s))
    codes, code, prev = {}, 0, length[order[0]]
    for s in order:
        code <<= length[s] - prev
        prev = length[s]
        codes[s] = (code, length[s])
        code += 1
    counts = [sum(1 for s in order if length[s] == n and s != 256) for n in range(1, 17)]
    return codes, bytes(counts) + bytes(s for s in order if s != 256)


def _jpeg_coefs(img, sampling=(1, 1)):
    """Quantised DCT coefficients of img ((H, W) grey or (H, W, 3) RGB) and the
    decoded image a conforming decoder gives (float64, rounded), as RGBA."""
    from scipy.fft import dctn, idctn
    h, w = img.shape[:2]
    x = img.astype(np.float64)
    if img.ndim == 2:
        planes, samp = [x], [(1, 1)]
        sampling = (1, 1)
    else:
        r, g, b = x[..., 0], x[..., 1], x[..., 2]
        planes = [0.299 * r + 0.587 * g + 0.114 * b,
                  -0.168736 * r - 0.331264 * g + 0.5 * b + 128.0,
                  0.5 * r - 0.418688 * g - 0.081312 * b + 128.0]
        samp = [sampling, (1, 1), (1, 1)]
    hmax, vmax = sampling
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    u = np.arange(8)
    qts = [2 + (u[:, None] + u[None, :]) // 2, 3 + (u[:, None] + u[None, :])]   # luma, chroma
    coefs, recon = [], []
    for ci, (p, (sh, sv)) in enumerate(zip(planes, samp)):
        full = np.pad(p, ((0, mcuy * 8 * vmax - h), (0, mcux * 8 * hmax - w)), mode="edge")
        fy, fx = vmax // sv, hmax // sh
        sub = full.reshape(full.shape[0] // fy, fy, full.shape[1] // fx, fx).mean(axis=(1, 3))
        bl = (sub - 128.0).reshape(sub.shape[0] // 8, 8, sub.shape[1] // 8, 8).transpose(0, 2, 1, 3)
        q = qts[min(ci, 1)]
        c = np.rint(dctn(bl, axes=(2, 3), norm="ortho") / q).astype(np.int64)
        coefs.append(c.reshape(c.shape[0], c.shape[1], 64))
        pix = np.clip(np.floor(idctn(c * q, axes=(2, 3), norm="ortho") + 128.5), 0, 255)
        plane = pix.transpose(0, 2, 1, 3).reshape(sub.shape)
        recon.append(plane[np.arange(h) * sv // vmax][:, np.arange(w) * sh // hmax])
    want = np.full((h, w, 4), 255, np.uint8)
    if img.ndim == 2:
        want[..., :3] = recon[0][..., None]
    else:
        yy, cb, cr = recon[0], recon[1] - 128.0, recon[2] - 128.0
        rgb = np.stack([yy + 1.402 * cr, yy - 0.344136 * cb - 0.714136 * cr, yy + 1.772 * cb], -1)
        want[..., :3] = np.clip(np.floor(rgb + 0.5), 0, 255)
    cbw = [(-(-w * sh // hmax) + 7) // 8 for sh, _ in samp]
    cbh = [(-(-h * sv // vmax) + 7) // 8 for _, sv in samp]
    return dict(h=h, w=w, samp=samp, coefs=coefs, qts=qts, want=want, mcux=mcux, mcuy=mcuy, cbw=cbw, cbh=cbh)


def _cat(v):
    return 0 if v == 0 else abs(int(v)).bit_length()


def _extra(v, t):
    return v if v >= 0 else v + (1 << t) - 1


class _ScanEvents:
    """The symbols and raw bits of one scan, in stream order: ('s', table, symbol),
    ('b', value, nbits) or ('rst',)."""

    def __init__(self):
        self.ev, self.eobrun, self.be = [], 0, []

    def sym(self, tab, v):
        self.ev.append(("s", tab, v))

    def bits(self, v, n):
        if n:
            self.ev.append(("b", v, n))

    def flush_eobrun(self, tab):
        if self.eobrun:
            nb = self.eobrun.bit_length() - 1
            self.sym(tab, nb << 4)
            self.bits(self.eobrun - (1 << nb), nb)
            for bit in self.be:
                self.bits(bit, 1)
            self.eobrun, self.be = 0, []


def _scan_events(J, comps, ss, se, ah, al, progressive, restart):
    """One scan over `comps` (indices) in the decoder's block order."""
    sc = _ScanEvents()
    single = len(comps) == 1
    units = J["cbw"][comps[0]] * J["cbh"][comps[0]] if single else J["mcux"] * J["mcuy"]
    pred = {ci: 0 for ci in comps}
    act = ("ac", min(comps[0], 1))

    def blocks(u):
        for ci in comps:
            if single:
                yield ci, J["coefs"][ci][u // J["cbw"][ci], u % J["cbw"][ci]]
                continue
            sh, sv = J["samp"][ci]
            my, mx = divmod(u, J["mcux"])
            for by in range(sv):
                for bx in range(sh):
                    yield ci, J["coefs"][ci][my * sv + by, mx * sh + bx]

    for u in range(units):
        if restart and u and u % restart == 0:
            sc.flush_eobrun(act)
            sc.ev.append(("rst",))
            pred = {ci: 0 for ci in comps}
        for ci, blk in blocks(u):
            zz = [int(v) for v in blk[ZIGZAG]]
            dct = ("dc", min(ci, 1))
            if not progressive or ss == 0:
                if ah == 0:                                   # DC (sequential or first)
                    v = zz[0] >> al
                    diff = v - pred[ci]
                    pred[ci] = v
                    sc.sym(dct, _cat(diff))
                    sc.bits(_extra(diff, _cat(diff)), _cat(diff))
                else:                                         # DC refinement
                    sc.bits((zz[0] >> al) & 1, 1)
                if progressive:
                    continue
                run, acti = 0, ("ac", min(ci, 1))
                last = max([k for k in range(1, 64) if zz[k]] or [0])
                for k in range(1, last + 1):
                    if zz[k] == 0:
                        run += 1
                        continue
                    while run > 15:
                        sc.sym(acti, 0xF0)
                        run -= 16
                    sz = _cat(zz[k])
                    sc.sym(acti, (run << 4) | sz)
                    sc.bits(_extra(zz[k], sz), sz)
                    run = 0
                if last < 63:
                    sc.sym(acti, 0x00)
                continue
            band = range(ss, se + 1)
            if ah == 0:                                       # AC first: magnitudes >> al
                vals = [(abs(zz[k]) >> al) * (1 if zz[k] >= 0 else -1) for k in band]
                run = 0
                for v in vals:
                    if v == 0:
                        run += 1
                        continue
                    sc.flush_eobrun(act)
                    while run > 15:
                        sc.sym(act, 0xF0)
                        run -= 16
                    sz = _cat(v)
                    sc.sym(act, (run << 4) | sz)
                    sc.bits(_extra(v, sz), sz)
                    run = 0
                if run:
                    sc.eobrun += 1
                    if sc.eobrun == 0x7FFF:
                        sc.flush_eobrun(act)
                continue
            # AC refinement (T.81 G.1.2.3, figure G.7)
            absv = [abs(zz[k]) >> al for k in band]
            eob = max([i for i, a in enumerate(absv) if a == 1] or [-1])
            run, br = 0, []
            for i, a in enumerate(absv):
                if a == 0:
                    run += 1
                    continue
                while run > 15 and i <= eob:
                    sc.flush_eobrun(act)
                    sc.sym(act, 0xF0)
                    run -= 16
                    for bit in br:
                        sc.bits(bit, 1)
                    br = []
                if a > 1:                                     # already nonzero: a correction bit
                    br.append(a & 1)
                    continue
                sc.flush_eobrun(act)
                sc.sym(act, (run << 4) | 1)
                sc.bits(1 if zz[ss + i] > 0 else 0, 1)
                for bit in br:
                    sc.bits(bit, 1)
                br, run = [], 0
            if run or br:
                sc.eobrun += 1
                sc.be += br
                if sc.eobrun == 0x7FFF:
                    sc.flush_eobrun(act)
    sc.flush_eobrun(act)
    return sc.ev


def _jpeg_write(path, J, mode="baseline", restart=0, q16=False):
    """Writes the coefficients of _jpeg_coefs as a JPEG: 'baseline' (one
    interleaved scan), 'baseline_split' (one scan per component) or
    'progressive' (spectral selection and successive approximation, with
    DC and AC refinement scans)."""
    ncomp = len(J["coefs"])
    if mode == "baseline":
        script = [(list(range(ncomp)), 0, 63, 0, 0)]
    elif mode == "baseline_split":
        script = [([ci], 0, 63, 0, 0) for ci in range(ncomp)]
    else:
        allc = list(range(ncomp))
        script = [(allc, 0, 0, 0, 1)]                                 # DC first, point transform 1
        script += [([0], 1, 5, 0, 2), ([0], 6, 63, 0, 2)]              # luma AC bands, two bits dropped
        script += [([ci], 1, 63, 0, 1) for ci in range(1, ncomp)]      # chroma AC, one bit dropped
        script += [([0], 1, 63, 2, 1)]                                # luma AC refinement, bit 1
        script += [(allc, 0, 0, 1, 0)]                                # DC refinement
        script += [([ci], 1, 63, 1, 0) for ci in range(ncomp)]        # AC refinement, bit 0
    progressive = mode == "progressive"

    def seg(marker, body):
        return b"\xff" + bytes([marker]) + struct.pack(">H", len(body) + 2) + body
    out = b"\xff\xd8" + seg(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    out += seg(0xFE, b"written by the test suite")
    for t, q in enumerate(J["qts"][:min(ncomp, 2)]):
        zq = q.reshape(64)[ZIGZAG]
        out += seg(0xDB, bytes([(16 if q16 else 0) | t]) +
                   (struct.pack(">64H", *zq) if q16 else bytes(zq.astype(np.uint8))))
    out += seg(0xC2 if progressive else 0xC0, struct.pack(">BHHB", 8, J["h"], J["w"], ncomp) +
               b"".join(bytes([ci + 1, (sh << 4) | sv, min(ci, 1)]) for ci, (sh, sv) in enumerate(J["samp"])))
    if restart:
        out += seg(0xDD, struct.pack(">H", restart))
    for comps, ss, se, ah, al in script:
        ev = _scan_events(J, comps, ss, se, ah, al, progressive, restart)
        freq = {}
        for e in ev:
            if e[0] == "s":
                freq.setdefault(e[1], {}).setdefault(e[2], 0)
                freq[e[1]][e[2]] += 1
        tables = {key: _huffman_table(f) for key, f in freq.items()}
        for (cls, t), (codes, spec) in sorted(tables.items()):
            out += seg(0xC4, bytes([(1 if cls == "ac" else 0) << 4 | t]) + spec)
        out += seg(0xDA, bytes([len(comps)]) + b"".join(bytes([ci + 1, (min(ci, 1) << 4) | min(ci, 1)])
                                                         for ci in comps) + bytes([ss, se, (ah << 4) | al]))
        parts, cur, nrst = [], [], 0
        for e in ev + [("rst",)]:
            if e[0] == "rst":
                bitstr = "".join(cur)
                bitstr += "1" * (-len(bitstr) % 8)
                parts.append(int(bitstr, 2).to_bytes(len(bitstr) // 8, "big") if bitstr else b"")
                cur = []
            elif e[0] == "s":
                code, n = tables[e[1]][0][e[2]]
                cur.append(format(code, "0%db" % n))
            else:
                cur.append(format(e[1], "0%db" % e[2]))
        for i, data in enumerate(parts):
            out += data.replace(b"\xff", b"\xff\x00")
            if i + 1 < len(parts):
                out += bytes([0xFF, 0xD0 + i % 8])
    out += b"\xff\xd9"
    with open(path, "wb") as fh:
        fh.write(out)


def _jpeg(path, img, sampling=(1, 1), restart=0, q16=False, mode="baseline"):
    """Writes img as a JPEG and returns what a conforming decoder gives."""
    J = _jpeg_coefs(img, sampling)
    _jpeg_write(path, J, mode=mode, restart=restart, q16=q16)
    return J["want"]


def _smooth(h, w, channels, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    chans = [128 + 90 * np.sin(xx / (5 + 3 * c) + yy / (7 + c) + c) + rng.normal(0, 4, (h, w))
             for c in range(channels)]
    arr = np.clip(np.rint(np.stack(chans, -1)), 0, 255).astype(np.uint8)
    return arr[..., 0] if channels == 1 else arr


def test_jpeg_zigzag_tables():
    """The readers' zig-zag order against the anti-diagonal walk of T.81 Figure 5."""
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io._ZIGZAG, ZIGZAG)
    src = open(os.path.join(ROOT, "astc_encoder_gb300", "csrc", "image_load.cpp")).read()
    body = src[src.index("kZigzag[64] = {") + 15:]
    table = [int(v) for v in body[:body.index("}")].replace("\n", " ").split(",")]
    assert table == list(ZIGZAG)


@pytest.mark.parametrize("kind,sampling,restart,q16", [
    ("grey", (1, 1), 0, False), ("grey", (1, 1), 5, True), ("rgb", (1, 1), 0, False),
    ("rgb", (2, 2), 0, False), ("rgb", (2, 1), 3, False), ("rgb", (1, 2), 1, True),
    ("rgb", (2, 2), 2, False)])
def test_cli_reads_jpeg(native, tmp_path, kind, sampling, restart, q16):
    img = _smooth(37, 29, 1 if kind == "grey" else 3, seed=sum(sampling) + restart)
    path = str(tmp_path / "in.jpg")
    want = _jpeg(path, img, sampling=sampling, restart=restart, q16=q16)
    got = _dump(native, path, tmp_path)[::-1]
    assert np.abs(got.astype(int) - want).max() <= 1          # float32 against float64 rounding
    assert np.mean(got != want) < 0.01
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    py = image_io.load_image(path)
    assert np.abs(py.astype(int) - want).max() <= 1 and np.mean(py != want) < 0.01
    ref = np.dstack([img] * 3) if kind == "grey" else img   # and the picture is the input's
    mse = np.mean((got[..., :3].astype(float) - ref) ** 2)
    assert 10 * np.log10(255.0 ** 2 / mse) > (33 if sampling == (1, 1) else 25)


def test_cli_reads_third_party_jpeg(native, tmp_path):
    """A baseline JPEG from another encoder (APPn segments, its own tables)."""
    sample = None
    try:
        import sklearn
        sample = os.path.join(os.path.dirname(sklearn.__file__), "datasets", "images", "china.jpg")
    except ImportError:
        pass
    if sample is None or not os.path.exists(sample):
        pytest.skip("no third-party JPEG sample here")
    got = _dump(native, sample, tmp_path)[::-1]
    from astc_encoder_gb300 import image_io
    py = image_io.load_image(sample)
    assert got.shape == (427, 640, 4) and np.abs(py.astype(int) - got).max() <= 1
    assert np.mean(py != got) < 0.01 and (got[..., 3] == 255).all()
    # a coherent decode: neighbours agree far better than chance, and the 8x8
    # block boundaries are no rougher than block interiors (a misplaced
    # coefficient or a wrong transform shows as block edges)
    dx = np.abs(np.diff(got[..., :3].astype(int), axis=1)).mean(axis=(0, 2))
    edges, inner = dx[7::8].mean(), np.delete(dx, np.arange(7, dx.size, 8)).mean()
    assert dx.mean() < 0.3 * got[..., :3].std() and edges < 1.15 * inner


@pytest.mark.parametrize("kind,sampling,restart,mode", [
    ("rgb", (2, 2), 0, "progressive"), ("rgb", (1, 1), 0, "progressive"), ("rgb", (2, 1), 3, "progressive"),
    ("grey", (1, 1), 4, "progressive"), ("rgb", (1, 2), 1, "progressive"), ("rgb", (2, 2), 2, "baseline_split"),
    ("rgb", (1, 1), 0, "baseline_split")])
def test_cli_reads_progressive_and_single_component_scans(native, tmp_path, kind, sampling, restart, mode):
    """The same coefficients written as one interleaved baseline scan and as
    `mode` (progressive: DC and AC first scans with point transforms, band
    splits, AC and DC refinement scans, EOB runs; or one baseline scan per
    component) decode to the same pixels."""
    img = _smooth(45, 38, 1 if kind == "grey" else 3, seed=7 + restart + sampling[0])
    J = _jpeg_coefs(img, sampling)
    base, other = str(tmp_path / "base.jpg"), str(tmp_path / "other.jpg")
    _jpeg_write(base, J, mode="baseline")
    _jpeg_write(other, J, mode=mode, restart=restart)
    got_base = _dump(native, base, tmp_path)
    got = _dump(native, other, tmp_path)
    assert np.array_equal(got, got_base)
    assert np.abs(got[::-1].astype(int) - J["want"]).max() <= 1
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    assert np.array_equal(image_io.load_image(other), image_io.load_image(base))


@pytest.mark.parametrize("restart", [0, 7])
def test_cli_reads_progressive_long_eob_runs(native, tmp_path, restart):
    """A smooth image: whole AC bands are zero, so EOB runs span the scan
    (run-length symbols up to 2^8 with appended bits)."""
    yy, xx = np.mgrid[0:160, 0:192].astype(np.float64)
    img = np.clip(np.rint(np.stack([40 + xx * 0.5, 60 + yy * 0.4, 200 - xx * 0.3], -1)), 0, 255).astype(np.uint8)
    img[40:56, 64:96] = [250, 20, 20]
    J = _jpeg_coefs(img, (2, 2))
    base, prog = str(tmp_path / "base.jpg"), str(tmp_path / "prog.jpg")
    _jpeg_write(base, J, mode="baseline")
    _jpeg_write(prog, J, mode="progressive", restart=restart)
    assert np.array_equal(_dump(native, prog, tmp_path), _dump(native, base, tmp_path))
    from astc_encoder_gb300 import image_io
    assert np.array_equal(image_io.load_image(prog), image_io.load_image(base))


def test_cli_refuses_unsupported_jpeg(native, tmp_path):
    path = str(tmp_path / "in.jpg")
    _jpeg(path, _smooth(16, 16, 3, 0))
    good = open(path, "rb").read()
    from astc_encoder_gb300 import image_io
    # a progressive frame whose scan carries sequential parameters; an arithmetic-coded frame
    for marker, msg in ((b"\xff\xc2", "bad JPEG scan parameters"), (b"\xff\xc9", "arithmetic")):
        open(path, "wb").write(good.replace(b"\xff\xc0", marker, 1))
        r = subprocess.run([CLI, path, "--dump-rgba", str(tmp_path / "o.pam")], capture_output=True, text=True)
        assert r.returncode != 0 and msg in r.stdout
        with pytest.raises(ValueError, match=msg):
            image_io.load_image(path)


@pytest.mark.parametrize("fmt", ["png", "jpg", "bmp", "tga", "pam"])
def test_cli_survives_corrupt_images(native, tmp_path, fmt):
    """Mutated, truncated and extended files: the reader returns an image or an
    error, never a crash, and never spends more than the file's size on work."""
    rng = np.random.default_rng(["png", "jpg", "bmp", "tga", "pam"].index(fmt))
    arr = _smooth(21, 27, 3, 5)
    rgba = np.dstack([arr, np.full(arr.shape[:2], 200, np.uint8)])
    path = str(tmp_path / ("in." + fmt))
    if fmt == "png":
        _png(path, rgba, 6)
    elif fmt == "jpg":
        _jpeg(path, arr, sampling=(2, 2), restart=2)
    elif fmt == "bmp":
        _bmp(path, rgba)
    elif fmt == "tga":
        _tga(path, rgba, rle=True)
    else:
        with open(path, "wb") as fh:
            fh.write(b"P7\nWIDTH 27\nHEIGHT 21\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n" + rgba.tobytes())
    good = open(path, "rb").read()
    for trial in range(60):
        data = bytearray(good)
        kind = trial % 4
        if kind == 0:                                   # flip bytes anywhere
            for i in rng.integers(0, len(data), 1 + trial % 5):
                data[i] = int(rng.integers(0, 256))
        elif kind == 1:                                 # flip bytes in the header
            for i in rng.integers(0, min(len(data), 64), 1 + trial % 3):
                data[i] = int(rng.integers(0, 256))
        elif kind == 2:                                 # truncate
            data = data[:int(rng.integers(1, len(data)))]
        else:                                           # splice in garbage
            i = int(rng.integers(0, len(data)))
            data[i:i] = rng.integers(0, 256, int(rng.integers(1, 40)), dtype=np.uint8).tobytes()
        bad = str(tmp_path / ("bad." + fmt))
        with open(bad, "wb") as fh:
            fh.write(bytes(data))
        r = subprocess.run([CLI, bad, "--dump-rgba", str(tmp_path / "o.pam")], capture_output=True,
                           text=True, timeout=60)
        assert r.returncode in (0, 255), (trial, r.returncode, r.stdout[-300:], r.stderr[-300:])
        assert r.returncode == 0 or "load source texture failed" in r.stdout


def test_image_reader_under_sanitizers(tmp_path):
    """The reader built with ASan + UBSan over 400 mutated files of every format."""
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "fuzz")
    csrc = os.path.join(ROOT, "astc_encoder_gb300", "csrc")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=undefined", "-I", csrc,
                        os.path.join(ROOT, "tests", "image_fuzz_main.cpp"), os.path.join(csrc, "image_load.cpp"),
                        "-o", exe], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime unavailable: " + r.stderr[-200:])
    arr = _smooth(21, 27, 3, 5)
    rgba = np.dstack([arr, np.full(arr.shape[:2], 200, np.uint8)])
    seeds = []
    for name, write in [("a.png", lambda p: _png(p, rgba, 6)), ("b.png", lambda p: _png(p, arr[..., 0], 3,
                                                                                         palette=np.arange(768) % 256)),
                        ("c.jpg", lambda p: _jpeg(p, arr, sampling=(2, 2), restart=2)),
                        ("d.jpg", lambda p: _jpeg(p, arr[..., 0])),
                        ("j.jpg", lambda p: _jpeg(p, arr, sampling=(2, 1), restart=3, mode="progressive")),
                        ("k.psd", lambda p: _psd(p, rgba.transpose(2, 0, 1).copy(), 3, 16, True, 1)),
                        ("l.psd", lambda p: _psd(p, rgba[..., :2].transpose(2, 0, 1).copy(), 1, 8, False)),
                        ("m.gif", lambda p: _gif(p, (arr[..., 0] // 16).astype(np.int64),
                                                 np.arange(48, dtype=np.uint8).reshape(16, 3) * 5,
                                                 transparent=3, interlace=True)),
                        ("n.hdr", lambda p: _hdr(p, np.dstack([arr, np.full(arr.shape[:2], 130, np.uint8)]))),
                        ("o.png", lambda p: _png(p, (arr[..., 0] // 64).astype(np.int64), 3, 2,
                                                 palette=np.arange(12).reshape(4, 3) * 20,
                                                 trns=np.array([0, 128]), interlace=True)),
                        ("q.png", lambda p: _png(p, arr.astype(np.int64) * 257, 2, 16,
                                                 trns=b"\x00\x01\x00\x02\x00\x03", interlace=True)),
                        ("t.tga", lambda p: _tga_mapped(p, (arr[..., 2] // 8).astype(np.int64),
                                                        np.arange(96).reshape(32, 3), 24, 3, True)),
                        ("u.pic", lambda p: _pic(p, rgba, [(2, 0xE0), (1, 0x10)])),
                        ("r.bmp", lambda p: _bmp_indexed(p, (arr[..., 1] // 16).astype(np.int64),
                                                         np.arange(48).reshape(16, 3) * 5, 4)),
                        ("s.bmp", lambda p: _bmp16(p, arr[..., 0].astype(np.int64) * 200, (0xF800, 0x07E0, 0x1F))),
                        ("e.bmp", lambda p: _bmp(p, rgba, bitfields=True)),
                        ("f.bmp", lambda p: _bmp(p, arr)), ("g.tga", lambda p: _tga(p, rgba, rle=True)),
                        ("h.tga", lambda p: _tga(p, arr[..., 0], rle=True))]:
        path = str(tmp_path / name)
        write(path)
        seeds.append(path)
    pam = str(tmp_path / "i.pam")
    with open(pam, "wb") as fh:
        fh.write(b"P7\nWIDTH 27\nHEIGHT 21\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n" + rgba.tobytes())
    seeds.append(pam)
    rng = np.random.default_rng(11)
    for batch in range(10):
        files = []
        for j in range(40):
            src = seeds[int(rng.integers(len(seeds)))]
            data = bytearray(open(src, "rb").read())
            kind = int(rng.integers(5))
            if kind == 0:
                for i in rng.integers(0, len(data), 1 + int(rng.integers(8))):
                    data[i] = int(rng.integers(256))
            elif kind == 1:
                for i in rng.integers(0, min(len(data), 80), 1 + int(rng.integers(4))):
                    data[i] = int(rng.integers(256))
            elif kind == 2:
                data = data[:int(rng.integers(1, len(data)))]
            elif kind == 3:
                i = int(rng.integers(0, len(data)))
                data[i:i] = rng.integers(0, 256, int(rng.integers(1, 60)), dtype=np.uint8).tobytes()
            else:                                       # a stray marker / tag byte pair
                i = int(rng.integers(0, len(data) - 4))
                data[i:i + 2] = bytes([0xFF, int(rng.integers(256))])
            path = str(tmp_path / ("m%d%s" % (j, os.path.splitext(src)[1])))
            with open(path, "wb") as fh:
                fh.write(bytes(data))
            files.append(path)
        r = subprocess.run([exe] + files, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]


def _packbits(row):
    """PackBits: runs of 3+ equal bytes as repeats, the rest as literals."""
    out, i = bytearray(), 0
    while i < len(row):
        j = i
        while j + 1 < len(row) and row[j + 1] == row[i] and j - i < 127:
            j += 1
        if j - i >= 2:
            out += bytes([257 - (j - i + 1)]) + bytes([row[i]])
            i = j + 1
            continue
        k = i
        while k < len(row) and k - i < 128 and not (k + 2 < len(row) and row[k] == row[k + 1] == row[k + 2]):
            k += 1
        out += bytes([k - i - 1]) + bytes(row[i:k])
        i = k
    return bytes(out)


def _psd(path, planes, mode, depth=8, rle=False, extra=0):
    """Writes a PSD whose merged image holds `planes` ((C, H, W) uint8 values,
    written as the high byte of 16-bit channels when depth is 16) plus
    `extra` unused channels."""
    c, h, w = planes.shape
    chans = list(planes) + [np.full((h, w), 77, np.uint8)] * extra
    data = []
    for p in chans:
        px = p if depth == 8 else np.stack([p, (p * 7) & 255], -1).reshape(h, w * 2)   # low bytes are noise
        data.append(px.reshape(h, -1))
    head = b"8BPS" + struct.pack(">H6xHIIHH", 1, len(chans), h, w, depth, mode)
    body = struct.pack(">I", 0) + struct.pack(">I", 4) + b"\x00\x01\x02\x03" + struct.pack(">I", 0)
    if not rle:
        img = struct.pack(">H", 0) + b"".join(p.astype(np.uint8).tobytes() for p in data)
    else:
        rows = [_packbits(bytes(r.astype(np.uint8))) for p in data for r in p]
        img = struct.pack(">H", 1) + struct.pack(">%dH" % len(rows), *[len(r) for r in rows]) + b"".join(rows)
    with open(path, "wb") as fh:
        fh.write(head + body + img)


@pytest.mark.parametrize("mode,nch,extra", [(3, 3, 0), (3, 4, 0), (3, 4, 2), (1, 1, 0), (1, 2, 1)])
@pytest.mark.parametrize("depth", [8, 16])
@pytest.mark.parametrize("rle", [False, True])
def test_cli_reads_psd(native, tmp_path, mode, nch, extra, depth, rle):
    rng = np.random.default_rng(nch * 10 + depth + rle)
    h, w = 23, 31
    color = rng.integers(0, 256, (nch, h, w), dtype=np.uint8)
    color[:, 5:12, 3:20] = color[:, 5, 3][:, None, None]                # runs for PackBits
    has_alpha = nch == (4 if mode == 3 else 2)
    planes = color.copy()
    if has_alpha:
        a = color[-1].astype(np.int64)
        a[0] = 0
        a[1] = 255
        planes[-1] = a
        # the merged image is matted against white: c = a x + (1 - a) 255
        x = color[:-1].astype(np.int64)
        planes[:-1] = np.clip(np.rint((a * x + (255 - a) * 255) / 255.0), 0, 255)
    path = str(tmp_path / "in.psd")
    _psd(path, planes, mode, depth, rle, extra)
    got = _dump(native, path, tmp_path)[::-1]
    want = np.full((h, w, 4), 255, np.uint8)
    if mode == 3:
        want[..., :3] = planes[:3].transpose(1, 2, 0)
    else:
        want[..., :3] = planes[0][..., None]
    if has_alpha:
        a = planes[-1].astype(np.int64)
        want[..., 3] = a
        part = (a > 0) & (a < 255)
        # the matte comes off with the reference loader's FP32 arithmetic:
        # c / f + 255 (1 - 1 / f) for f = A / 255, truncated (0 below 0)
        f = a.astype(np.float32) / np.float32(255)
        ra = np.float32(1) / np.maximum(f, np.float32(1e-30))
        v = want[..., :3].astype(np.float32) * ra[..., None] + (np.float32(255) * (np.float32(1) - ra))[..., None]
        x = np.where(v <= 0, 0, np.floor(np.maximum(v, 0))).astype(np.uint8)
        want[..., :3] = np.where(part[..., None], x, want[..., :3])
        # the un-matted colour is the original within the matte's rounding
        orig = color[:-1].transpose(1, 2, 0).astype(int) if mode == 3 else color[0][..., None].astype(int)
        sel = part & (a >= 32)
        assert np.abs(want[..., :3].astype(int) - orig)[sel].max() <= 6
    assert np.array_equal(got, want)
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    assert np.array_equal(image_io.load_image(path), want)


def _lzw(indices, minsize):
    """GIF LZW, codes packed least-significant bit first; a clear code first
    and whenever the 4096-entry table is full."""
    clear, stop = 1 << minsize, (1 << minsize) + 1
    acc, nacc, out = 0, 0, bytearray()

    def emit(code, width):
        nonlocal acc, nacc
        acc |= code << nacc
        nacc += width
        while nacc >= 8:
            out.append(acc & 255)
            acc >>= 8
            nacc -= 8

    def fresh():
        return {bytes([i]): i for i in range(clear)}, clear + 2, minsize + 1
    table, nxt, width = fresh()
    emit(clear, width)
    w = b""
    for k in indices:
        wk = w + bytes([int(k)])
        if wk in table:
            w = wk
            continue
        emit(table[w], width)
        if nxt < 4096:
            table[wk] = nxt
            nxt += 1
            if nxt > (1 << width) and width < 12:
                width += 1
        else:
            emit(clear, width)
            table, nxt, width = fresh()
        w = bytes([int(k)])
    emit(table[w], width)
    emit(stop, width)
    if nacc:
        out.append(acc & 255)
    return bytes(out)


def _gif(path, idx, pal, screen=None, offset=(0, 0), transparent=None, interlace=False, local=False):
    fh, fw = idx.shape
    sh, sw = screen or (fh, fw)
    nbits = max(1, int(np.ceil(np.log2(len(pal)))))
    size = 1 << nbits
    ptab = np.zeros((size, 3), np.uint8)
    ptab[:len(pal)] = pal
    minsize = max(2, nbits)
    out = b"GIF89a" + struct.pack("<HHBBB", sw, sh, 0 if local else 0x80 | (nbits - 1), 0, 0)
    if not local:
        out += ptab.tobytes()
    if transparent is not None:
        out += b"\x21\xf9\x04" + struct.pack("<BHB", 1, 0, transparent) + b"\x00"
    out += b"\x21\xfe\x05hello\x00"                        # a comment extension
    out += b"\x2c" + struct.pack("<HHHHB", offset[1], offset[0], fw, fh,
                                  (0x80 | (nbits - 1) if local else 0) | (0x40 if interlace else 0))
    if local:
        out += ptab.tobytes()
    rows = idx
    if interlace:
        rows = idx[[y for start, step in ((0, 8), (4, 8), (2, 4), (1, 2)) for y in range(start, fh, step)]]
    data = _lzw(rows.reshape(-1), minsize)
    out += bytes([minsize]) + b"".join(bytes([len(data[i:i + 255])]) + data[i:i + 255]
                                      for i in range(0, len(data), 255)) + b"\x00\x3b"
    with open(path, "wb") as fh_:
        fh_.write(out)


@pytest.mark.parametrize("case", ["plain", "transparent", "interlaced", "offset_local", "big_table", "two_colour"])
def test_cli_reads_gif(native, tmp_path, case):
    rng = np.random.default_rng(["plain", "transparent", "interlaced", "offset_local", "big_table",
                                 "two_colour"].index(case))
    ncol = 2 if case == "two_colour" else 256 if case == "big_table" else 37
    h, w = (96, 128) if case == "big_table" else (29, 41)
    pal = rng.integers(0, 256, (ncol, 3), dtype=np.uint8)
    idx = rng.integers(0, ncol, (h, w))
    idx[4:12, 5:30] = 3 % ncol                                      # repeats for the string table
    kw, screen, offset = {}, None, (0, 0)
    if case == "transparent":
        kw["transparent"] = 5
    if case == "interlaced":
        kw["interlace"] = True
    if case == "offset_local":
        screen, offset, kw["local"] = (40, 50), (6, 4), True
    path = str(tmp_path / "in.gif")
    _gif(path, idx, pal, screen=screen, offset=offset, **kw)
    sh, sw = screen or (h, w)
    want = np.zeros((sh, sw, 4), np.uint8)
    region = want[offset[0]:offset[0] + h, offset[1]:offset[1] + w]
    region[..., :3] = pal[idx]
    region[..., 3] = 255
    if case == "transparent":
        region[idx == 5] = 0
    assert np.array_equal(_dump(native, path, tmp_path)[::-1], want)
    from astc_encoder_gb300 import image_io                 # the Python reader agrees
    assert np.array_equal(image_io.load_image(path), want)


def _hdr(path, rgbe, rle=True):
    """Radiance HDR: run-length scanlines (runs of 3+ as 128 + n, else literals)."""
    h, w = rgbe.shape[:2]
    out = b"#?RADIANCE\n# written by the test suite\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n"
    out += ("-Y %d +X %d\n" % (h, w)).encode()
    for y in range(h):
        if not rle:
            out += rgbe[y].tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            ch, x = rgbe[y, :, c], 0
            while x < w:
                r = x
                while r + 1 < w and ch[r + 1] == ch[x] and r - x < 126:
                    r += 1
                if r - x >= 2:
                    out += bytes([128 + r - x + 1, int(ch[x])])
                    x = r + 1
                    continue
                k = x
                while k < w and k - x < 128 and not (k + 2 < w and ch[k] == ch[k + 1] == ch[k + 2]):
                    k += 1
                out += bytes([k - x]) + ch[x:k].tobytes()
                x = k
    with open(path, "wb") as fh:
        fh.write(out)


@pytest.mark.parametrize("rle", [False, True])
def test_cli_reads_hdr(native, tmp_path, rle):
    rng = np.random.default_rng(3 + rle)
    h, w = 19, 37
    rgbe = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    rgbe[..., 3] = rng.integers(120, 140, (h, w))                       # values around 2^-16 .. 2^4
    rgbe[2, :, 3] = 0                                                    # zero texels
    rgbe[5:9, 4:30] = rgbe[5, 4]                                         # runs
    path = str(tmp_path / "in.hdr")
    _hdr(path, rgbe, rle)
    v = rgbe[..., :3].astype(np.float64) * np.where(rgbe[..., 3] > 0, 2.0 ** (rgbe[..., 3].astype(np.float64) - 136), 0)[..., None]
    want = np.floor(np.clip(v ** (1 / 2.2) * 255 + 0.5, 0, 255))
    got = _dump(native, path, tmp_path)[::-1]
    assert (got[..., 3] == 255).all()
    diff = np.abs(got[..., :3].astype(int) - want)
    assert diff.max() <= 1 and (diff > 0).mean() < 0.01                 # float32 pow against float64
    from astc_encoder_gb300 import image_io
    py = image_io.load_image(path)
    assert np.abs(py.astype(int) - got).max() <= 1 and (py != got).mean() < 0.01


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
