"""Image loading for the encoder's command line (PNG, PAM/PPM/PGM, BMP, TGA).

The reference loads images with stb_image forced to RGBA and flipped
vertically (main.cpp:24-25).  This module is a small self-contained reader:
PNG (8-bit greyscale / grey+alpha / RGB / RGBA / palette, non-interlaced,
all five row filters, zlib from the Python standard library), Netpbm
P5/P6/P7, Windows BMP (24/32-bit, uncompressed or bit fields) and Truevision
TGA (8-bit grey, 24/32-bit true colour, raw or run-length encoded) -- the
same formats as the C++ reader of the command line tool.  It always returns
a (H, W, 4) uint8 array, row 0 first; the caller flips when it wants the
reference's orientation.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

PNG_SIG = b"\x89PNG\r\n\x1a\n"


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(h):
        f = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += stride + 1
        if f == 0:
            cur = line
        elif f == 1:
            cur = line.copy()
            for x in range(bpp, stride):                 # left neighbour, byte-wise
                cur[x] = (cur[x] + cur[x - bpp]) & 255
        elif f == 2:
            cur = (line + prev) & 255
        elif f == 3:
            cur = line.copy()
            cur[:bpp] = (cur[:bpp] + (prev[:bpp] >> 1)) & 255
            for x in range(bpp, stride):
                cur[x] = (cur[x] + ((cur[x - bpp] + prev[x]) >> 1)) & 255
        elif f == 4:
            cur = line.copy()
            cur[:bpp] = (cur[:bpp] + prev[:bpp]) & 255   # paeth(0, b, 0) = b
            for x in range(bpp, stride):
                a, b, c = int(cur[x - bpp]), int(prev[x]), int(prev[x - bpp])
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (cur[x] + pr) & 255
        else:
            raise ValueError(f"bad PNG filter type {f}")
        out[y] = cur
        prev = cur
    return out


def load_png(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:8] != PNG_SIG:
        raise ValueError("not a PNG file")
    pos, idat, hdr, plte, trns = 8, [], None, None, None
    while pos + 8 <= len(data):
        (ln,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif typ == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0:
        raise ValueError("only 8-bit non-interlaced PNG is supported")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(b"".join(idat))
    px = _unfilter(raw, h, w * chans, chans).reshape(h, w, chans)
    out = np.empty((h, w, 4), np.uint8)
    if ctype == 6:
        out[:] = px
    elif ctype == 2:
        out[..., :3] = px
        out[..., 3] = 255
    elif ctype == 0:
        out[..., :3] = px
        out[..., 3] = 255
    elif ctype == 4:
        out[..., :3] = px[..., :1]
        out[..., 3] = px[..., 1]
    else:
        if plte is None:
            raise ValueError("palette PNG without PLTE")
        idx = px[..., 0]
        out[..., :3] = plte[idx]
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = trns
        out[..., 3] = alpha[idx]
    return out


def load_pnm(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        data = fh.read()
    magic = data[:2]
    if magic == b"P7":
        head, _, body = data.partition(b"ENDHDR\n")
        fields = dict(line.split(None, 1) for line in head.decode().splitlines()[1:] if " " in line)
        w, h, d = int(fields["WIDTH"]), int(fields["HEIGHT"]), int(fields["DEPTH"])
        px = np.frombuffer(body, np.uint8, w * h * d).reshape(h, w, d)
    elif magic in (b"P5", b"P6"):
        toks, pos = [], 2
        while len(toks) < 3:
            while data[pos:pos + 1].isspace():
                pos += 1
            if data[pos:pos + 1] == b"#":
                pos = data.index(b"\n", pos) + 1
                continue
            end = pos
            while not data[end:end + 1].isspace():
                end += 1
            toks.append(int(data[pos:end]))
            pos = end
        pos += 1
        w, h, maxv = toks
        if maxv != 255:
            raise ValueError("only 8-bit PNM is supported")
        d = 3 if magic == b"P6" else 1
        px = np.frombuffer(data, np.uint8, w * h * d, pos).reshape(h, w, d)
    else:
        raise ValueError("not a PAM/PPM/PGM file")
    out = np.empty((h, w, 4), np.uint8)
    if px.shape[2] >= 3:
        out[..., :3] = px[..., :3]
    else:
        out[..., :3] = px[..., :1]
    out[..., 3] = px[..., 3] if px.shape[2] == 4 else (px[..., 1] if px.shape[2] == 2 else 255)
    return out


def load_bmp(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:2] != b"BM" or len(data) < 54:
        raise ValueError("not a BMP file")
    off, hdr = struct.unpack_from("<I", data, 10)[0], struct.unpack_from("<I", data, 14)[0]
    w, hraw, _, bpp, comp = struct.unpack_from("<iiHHI", data, 18)
    if hdr < 40 or w <= 0 or hraw == 0 or bpp not in (24, 32) or not (comp == 0 or (comp == 3 and bpp == 32)):
        raise ValueError("unsupported BMP format (24/32-bit uncompressed or 32-bit bit fields only)")
    h = abs(hraw)
    masks = [0x00FF0000, 0x0000FF00, 0x000000FF, 0xFF000000 if bpp == 32 else 0]
    if comp == 3:
        masks[:3] = struct.unpack_from("<III", data, 54)
        masks[3] = struct.unpack_from("<I", data, 66)[0] if hdr >= 56 else 0
    c = bpp // 8
    stride = (w * c + 3) & ~3
    rows = np.frombuffer(data, np.uint8, stride * h, off).reshape(h, stride)[:, :w * c].reshape(h, w, c)
    if hraw > 0:
        rows = rows[::-1]
    out = np.full((h, w, 4), 255, np.uint8)
    if bpp == 24:
        out[..., :3] = rows[..., [2, 1, 0]]
        return out
    v = rows.astype(np.uint32)
    v = v[..., 0] | (v[..., 1] << 8) | (v[..., 2] << 16) | (v[..., 3] << 24)
    for ch, m in enumerate(masks):
        if not m:
            continue
        shift = (m & -m).bit_length() - 1
        top = m >> shift
        x = (v & m) >> shift
        out[..., ch] = x if top == 255 else (x * 255 + top // 2) // top
    return out


def load_tga(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        data = fh.read()
    if len(data) < 18:
        raise ValueError("TGA header too short")
    idlen, cmap, itype = data[0], data[1], data[2]
    w, h = struct.unpack_from("<HH", data, 12)
    bpp, desc = data[16], data[17]
    grey = itype in (3, 11)
    if cmap != 0 or itype not in (2, 3, 10, 11) or w == 0 or h == 0 or bpp != (8 if grey else bpp) or \
            (not grey and bpp not in (24, 32)):
        raise ValueError("unsupported TGA file")
    px = bpp // 8
    pos = 18 + idlen
    n = w * h * px
    if itype in (2, 3):
        raw = np.frombuffer(data, np.uint8, n, pos)
    else:
        buf = bytearray()
        while len(buf) < n:
            c = data[pos]
            pos += 1
            count = (c & 0x7F) + 1
            if c & 0x80:
                buf += data[pos:pos + px] * count
                pos += px
            else:
                buf += data[pos:pos + count * px]
                pos += count * px
        raw = np.frombuffer(bytes(buf[:n]), np.uint8)
    raw = raw.reshape(h, w, px)
    if not (desc >> 5) & 1:
        raw = raw[::-1]
    out = np.full((h, w, 4), 255, np.uint8)
    if grey:
        out[..., :3] = raw[..., :1]
    else:
        out[..., :3] = raw[..., [2, 1, 0]]
        if px == 4:
            out[..., 3] = raw[..., 3]
    return out


def load_image(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        head = fh.read(8)
    if head == PNG_SIG:
        return load_png(path)
    if head[:1] == b"P" and head[1:2] in (b"5", b"6", b"7"):
        return load_pnm(path)
    if head[:2] == b"BM":
        return load_bmp(path)
    if path.lower().endswith(".tga"):                  # TGA has no magic number
        return load_tga(path)
    raise ValueError("unsupported image format (PNG, PAM/PPM/PGM, BMP and TGA are read)")
