"""Image loading for the encoder's command line (PNG, PAM/PPM/PGM).

The reference loads images with stb_image forced to RGBA and flipped
vertically (main.cpp:24-25).  This module is a small self-contained reader:
PNG (8-bit greyscale / grey+alpha / RGB / RGBA / palette, non-interlaced,
all five row filters, zlib from the Python standard library) and Netpbm
P5/P6/P7.  It always returns a (H, W, 4) uint8 array, row 0 first; the caller
flips when it wants the reference's orientation.
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


def load_image(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        head = fh.read(8)
    if head == PNG_SIG:
        return load_png(path)
    return load_pnm(path)
