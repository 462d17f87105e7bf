"""Image loading for the encoder's command line (PNG, JPEG, PAM/PPM/PGM, BMP, TGA).

The reference loads images with stb_image forced to RGBA and flipped
vertically (main.cpp:24-25).  This module is a small self-contained reader:
PNG (8-bit greyscale / grey+alpha / RGB / RGBA / palette, non-interlaced,
all five row filters, zlib from the Python standard library), Netpbm
P5/P6/P7, Windows BMP (24/32-bit, uncompressed or bit fields), Truevision
TGA (8-bit grey, 24/32-bit true colour, raw or run-length encoded) and
baseline JPEG (8-bit grey or YCbCr, Huffman coded, one interleaved scan) -- the
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


_ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48,
                    41, 34, 27, 20, 13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22,
                    15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55,
                    62, 63])


def _jpeg_huffman(counts, syms):
    """(code length, code) -> symbol, as a 16-bit peek table of (symbol, length)."""
    table = np.full((1 << 16, 2), -1, np.int32)
    code, k = 0, 0
    for length in range(1, 17):
        for _ in range(counts[length - 1]):
            lo = code << (16 - length)
            table[lo:lo + (1 << (16 - length))] = (syms[k], length)
            code += 1
            k += 1
        code <<= 1
    return table


def load_jpeg(path: str) -> np.ndarray:
    """Baseline sequential JPEG (ITU-T T.81 SOF0/SOF1, 8-bit, Huffman, grey or
    YCbCr with sampling factors 1..2, one interleaved scan, restart intervals):
    the same decoding as the command line tool's reader, in float64."""
    with open(path, "rb") as fh:
        d = fh.read()
    if d[:2] != b"\xff\xd8":
        raise ValueError("not a JPEG file")
    qt = np.zeros((4, 64), np.int64)
    huff = {}
    comps, restart, pos = [], 0, 2
    width = height = 0
    while pos + 4 <= len(d):
        if d[pos] != 0xFF:
            pos += 1
            continue
        m = d[pos + 1]
        if m == 0xFF:
            pos += 1
            continue
        if m == 0xD8 or 0xD0 <= m <= 0xD7 or m == 0x01:
            pos += 2
            continue
        if m == 0xD9:
            break
        length = struct.unpack_from(">H", d, pos + 2)[0]
        seg, end = pos + 4, pos + 2 + length
        if m == 0xDB:
            o = seg
            while o < end:
                pq, tq = d[o] >> 4, d[o] & 15
                vals = struct.unpack_from(">64H", d, o + 1) if pq else list(d[o + 1:o + 65])
                qt[tq, _ZIGZAG] = vals
                o += 129 if pq else 65
        elif m == 0xC4:
            o = seg
            while o < end:
                counts = d[o + 1:o + 17]
                total = sum(counts)
                huff[(d[o] >> 4, d[o] & 15)] = _jpeg_huffman(counts, d[o + 17:o + 17 + total])
                o += 17 + total
        elif m in (0xC0, 0xC1):
            if d[seg] != 8:
                raise ValueError("only 8-bit JPEG is read")
            height, width = struct.unpack_from(">HH", d, seg + 1)
            nc = d[seg + 5]
            if nc not in (1, 3):
                raise ValueError("unsupported JPEG frame (grey or YCbCr only)")
            for i in range(nc):
                c = d[seg + 6 + 3 * i:seg + 9 + 3 * i]
                comps.append({"id": c[0], "h": c[1] >> 4, "v": c[1] & 15, "tq": c[2] & 3})
            if nc == 1:
                comps[0]["h"] = comps[0]["v"] = 1
        elif 0xC2 <= m <= 0xCF and m not in (0xC4, 0xC8, 0xCC):
            raise ValueError("progressive, lossless or arithmetic-coded JPEG is not read")
        elif m == 0xDD:
            restart = struct.unpack_from(">H", d, seg)[0]
        elif m == 0xDA:
            ns = d[seg]
            if ns != len(comps):
                raise ValueError("non-interleaved JPEG scans are not read")
            for i in range(ns):
                cid, t = d[seg + 1 + 2 * i], d[seg + 2 + 2 * i]
                for c in comps:
                    if c["id"] == cid:
                        c["td"], c["ta"] = t >> 4, t & 15
            return _jpeg_scan(d, end, width, height, comps, qt, huff, restart)
        pos = end
    raise ValueError("JPEG has no image scan")


def _jpeg_segments(d, pos):
    """The entropy-coded data from pos, split at RSTn markers, unstuffed."""
    segs, cur = [], bytearray()
    while pos < len(d):
        b = d[pos]
        if b == 0xFF and pos + 1 < len(d):
            nx = d[pos + 1]
            if nx == 0x00:
                cur.append(0xFF)
                pos += 2
                continue
            if 0xD0 <= nx <= 0xD7:
                segs.append(bytes(cur))
                cur = bytearray()
                pos += 2
                continue
            break
        cur.append(b)
        pos += 1
    segs.append(bytes(cur))
    return segs


def _jpeg_scan(d, pos, width, height, comps, qt, huff, restart):
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    mcux, mcuy = -(-width // (8 * hmax)), -(-height // (8 * vmax))
    nmcu = mcux * mcuy
    if nmcu * sum(c["h"] * c["v"] for c in comps) > 4 * (len(d) - pos) + 64:
        raise ValueError("JPEG data too short for its size")   # >= 2 bits per block
    segs = _jpeg_segments(d, pos)
    coef = [np.zeros((mcuy * c["v"], mcux * c["h"], 64), np.float64) for c in comps]
    seg_i, data, bitpos, dc = -1, b"", 0, [0] * len(comps)

    def bits(k):
        nonlocal bitpos
        v = 0
        for _ in range(k):
            byte = bitpos >> 3
            b = data[byte] if byte < len(data) else 0
            v = (v << 1) | ((b >> (7 - (bitpos & 7))) & 1)
            bitpos += 1
        return v

    def sym(table):
        nonlocal bitpos
        byte = bitpos >> 3
        w = int.from_bytes((data[byte:byte + 3] + b"\0\0\0")[:3], "big")
        peek = (w >> (8 - (bitpos & 7))) & 0xFFFF
        s, length = table[peek]
        if length < 0:
            raise ValueError("corrupt JPEG data")
        bitpos += int(length)
        return int(s)

    def extend(v, t):
        return 0 if t == 0 else (v - (1 << t) + 1 if v < (1 << (t - 1)) else v)

    for n in range(nmcu):
        if n == 0 or (restart and n % restart == 0):
            seg_i += 1
            data = segs[seg_i] if seg_i < len(segs) else b""
            bitpos, dc = 0, [0] * len(comps)
        my, mx = divmod(n, mcux)
        for ci, c in enumerate(comps):
            dct, act = huff[(0, c["td"])], huff[(1, c["ta"])]
            for by in range(c["v"]):
                for bx in range(c["h"]):
                    if bitpos > 8 * len(data) + 64:
                        raise ValueError("JPEG data too short")
                    blk = coef[ci][my * c["v"] + by, mx * c["h"] + bx]
                    t = sym(dct)
                    dc[ci] += extend(bits(t), t)
                    blk[0] = dc[ci]
                    k = 1
                    while k < 64:
                        rs = sym(act)
                        r, sz = rs >> 4, rs & 15
                        if sz == 0:
                            if r != 15:
                                break
                            k += 16
                            continue
                        k += r
                        blk[_ZIGZAG[k]] = extend(bits(sz), sz)
                        k += 1
    xs = np.arange(8)
    cosv = np.cos((2 * xs[:, None] + 1) * xs[None, :] * np.pi / 16) * np.where(xs == 0, np.sqrt(0.5), 1.0)
    planes = []
    for ci, c in enumerate(comps):
        blocks = (coef[ci] * qt[c["tq"]]).reshape(coef[ci].shape[:2] + (8, 8))
        pix = np.einsum("xu,abvu,yv->abyx", cosv, blocks, cosv) * 0.25
        pix = np.clip(np.floor(pix + 128.5), 0, 255)
        plane = pix.transpose(0, 2, 1, 3).reshape(blocks.shape[0] * 8, blocks.shape[1] * 8)
        ys = np.arange(height) * c["v"] // vmax
        xs_ = np.arange(width) * c["h"] // hmax
        planes.append(plane[ys][:, xs_])
    out = np.full((height, width, 4), 255, np.uint8)
    if len(comps) == 1:
        out[..., :3] = planes[0][..., None].astype(np.uint8)
        return out
    y, cb, cr = planes[0], planes[1] - 128.0, planes[2] - 128.0
    rgb = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], -1)
    out[..., :3] = np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)
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
    if head[:3] == b"\xff\xd8\xff":
        return load_jpeg(path)
    if path.lower().endswith(".tga"):                  # TGA has no magic number
        return load_tga(path)
    raise ValueError("unsupported image format (PNG, JPEG, PAM/PPM/PGM, BMP and TGA are read)")
