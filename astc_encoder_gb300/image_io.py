"""Image loading for the encoder's command line (PNG, JPEG, PSD, GIF, HDR, PIC, PNM, BMP, TGA).

The reference loads images with stb_image forced to RGBA and flipped
vertically (main.cpp:24-25).  This module is a small self-contained reader:
PNG (greyscale / grey+alpha / RGB / RGBA / palette at every bit depth the
format allows, 16-bit channels reduced to their high byte, Adam7 interlacing,
tRNS, all five row filters, zlib from the Python standard library), Netpbm
P5/P6/P7, Windows BMP (1/4/8-bit palettes, 16/24/32-bit, bit fields), Truevision
TGA (colour-mapped, 8-bit grey, 15/16/24/32-bit true colour, raw or
run-length encoded),
JPEG (8-bit grey or YCbCr, Huffman coded, baseline or progressive),
Photoshop PSD (the merged image; 8/16-bit grey or RGB, optional alpha),
GIF (the first image; transparency as (0, 0, 0, 0)), Radiance HDR (taken
to 8 bits with gamma 1/2.2) and Softimage PIC -- the
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
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    if not (depth == 8 or (depth == 16 and ctype != 3) or (ctype in (0, 3) and depth in (1, 2, 4))):
        raise ValueError("bad PNG bit depth")
    raw = _zlib_inflate(b"".join(idat))
    passes = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
              (0, 1, 1, 2)] if interlace else [(0, 0, 1, 1)]
    samples = np.zeros((h, w, chans), np.int64)               # in the image's own bit depth
    off = 0
    for x0, y0, dx, dy in passes:
        pw, ph = max(0, -(-(w - x0) // dx)), max(0, -(-(h - y0) // dy))
        if pw == 0 or ph == 0:
            continue
        stride = (pw * chans * depth + 7) // 8
        rows = _unfilter(raw[off:off + (stride + 1) * ph], ph, stride, max(1, chans * depth // 8))
        off += (stride + 1) * ph
        if depth == 16:
            v = rows.reshape(ph, pw * chans, 2).astype(np.int64)
            v = (v[..., 0] << 8) | v[..., 1]
        elif depth == 8:
            v = rows.astype(np.int64)
        else:
            bits = np.unpackbits(rows, axis=1)[:, :pw * chans * depth].reshape(ph, pw * chans, depth)
            v = (bits.astype(np.int64) << np.arange(depth - 1, -1, -1)).sum(-1)
        samples[y0::dy, x0::dx] = v.reshape(ph, pw, chans)
    maxv = (1 << depth) - 1
    to8 = (lambda x: x >> 8) if depth == 16 else (lambda x: x * (255 // maxv))
    out = np.empty((h, w, 4), np.uint8)
    if ctype == 3:
        if plte is None:
            raise ValueError("palette PNG without PLTE")
        idx = samples[..., 0]
        if idx.max(initial=0) >= len(plte):
            raise ValueError("palette index out of range")
        out[..., :3] = plte[idx]
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = trns[:256]
        out[..., 3] = alpha[idx]
        return out
    key = None
    if trns is not None and ctype in (0, 2) and len(trns) >= 2 * (1 if ctype == 0 else 3):
        key = [(int(trns[2 * c]) << 8) | int(trns[2 * c + 1]) for c in range(1 if ctype == 0 else 3)]
    if ctype in (2, 6):
        out[..., :3] = to8(samples[..., :3])
    else:
        out[..., :3] = to8(samples[..., :1])
    if ctype in (4, 6):
        out[..., 3] = to8(samples[..., -1])
    else:
        out[..., 3] = 255
        if key is not None:
            out[..., 3] = np.where((samples[..., :len(key)] == key).all(-1), 0, 255)
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
    pal = bpp in (1, 4, 8)
    if hdr < 40 or w <= 0 or hraw == 0 or not (pal or bpp in (16, 24, 32)) or \
            not (comp == 0 or (comp == 3 and bpp in (16, 32))):
        raise ValueError("unsupported BMP format (1/4/8/16/24/32-bit uncompressed or 16/32-bit bit fields)")
    h = abs(hraw)
    masks = [0x00FF0000, 0x0000FF00, 0x000000FF, 0xFF000000 if bpp == 32 else 0]
    if bpp == 16:
        masks = [0x7C00, 0x03E0, 0x001F, 0]
    if comp == 3:
        masks[:3] = struct.unpack_from("<III", data, 54)
        masks[3] = struct.unpack_from("<I", data, 66)[0] if hdr >= 56 else 0
    stride = ((w * bpp + 31) // 32) * 4
    rows = np.frombuffer(data, np.uint8, stride * h, off).reshape(h, stride)
    if hraw > 0:
        rows = rows[::-1]
    out = np.full((h, w, 4), 255, np.uint8)
    if pal:
        used = struct.unpack_from("<I", data, 46)[0]
        n = 1 << bpp if used == 0 or used > 1 << bpp else used
        table = np.frombuffer(data, np.uint8, 4 * n, 14 + hdr).reshape(n, 4)[:, [2, 1, 0]]
        bits = np.unpackbits(rows, axis=1)[:, :w * bpp].reshape(h, w, bpp).astype(np.int64)
        idx = (bits << np.arange(bpp - 1, -1, -1)).sum(-1)
        if idx.max() >= n:
            raise ValueError("BMP palette index out of range")
        out[..., :3] = table[idx]
        return out
    c = bpp // 8
    px = rows[:, :w * c].reshape(h, w, c)
    if bpp == 24:
        out[..., :3] = px[..., [2, 1, 0]]
        return out
    v = px.astype(np.uint64)
    v = sum(v[..., i] << (8 * i) for i in range(c))
    for ch, m in enumerate(masks):
        if not m:
            continue
        out[..., ch] = _widen_field(v, m)
    # a 32-bit BI_RGB image whose fourth byte is 0 everywhere reads as opaque
    # (stb_image, the reference's loader, for 40- and 56-byte headers)
    if bpp == 32 and comp == 0 and hdr in (40, 56) and not out[..., 3].any():
        out[..., 3] = 255
    return out


def _widen_field(v, m):
    """A BMP mask's field widened to 8 bits as stb_image (the reference's
    loader) widens it: the masked value moved so the mask's top bit sits at
    bit 7, its top n bits (n = the mask's bit count) taken as the field and
    repeated to fill 8 bits; 8 or more bits keep the 8 below the top bit."""
    hb = m.bit_length() - 1
    n = bin(m).count("1")
    y = ((v & m) >> (hb - 7) if hb >= 7 else (v & m) << (7 - hb)) & 0xFF
    if n >= 8:
        return y.astype(np.uint8)
    x = y >> (8 - n)
    acc, bits = np.zeros_like(x), 0
    while bits < 8:
        acc = (acc << n) | x
        bits += n
    return (acc >> (bits - 8)).astype(np.uint8)


def _rgb16(v):
    """15/16-bit TGA colours x RRRRR GGGGG BBBBB -> RGBA (x 255 / 31, alpha 255)."""
    v = v.astype(np.int64)
    out = np.full(v.shape + (4,), 255, np.uint8)
    for c, sh in enumerate((10, 5, 0)):
        out[..., c] = ((v >> sh) & 31) * 255 // 31
    return out


def load_tga(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        data = fh.read()
    if len(data) < 18:
        raise ValueError("TGA header too short")
    idlen, cmap, itype = data[0], data[1], data[2]
    cfirst, clen, cbits = struct.unpack_from("<HHB", data, 3)
    w, h = struct.unpack_from("<HH", data, 12)
    bpp, desc = data[16], data[17]
    grey, mapped = itype in (3, 11), itype in (1, 9)
    if itype not in (1, 2, 3, 9, 10, 11) or (mapped and cmap != 1) or w == 0 or h == 0 or \
            not (bpp == 8 if (grey or mapped) else bpp in (15, 16, 24, 32)):
        raise ValueError("unsupported TGA file")
    px = (bpp + 7) // 8
    pos = 18 + idlen
    colours = None
    # as stb_image (the reference's loader): the map of an unmapped image is
    # skipped; for a mapped one the first-entry field counts bytes to skip
    if cmap == 1 and not mapped:
        pos += clen * ((cbits + 7) // 8)
    elif cmap == 1:
        pos += cfirst
        cb = (cbits + 7) // 8
        if cbits not in (15, 16, 24, 32) or clen == 0:
            raise ValueError("bad TGA colour map")
        table = np.frombuffer(data, np.uint8, clen * cb, pos).reshape(clen, cb)
        pos += clen * cb
        if cb == 2:
            colours = _rgb16(table[:, 0].astype(np.int64) | (table[:, 1].astype(np.int64) << 8))
        else:
            colours = np.full((clen, 4), 255, np.uint8)
            colours[:, :3] = table[:, [2, 1, 0]]
            if cb == 4:
                colours[:, 3] = table[:, 3]
    n = w * h * px
    if itype in (1, 2, 3):
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
    elif mapped:
        idx = raw[..., 0].astype(np.int64)
        idx = np.where(idx < clen, idx, 0)              # past the map: entry 0
        out[:] = colours[idx]
    elif px == 2:
        out[:] = _rgb16(raw[..., 0].astype(np.int64) | (raw[..., 1].astype(np.int64) << 8))
    else:
        out[..., :3] = raw[..., [2, 1, 0]]
        if px == 4:
            out[..., 3] = raw[..., 3]
    return out


_ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48,
                    41, 34, 27, 20, 13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22,
                    15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55,
                    62, 63])


def _zlib_inflate(z: bytes) -> bytes:
    """A zlib stream's data: the header is checked (deflate, no preset
    dictionary), the trailing Adler-32 is not -- as the command line tool's
    reader and stb_image (the reference's loader) do."""
    if len(z) < 6 or (z[0] & 0x0F) != 8 or ((z[0] << 8) | z[1]) % 31 or z[1] & 0x20:
        raise ValueError("bad zlib header")
    d = zlib.decompressobj(-15)
    out = d.decompress(z[2:])
    if not d.eof:
        raise ValueError("zlib stream truncated")
    return out


def _jpeg_huffman(counts, syms):
    """(code length, code) -> symbol, as a 16-bit peek table of (symbol, length).
    Code lengths that over-fill the code space are refused (T.81)."""
    table = np.full((1 << 16, 2), -1, np.int32)
    code, k = 0, 0
    for length in range(1, 17):
        if code + counts[length - 1] > (1 << length):
            raise ValueError("bad JPEG Huffman table")
        for _ in range(counts[length - 1]):
            lo = code << (16 - length)
            table[lo:lo + (1 << (16 - length))] = (syms[k], length)
            code += 1
            k += 1
        code <<= 1
    return table


def load_jpeg(path: str) -> np.ndarray:
    """Baseline and progressive JPEG (ITU-T T.81 SOF0/SOF1/SOF2, 8-bit, Huffman,
    grey or YCbCr with sampling factors 1..2, interleaved and single-component
    scans, spectral selection and successive approximation, restart
    intervals): the same decoding as the command line tool's reader, in
    float64."""
    with open(path, "rb") as fh:
        d = fh.read()
    if d[:2] != b"\xff\xd8":
        raise ValueError("not a JPEG file")
    qt = np.zeros((4, 64), np.int64)
    huff = {}
    comps, restart, pos, frame = [], 0, 2, None
    scans = 0
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
                if d[o] >> 4 > 1 or d[o] & 15 > 3 or o + 17 > end or total > 256 or o + 17 + total > end:
                    raise ValueError("bad JPEG Huffman table")
                huff[(d[o] >> 4, d[o] & 15)] = _jpeg_huffman(counts, d[o + 17:o + 17 + total])
                o += 17 + total
        elif m in (0xC0, 0xC1, 0xC2):
            if d[seg] != 8:
                raise ValueError("only 8-bit JPEG is read")
            height, width = struct.unpack_from(">HH", d, seg + 1)
            nc = d[seg + 5]
            if nc not in (1, 3):
                raise ValueError("unsupported JPEG frame (grey or YCbCr only)")
            for i in range(nc):
                c = d[seg + 6 + 3 * i:seg + 9 + 3 * i]
                comps.append({"id": c[0], "h": c[1] >> 4, "v": c[1] & 15, "tq": c[2] & 3})
                if not (1 <= c[1] >> 4 <= 2 and 1 <= c[1] & 15 <= 2):
                    raise ValueError("unsupported JPEG sampling")
            if nc == 1:
                comps[0]["h"] = comps[0]["v"] = 1
            hmax = max(c["h"] for c in comps)
            vmax = max(c["v"] for c in comps)
            mcux, mcuy = -(-width // (8 * hmax)), -(-height // (8 * vmax))
            for c in comps:
                c["bw"], c["bh"] = mcux * c["h"], mcuy * c["v"]
                c["cbw"] = (-(-width * c["h"] // hmax) + 7) // 8
                c["cbh"] = (-(-height * c["v"] // vmax) + 7) // 8
                c["coef"] = None
            frame = dict(width=width, height=height, hmax=hmax, vmax=vmax, mcux=mcux, mcuy=mcuy,
                         progressive=m == 0xC2)
        elif 0xC3 <= m <= 0xCF and m not in (0xC4, 0xC8, 0xCC):
            raise ValueError("lossless, hierarchical or arithmetic-coded JPEG is not read")
        elif m == 0xDD:
            restart = struct.unpack_from(">H", d, seg)[0]
        elif m == 0xDA:
            if frame is None:
                raise ValueError("JPEG scan before the frame header")
            scans += 1
            ns = d[seg]
            sc = []
            for i in range(ns):
                cid, t = d[seg + 1 + 2 * i], d[seg + 2 + 2 * i]
                c = next((c for c in comps if c["id"] == cid), None)
                if c is None:
                    raise ValueError("JPEG scan names an unknown component")
                c["td"], c["ta"] = t >> 4, t & 15
                sc.append(c)
            q = seg + 1 + 2 * ns
            ss, se, ah, al = d[q], d[q + 1], d[q + 2] >> 4, d[q + 2] & 15
            prog = frame["progressive"]
            if (not prog and (ss, se, ah, al) != (0, 63, 0, 0)) or \
                    (prog and (se > 63 or ss > se or (ss == 0 and se != 0) or (ss > 0 and ns != 1))):
                raise ValueError("bad JPEG scan parameters")
            for c in sc:
                if c["coef"] is None:
                    if not (ss == 0 and ah == 0):
                        raise ValueError("JPEG AC scan before the DC scan")
                    c["coef"] = np.zeros((c["bh"], c["bw"], 64), np.int64)
            pos = _jpeg_scan(d, end, frame, sc, ss, se, ah, al, huff, restart)
            continue
        pos = end
    if frame is None or scans == 0:
        raise ValueError("JPEG has no image scan")
    if any(c["coef"] is None for c in comps):
        raise ValueError("JPEG component without a scan")
    return _jpeg_image(frame, comps, qt)


class _JpegBits:
    """Entropy-coded data from `pos`: unstuffed bytes, with the positions of
    the RSTn markers; reads past the data (or a marker) give zero bits."""

    def __init__(self, d, pos):
        out, rst = bytearray(), []
        while pos < len(d):
            b = d[pos]
            if b == 0xFF and pos + 1 < len(d):
                nx = d[pos + 1]
                if nx == 0x00:
                    out.append(0xFF)
                    pos += 2
                    continue
                if 0xD0 <= nx <= 0xD7:
                    rst.append(len(out))
                    pos += 2
                    continue
                break
            out.append(b)
            pos += 1
        self.data, self.rst, self.end = bytes(out) + b"\0\0\0\0", rst, pos
        self.limit, self.bitpos, self.seg = len(out) if not rst else rst[0], 0, 0

    def restart(self):
        self.bitpos = 8 * self.rst[self.seg] if self.seg < len(self.rst) else 8 * (len(self.data) - 4)
        self.seg += 1
        self.limit = self.rst[self.seg] if self.seg < len(self.rst) else len(self.data) - 4

    def bit(self):
        byte = self.bitpos >> 3
        v = (self.data[byte] >> (7 - (self.bitpos & 7))) & 1 if byte < self.limit else 0
        self.bitpos += 1
        return v

    def get(self, k):
        v = 0
        for _ in range(k):
            v = (v << 1) | self.bit()
        return v

    def sym(self, table):
        byte = self.bitpos >> 3
        w = int.from_bytes(self.data[byte:byte + 3], "big") if byte + 3 <= self.limit else \
            int.from_bytes((self.data[byte:self.limit] + b"\0\0\0")[:3], "big")
        peek = (w >> (8 - (self.bitpos & 7))) & 0xFFFF
        s, length = table[peek]
        if length < 0:
            raise ValueError("corrupt JPEG data")
        self.bitpos += int(length)
        return int(s)

    def overrun(self):
        return self.bitpos > 8 * self.limit + 64


def _extend(v, t):
    return 0 if t == 0 else (v - (1 << t) + 1 if v < (1 << (t - 1)) else v)


def _jpeg_scan(d, pos, frame, sc, ss, se, ah, al, huff, restart):
    """Decodes one scan into the components' coefficients; returns the
    position of the next marker."""
    bits = _JpegBits(d, pos)
    prog = frame["progressive"]
    single = len(sc) == 1
    units = sc[0]["cbw"] * sc[0]["cbh"] if single else frame["mcux"] * frame["mcuy"]
    eobrun = [0]
    for c in sc:
        c["pred"] = 0
    p1, m1 = 1 << al, -(1 << al)

    def refine(blk, z):
        if bits.bit() and (blk[z] & p1) == 0:
            blk[z] += p1 if blk[z] >= 0 else m1

    def block(c, blk):
        if not prog or ss == 0:
            if ah == 0:
                t = bits.sym(huff[(0, c["td"])])
                if t > 11:
                    raise ValueError("corrupt JPEG data")
                c["pred"] += _extend(bits.get(t), t)
                blk[0] = c["pred"] << al
            elif bits.bit():
                blk[0] |= p1
            if prog:
                return
            k = 1
            act = huff[(1, c["ta"])]
            while k < 64:
                rs = bits.sym(act)
                r, sz = rs >> 4, rs & 15
                if sz == 0:
                    if r != 15:
                        break
                    k += 16
                    continue
                k += r
                if k > 63:
                    raise ValueError("corrupt JPEG data")
                blk[_ZIGZAG[k]] = _extend(bits.get(sz), sz)
                k += 1
            return
        act = huff[(1, c["ta"])]
        if ah == 0:                                      # AC first
            if eobrun[0] > 0:
                eobrun[0] -= 1
                return
            k = ss
            while k <= se:
                rs = bits.sym(act)
                r, sz = rs >> 4, rs & 15
                if sz == 0:
                    if r < 15:
                        eobrun[0] = (1 << r) - 1 + (bits.get(r) if r else 0)
                        break
                    k += 16
                    continue
                k += r
                if k > se:
                    raise ValueError("corrupt JPEG data")
                blk[_ZIGZAG[k]] = _extend(bits.get(sz), sz) << al
                k += 1
            return
        k = ss                                           # AC refinement
        if eobrun[0] == 0:
            while k <= se:
                rs = bits.sym(act)
                r, sz = rs >> 4, rs & 15
                val = 0
                if sz:
                    if sz != 1:
                        raise ValueError("corrupt JPEG data")
                    val = p1 if bits.bit() else m1
                elif r != 15:
                    eobrun[0] = (1 << r) + (bits.get(r) if r else 0)
                    break
                while k <= se:
                    z = _ZIGZAG[k]
                    if blk[z] != 0:
                        refine(blk, z)
                    else:
                        if r == 0:
                            break
                        r -= 1
                    k += 1
                if val:
                    if k > se:
                        raise ValueError("corrupt JPEG data")
                    blk[_ZIGZAG[k]] = val
                k += 1
        if eobrun[0] > 0:
            while k <= se:
                if blk[_ZIGZAG[k]] != 0:
                    refine(blk, _ZIGZAG[k])
                k += 1
            eobrun[0] -= 1

    mcux = frame["mcux"]
    for u in range(units):
        if restart and u and u % restart == 0:
            bits.restart()
            eobrun[0] = 0
            for c in sc:
                c["pred"] = 0
        for c in sc:
            if single:
                block(c, c["coef"][u // c["cbw"], u % c["cbw"]])
                continue
            my, mx = divmod(u, mcux)
            for by in range(c["v"]):
                for bx in range(c["h"]):
                    block(c, c["coef"][my * c["v"] + by, mx * c["h"] + bx])
        if bits.overrun():
            raise ValueError("JPEG data too short")
    return bits.end


def _jpeg_image(frame, comps, qt):
    width, height, hmax, vmax = frame["width"], frame["height"], frame["hmax"], frame["vmax"]
    xs = np.arange(8)
    cosv = np.cos((2 * xs[:, None] + 1) * xs[None, :] * np.pi / 16) * np.where(xs == 0, np.sqrt(0.5), 1.0)
    planes = []
    for c in comps:
        blocks = (c["coef"] * qt[c["tq"]]).reshape(c["bh"], c["bw"], 8, 8).astype(np.float64)
        pix = np.einsum("xu,abvu,yv->abyx", cosv, blocks, cosv) * 0.25
        pix = np.clip(np.floor(pix + 128.5), 0, 255)
        plane = pix.transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)
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


def load_psd(path: str) -> np.ndarray:
    """Photoshop PSD (version 1), the merged image: greyscale or RGB, 8 or 16
    bits per channel (high byte kept), optional alpha, raw or PackBits; the
    white matte of partly transparent pixels removed (as the command line
    tool's reader)."""
    with open(path, "rb") as fh:
        d = fh.read()
    if len(d) < 26 or d[:4] != b"8BPS":
        raise ValueError("not a PSD file")
    version, channels, h, w, depth, mode = struct.unpack_from(">H6xHIIHH", d, 4)
    if version != 1:
        raise ValueError("only version-1 PSD is read")
    if mode not in (1, 3):
        raise ValueError("PSD colour mode not read (greyscale and RGB are)")
    if depth not in (8, 16):
        raise ValueError("only 8- and 16-bit PSD is read")
    if not 1 <= channels <= 56:
        raise ValueError("bad PSD channel count")
    if not (0 < w <= 1 << 30 and 0 < h <= 1 << 30 and w * h <= 1 << 30):
        raise ValueError("bad image size")
    pos = 26
    for _ in range(3):
        pos += 4 + struct.unpack_from(">I", d, pos)[0]
    comp = struct.unpack_from(">H", d, pos)[0]
    pos += 2
    bps, used = depth // 8, min(channels, 4 if mode == 3 else 2)
    row = w * bps
    chans = []
    if comp == 0:
        for c in range(used):
            raw = np.frombuffer(d, np.uint8, row * h, pos + c * row * h)
            chans.append(raw.reshape(h, w, bps)[..., 0])
    elif comp == 1:
        counts = struct.unpack_from(">%dH" % (channels * h), d, pos)
        p = pos + 2 * channels * h
        for c in range(used):
            plane = np.zeros((h, row), np.uint8)
            for y in range(h):
                stop, line, q = p + counts[c * h + y], bytearray(), p
                while q < stop and len(line) < row:
                    k = d[q] - 256 if d[q] > 127 else d[q]
                    q += 1
                    if k >= 0:
                        line += d[q:q + k + 1]
                        q += k + 1
                    elif k != -128:
                        line += bytes([d[q]]) * (1 - k)
                        q += 1
                if len(line) != row:
                    raise ValueError("bad PSD run")
                plane[y] = np.frombuffer(bytes(line), np.uint8)
                p = stop
            chans.append(plane.reshape(h, w, bps)[..., 0])
    else:
        raise ValueError("PSD compression not read (raw and run-length are)")
    out = np.full((h, w, 4), 255, np.uint8)
    if mode == 3:
        for c in range(min(used, 3)):
            out[..., c] = chans[c]
        if used < 3:
            out[..., used:3] = 0
    else:
        out[..., :3] = chans[0][..., None]
    if used == (4 if mode == 3 else 2):
        a = chans[-1].astype(np.int64)
        out[..., 3] = a
        part = (a > 0) & (a < 255)
        # the reference loader's FP32 arithmetic: c / a + 255 (1 - 1 / a),
        # a = A / 255, truncated, 0 below 0
        af = a.astype(np.float32) / np.float32(255.0)
        ra = np.float32(1.0) / np.maximum(af, np.float32(1e-30))
        inv_a = np.float32(255.0) * (np.float32(1.0) - ra)
        v = out[..., :3].astype(np.float32) * ra[..., None] + inv_a[..., None]
        x = np.where(v <= 0, 0, np.floor(np.maximum(v, 0))).astype(np.uint8)
        out[..., :3] = np.where(part[..., None], x, out[..., :3])
    return out


def load_gif(path: str) -> np.ndarray:
    """GIF 87a / 89a, the first image on its logical screen (transparent black
    where the image or its transparent index leaves it), as the command line
    tool's reader."""
    with open(path, "rb") as fh:
        d = fh.read()
    if len(d) < 13 or d[:4] != b"GIF8" or d[4:6] not in (b"7a", b"9a"):
        raise ValueError("not a GIF file")
    sw, sh, flags = struct.unpack_from("<HHB", d, 6)
    pos, gpal, transparent = 13, None, -1
    if flags & 0x80:
        n = 2 << (flags & 7)
        gpal = np.frombuffer(d, np.uint8, 3 * n, pos).reshape(n, 3)
        pos += 3 * n
    while pos < len(d):
        b = d[pos]
        pos += 1
        if b == 0x3B:
            break
        if b == 0x21:
            label, first = d[pos], True
            pos += 1
            while d[pos] != 0:
                ln = d[pos]
                if label == 0xF9 and first and ln >= 4:
                    transparent = d[pos + 4] if d[pos + 1] & 1 else -1
                first = False
                pos += 1 + ln
            pos += 1
            continue
        if b != 0x2C:
            raise ValueError("bad GIF block")
        fx, fy, fw, fh, ff = struct.unpack_from("<HHHHB", d, pos)
        pos += 9
        pal = gpal
        if ff & 0x80:
            n = 2 << (ff & 7)
            pal = np.frombuffer(d, np.uint8, 3 * n, pos).reshape(n, 3)
            pos += 3 * n
        minsize = d[pos]
        pos += 1
        data = bytearray()
        while d[pos] != 0:
            data += d[pos + 1:pos + 1 + d[pos]]
            pos += 1 + d[pos]
        clear, stop = 1 << minsize, (1 << minsize) + 1
        table, width, out, prev = None, minsize + 1, [], None
        npix, bitpos, nbits = fw * fh, 0, len(data) * 8
        bits = int.from_bytes(bytes(data), "little")
        while len(out) < npix and bitpos + width <= nbits:
            code = (bits >> bitpos) & ((1 << width) - 1)
            bitpos += width
            if code == clear:
                table = [bytes([i]) for i in range(clear)] + [b"", b""]
                width, prev = minsize + 1, None
                continue
            if code == stop:
                break
            if table is None:
                table = [bytes([i]) for i in range(clear)] + [b"", b""]
            if prev is None:
                if code >= clear:
                    raise ValueError("corrupt GIF data")
                out.extend(table[code])
                prev = code
                continue
            if code < len(table):
                cur = table[code]
            elif code == len(table):
                cur = table[prev] + table[prev][:1]
            else:
                raise ValueError("corrupt GIF data")
            out.extend(cur)
            if len(table) < 4096:
                table.append(table[prev] + cur[:1])
                if len(table) == (1 << width) and width < 12:
                    width += 1
            prev = code
        idx = np.zeros(npix, np.int64)
        idx[:min(npix, len(out))] = out[:npix]
        idx = idx.reshape(fh, fw)
        if ff & 0x40:
            order = [y for start, step in ((0, 8), (4, 8), (2, 4), (1, 2)) for y in range(start, fh, step)]
            rows = np.zeros_like(idx)
            rows[order] = idx
            idx = rows
        img = np.zeros((sh, sw, 4), np.uint8)
        psize = 0 if pal is None else len(pal)
        for y in range(fh):
            if fy + y >= sh:
                continue
            for x in range(fw):
                c = idx[y, x]
                if fx + x >= sw or c == transparent or c >= psize:
                    continue
                img[fy + y, fx + x, :3] = pal[c]
                img[fy + y, fx + x, 3] = 255
        return img
    raise ValueError("GIF has no image")


def load_hdr(path: str) -> np.ndarray:
    """Radiance HDR (RGBE; flat or run-length scanlines, -Y h +X w), taken to
    8 bits as the command line tool's reader does: 255 v^(1/2.2) + 0.5,
    clamped and truncated (float32)."""
    with open(path, "rb") as fh:
        d = fh.read()
    lines, pos = [], 0
    while True:
        e = d.index(b"\n", pos)
        lines.append(d[pos:e].decode("latin-1"))
        pos = e + 1
        if len(lines) > 1 and lines[-1] == "":
            break
    if lines[0] not in ("#?RADIANCE", "#?RGBE"):
        raise ValueError("not a Radiance HDR file")
    for ln in lines:
        if ln.startswith("FORMAT=") and ln != "FORMAT=32-bit_rle_rgbe":
            raise ValueError("HDR format not read (32-bit_rle_rgbe is)")
    e = d.index(b"\n", pos)
    parts = d[pos:e].decode("latin-1").split()
    pos = e + 1
    if len(parts) != 4 or parts[0] != "-Y" or parts[2] != "+X":
        raise ValueError("HDR orientation not read (-Y h +X w is)")
    h, w = int(parts[1]), int(parts[3])
    rgbe = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w < 32768 and d[pos] == 2 and d[pos + 1] == 2 and not d[pos + 2] & 0x80:
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    k = d[pos]
                    pos += 1
                    if k > 128:
                        rgbe[y, x:x + k - 128, c] = d[pos]
                        pos += 1
                        x += k - 128
                    else:
                        rgbe[y, x:x + k, c] = np.frombuffer(d, np.uint8, k, pos)
                        pos += k
                        x += k
        else:
            rgbe[y] = np.frombuffer(d, np.uint8, 4 * w, pos).reshape(w, 4)
            pos += 4 * w
    f = np.where(rgbe[..., 3] > 0, np.ldexp(np.float32(1.0), rgbe[..., 3].astype(np.int32) - 136), 0).astype(np.float32)
    v = rgbe[..., :3].astype(np.float32) * f[..., None]
    z = np.power(v, np.float32(1.0 / 2.2)) * np.float32(255.0) + np.float32(0.5)
    out = np.full((h, w, 4), 255, np.uint8)
    out[..., :3] = np.clip(z, 0, 255).astype(np.int32)
    return out


def load_pic(path: str) -> np.ndarray:
    """Softimage PIC (8-bit channel packets; uncompressed, pure or mixed
    run-length), as the command line tool's reader."""
    with open(path, "rb") as fh:
        d = fh.read()
    if len(d) < 104 or d[:4] != b"\x53\x80\xf6\x34" or d[88:92] != b"PICT":
        raise ValueError("not a Softimage PIC file")
    w, h = struct.unpack_from(">HH", d, 92)
    pos, packets, chained = 104, [], True
    while chained:
        chained, size, typ, mask = d[pos:pos + 4]
        if size != 8 or typ > 2:
            raise ValueError("PIC packet not read (8-bit channels are)")
        packets.append((typ, mask))
        pos += 4
    out = np.full((h, w, 4), 255, np.uint8)
    for y in range(h):
        for typ, mask in packets:
            chans = [c for c in range(4) if mask & (0x80 >> c)]
            nch = len(chans)
            x = 0
            while x < w:
                if typ == 0:
                    count, literal = 1, True
                else:
                    c = d[pos]
                    pos += 1
                    if typ == 1:
                        count, literal = min(c, w - x), False   # cut at the row's end
                    elif c < 128:
                        count, literal = c + 1, True
                    elif c == 128:
                        count, literal = struct.unpack_from(">H", d, pos)[0], False
                        pos += 2
                    else:
                        count, literal = c - 127, False
                if count < 0 or x + count > w or (count == 0 and literal):
                    raise ValueError("bad PIC run")
                seg = out[y, x:x + count]
                if literal:
                    seg[:, chans] = np.frombuffer(d, np.uint8, count * nch, pos).reshape(count, nch)
                    pos += count * nch
                else:
                    seg[:, chans] = np.frombuffer(d, np.uint8, nch, pos)
                    pos += nch
                x += count
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
    if head[:4] == b"8BPS":
        return load_psd(path)
    if head[:4] == b"GIF8":
        return load_gif(path)
    if head[:6] == b"#?RGBE" or head[:8] == b"#?RADIAN":
        return load_hdr(path)
    if head[:4] == b"\x53\x80\xf6\x34":
        return load_pic(path)
    if path.lower().endswith(".tga"):                  # TGA has no magic number
        return load_tga(path)
    raise ValueError("unsupported image format (PNG, JPEG, PSD, GIF, HDR, PIC, PAM/PPM/PGM, BMP and TGA are read)")
