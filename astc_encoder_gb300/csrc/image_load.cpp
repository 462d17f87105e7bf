// image_load.cpp -- PNG / JPEG / PSD / GIF / HDR / PIC / Netpbm / BMP / TGA
// reader for the command line tool.
// Inflate follows RFC 1951 (stored, fixed and dynamic Huffman blocks,
// canonical codes decoded one bit at a time); the zlib wrapper RFC 1950;
// PNG chunk layout, filters 0-4, colour types, bit depths, Adam7 and tRNS the
// PNG specification.
#include "image_load.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

namespace astc {
namespace {

// Images up to 2^30 texels (4 GiB of RGBA8); larger or empty headers are refused
// before anything is allocated.
bool dims_ok(long long w, long long h, std::string& err) {
    if (w <= 0 || h <= 0 || w > (1ll << 30) || h > (1ll << 30) || w * h > (1ll << 30)) {
        err = "bad image size";
        return false;
    }
    return true;
}

struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool over = false;
    int bit() {
        if (cnt == 0) {
            if (pos >= n) { over = true; return 0; }
            buf = p[pos++];
            cnt = 8;
        }
        const int b = buf & 1;
        buf >>= 1;
        --cnt;
        return b;
    }
    uint32_t take(int k) {          // k bits, least significant first
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
};

struct Huffman {
    uint16_t count[16] = {};        // codes per length
    uint16_t symbol[320] = {};      // symbols ordered by (length, value)
};

// Canonical code from lengths; returns false for an over-subscribed set.
bool build(Huffman& h, const uint8_t* len, int n) {
    memset(h.count, 0, sizeof(h.count));
    for (int i = 0; i < n; ++i) h.count[len[i]]++;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    for (int i = 0; i < n; ++i)
        if (len[i]) h.symbol[offs[len[i]]++] = (uint16_t)i;
    return true;
}

// Walks the code one bit at a time: at each length the first `count` codes
// of that length map to the next symbols.
int decode(Bits& b, const Huffman& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= b.bit();
        const int count = h.count[l];
        if (code - first < count) return h.symbol[index + (code - first)];
        index += count;
        first += count;
        first <<= 1;
        code <<= 1;
        if (b.over) return -1;
    }
    return -1;
}

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                               2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,
                                33,  49,  65,  97,  129, 193,  257,  385,  513,  769,
                                1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits& b, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out,
                   std::string& err) {
    for (;;) {
        const int sym = decode(b, lit);
        if (sym < 0) { err = "bad literal/length code"; return false; }
        if (sym < 256) { out.push_back((uint8_t)sym); continue; }
        if (sym == 256) return true;
        const int li = sym - 257;
        if (li >= 29) { err = "bad length symbol"; return false; }
        const size_t len = kLenBase[li] + b.take(kLenExtra[li]);
        const int ds = decode(b, dist);
        if (ds < 0 || ds >= 30) { err = "bad distance code"; return false; }
        const size_t d = kDistBase[ds] + b.take(kDistExtra[ds]);
        if (d > out.size()) { err = "distance beyond the output"; return false; }
        const size_t from = out.size() - d;
        for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
        if (b.over) { err = "truncated deflate stream"; return false; }
    }
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

}  // namespace

bool zlib_inflate(const uint8_t* data, size_t size, std::vector<uint8_t>& out, std::string& err) {
    if (size < 6) { err = "zlib stream too short"; return false; }
    if ((data[0] & 0x0F) != 8 || ((data[0] << 8) | data[1]) % 31 != 0 || (data[1] & 0x20)) {
        err = "bad zlib header";
        return false;
    }
    Bits b{data + 2, size - 2};
    out.clear();
    int last = 0;
    do {
        last = b.bit();
        const int type = (int)b.take(2);
        if (type == 0) {
            b.buf = 0;
            b.cnt = 0;                                  // to the byte boundary
            if (b.pos + 4 > b.n) { err = "truncated stored block"; return false; }
            const uint32_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8);
            const uint32_t nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || b.pos + len > b.n) { err = "bad stored block"; return false; }
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            static Huffman flit, fdist;
            static bool ready = false;
            if (!ready) {
                uint8_t l[288];
                for (int i = 0; i < 144; ++i) l[i] = 8;
                for (int i = 144; i < 256; ++i) l[i] = 9;
                for (int i = 256; i < 280; ++i) l[i] = 7;
                for (int i = 280; i < 288; ++i) l[i] = 8;
                build(flit, l, 288);
                uint8_t d[30];
                for (int i = 0; i < 30; ++i) d[i] = 5;
                build(fdist, d, 30);
                ready = true;
            }
            if (!inflate_codes(b, flit, fdist, out, err)) return false;
        } else if (type == 2) {
            const int nlen = (int)b.take(5) + 257, ndist = (int)b.take(5) + 1, ncode = (int)b.take(4) + 4;
            if (nlen > 286 || ndist > 30) { err = "bad dynamic block counts"; return false; }
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)b.take(3);
            Huffman clh;
            if (!build(clh, cl, 19)) { err = "bad code-length code"; return false; }
            uint8_t lens[320] = {};
            int i = 0;
            while (i < nlen + ndist) {
                const int sym = decode(b, clh);
                if (sym < 0) { err = "bad code-length symbol"; return false; }
                if (sym < 16) { lens[i++] = (uint8_t)sym; continue; }
                int rep = 0;
                uint8_t val = 0;
                if (sym == 16) {
                    if (i == 0) { err = "repeat with no previous length"; return false; }
                    val = lens[i - 1];
                    rep = 3 + (int)b.take(2);
                } else if (sym == 17) {
                    rep = 3 + (int)b.take(3);
                } else {
                    rep = 11 + (int)b.take(7);
                }
                if (i + rep > nlen + ndist) { err = "code lengths overrun"; return false; }
                while (rep--) lens[i++] = val;
            }
            Huffman lit, dist;
            if (!build(lit, lens, nlen) || !build(dist, lens + nlen, ndist)) {
                err = "bad dynamic Huffman code";
                return false;
            }
            if (!inflate_codes(b, lit, dist, out, err)) return false;
        } else {
            err = "bad deflate block type";
            return false;
        }
        if (b.over) { err = "truncated deflate stream"; return false; }
    } while (!last);
    return true;
}

bool decode_png(const uint8_t* d, size_t n, Image& img, std::string& err) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (n < 8 || memcmp(d, sig, 8) != 0) { err = "not a PNG file"; return false; }
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    while (pos + 12 <= n) {
        const uint32_t len = be32(d + pos);
        const uint8_t* type = d + pos + 4;
        const uint8_t* body = d + pos + 8;
        if (pos + 12 + (size_t)len > n) { err = "truncated PNG chunk"; return false; }
        if (!memcmp(type, "IHDR", 4) && len >= 13) {
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
        } else if (!memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + (size_t)len;
    }
    if (!dims_ok(w, h, err)) return false;
    if (interlace > 1) { err = "bad PNG interlace method"; return false; }
    int chans = 0;
    switch (ctype) {
    case 0: chans = 1; break;
    case 2: chans = 3; break;
    case 3: chans = 1; break;
    case 4: chans = 2; break;
    case 6: chans = 4; break;
    default: err = "bad PNG colour type"; return false;
    }
    const bool low_ok = ctype == 0 || ctype == 3;              // 1/2/4-bit: grey and palette only
    if (!(depth == 8 || (depth == 16 && ctype != 3) || (low_ok && (depth == 1 || depth == 2 || depth == 4)))) {
        err = "bad PNG bit depth";
        return false;
    }
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), raw, err)) return false;
    // Adam7 passes (x0, y0, dx, dy), or the whole image as one pass
    static const int kAdam7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                     {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    static const int kWhole[1][4] = {{0, 0, 1, 1}};
    const int npass = interlace ? 7 : 1;
    const int(*passes)[4] = interlace ? kAdam7 : kWhole;
    const size_t fbpp = std::max<size_t>(1, (size_t)chans * depth / 8);   // filter unit in bytes
    const uint32_t maxv = (1u << depth) - 1;
    // tRNS key colour of grey / RGB images, in sample units
    int key[3] = {-1, -1, -1};
    if (ctype == 0 && trns.size() >= 2) key[0] = (trns[0] << 8) | trns[1];
    if (ctype == 2 && trns.size() >= 6)
        for (int c = 0; c < 3; ++c) key[c] = (trns[2 * c] << 8) | trns[2 * c + 1];
    img.width = (int)w;
    img.height = (int)h;
    img.rgba.assign((size_t)w * h * 4, 0);
    size_t off = 0;
    for (int p = 0; p < npass; ++p) {
        const uint32_t x0 = passes[p][0], y0 = passes[p][1], dx = passes[p][2], dy = passes[p][3];
        const uint32_t pw = w > x0 ? (w - x0 + dx - 1) / dx : 0, ph = h > y0 ? (h - y0 + dy - 1) / dy : 0;
        if (pw == 0 || ph == 0) continue;
        const size_t stride = ((size_t)pw * chans * depth + 7) / 8;
        if (raw.size() < off + (stride + 1) * ph) { err = "PNG image data too short"; return false; }
        std::vector<uint8_t> cur(stride), prev(stride, 0);
        for (uint32_t y = 0; y < ph; ++y, off += stride + 1) {
            const uint8_t* line = raw.data() + off;
            const int f = line[0];
            for (size_t x = 0; x < stride; ++x) {
                const int a = x >= fbpp ? cur[x - fbpp] : 0, b = prev[x], c = x >= fbpp ? prev[x - fbpp] : 0;
                int pr = 0;
                switch (f) {
                case 0: pr = 0; break;
                case 1: pr = a; break;
                case 2: pr = b; break;
                case 3: pr = (a + b) >> 1; break;
                case 4: {
                    const int e = a + b - c, pa = abs(e - a), pb = abs(e - b), pc = abs(e - c);
                    pr = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: err = "bad PNG filter type"; return false;
                }
                cur[x] = (uint8_t)(line[1 + x] + pr);
            }
            // sample i of this row, in its own bit depth
            auto sample = [&](size_t i) -> uint32_t {
                if (depth == 16) return ((uint32_t)cur[2 * i] << 8) | cur[2 * i + 1];
                if (depth == 8) return cur[i];
                const size_t bit = i * depth;
                return (cur[bit >> 3] >> (8 - depth - (bit & 7))) & maxv;
            };
            auto to8 = [&](uint32_t v) -> uint8_t {
                return (uint8_t)(depth == 16 ? v >> 8 : depth == 8 ? v : v * (255 / maxv));
            };
            uint8_t* orow = img.rgba.data() + (size_t)(y0 + y * dy) * w * 4;
            for (uint32_t x = 0; x < pw; ++x) {
                uint8_t* o = orow + (size_t)(x0 + x * dx) * 4;
                const size_t i = (size_t)x * chans;
                if (ctype == 3) {
                    const uint32_t idx = sample(i);
                    if ((size_t)idx * 3 + 2 >= plte.size()) { err = "palette index out of range"; return false; }
                    o[0] = plte[idx * 3];
                    o[1] = plte[idx * 3 + 1];
                    o[2] = plte[idx * 3 + 2];
                    o[3] = idx < trns.size() ? trns[idx] : 255;
                } else if (chans >= 3) {
                    const uint32_t r = sample(i), g = sample(i + 1), bl = sample(i + 2);
                    o[0] = to8(r);
                    o[1] = to8(g);
                    o[2] = to8(bl);
                    o[3] = chans == 4 ? to8(sample(i + 3))
                                      : ((int)r == key[0] && (int)g == key[1] && (int)bl == key[2] ? 0 : 255);
                } else {
                    const uint32_t v = sample(i);
                    o[0] = o[1] = o[2] = to8(v);
                    o[3] = chans == 2 ? to8(sample(i + 1)) : ((int)v == key[0] ? 0 : 255);
                }
            }
            std::swap(cur, prev);
        }
    }
    return true;
}

bool decode_pnm(const uint8_t* d, size_t n, Image& img, std::string& err) {
    if (n < 3 || d[0] != 'P') { err = "not a PNM/PAM file"; return false; }
    size_t pos = 2;
    auto token = [&](std::string& t) {
        t.clear();
        while (pos < n) {
            if (d[pos] == '#') { while (pos < n && d[pos] != '\n') ++pos; continue; }
            if (d[pos] == ' ' || d[pos] == '\t' || d[pos] == '\r' || d[pos] == '\n') { ++pos; continue; }
            break;
        }
        while (pos < n && !(d[pos] == ' ' || d[pos] == '\t' || d[pos] == '\r' || d[pos] == '\n'))
            t.push_back((char)d[pos++]);
        return !t.empty();
    };
    int w = 0, h = 0, depth = 0, maxv = 0;
    std::string t;
    if (d[1] == '7') {
        while (token(t) && t != "ENDHDR") {
            std::string v;
            if (t == "WIDTH" && token(v)) w = atoi(v.c_str());
            else if (t == "HEIGHT" && token(v)) h = atoi(v.c_str());
            else if (t == "DEPTH" && token(v)) depth = atoi(v.c_str());
            else if (t == "MAXVAL" && token(v)) maxv = atoi(v.c_str());
            else if (t == "TUPLTYPE") token(v);
        }
    } else if (d[1] == '5' || d[1] == '6') {
        depth = d[1] == '6' ? 3 : 1;
        if (!token(t)) { err = "bad PNM header"; return false; }
        w = atoi(t.c_str());
        if (!token(t)) { err = "bad PNM header"; return false; }
        h = atoi(t.c_str());
        if (!token(t)) { err = "bad PNM header"; return false; }
        maxv = atoi(t.c_str());
    } else {
        err = "unsupported PNM type";
        return false;
    }
    ++pos;                                               // one whitespace byte before the data
    if (depth < 1 || depth > 4 || maxv != 255) { err = "unsupported PNM header"; return false; }
    if (!dims_ok(w, h, err)) return false;
    if (pos + (size_t)w * h * depth > n) { err = "PNM data too short"; return false; }
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 255);
    const uint8_t* s = d + pos;
    for (size_t i = 0; i < (size_t)w * h; ++i, s += depth) {
        uint8_t* o = img.rgba.data() + i * 4;
        if (depth >= 3) { o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; if (depth == 4) o[3] = s[3]; }
        else { o[0] = o[1] = o[2] = s[0]; if (depth == 2) o[3] = s[1]; }
    }
    return true;
}

// Truevision TGA: image types 1 / 9 (8-bit indices into a 15/16/24/32-bit
// colour map), 2 / 10 (true colour: 15/16-bit x RRRRR GGGGG BBBBB without
// alpha, 24 or 32 bit BGR(A)), 3 / 11 (8-bit grey), raw or run-length
// encoded; bit 5 of the descriptor says the rows run top-down, otherwise
// bottom-up.
bool decode_tga(const uint8_t* d, size_t n, Image& img, std::string& err) {
    if (n < 18) { err = "TGA header too short"; return false; }
    const int idlen = d[0], cmap = d[1], type = d[2];
    const int cfirst = d[3] | (d[4] << 8), clen = d[5] | (d[6] << 8), cbits = d[7];
    const int w = d[12] | (d[13] << 8), h = d[14] | (d[15] << 8), bpp = d[16], desc = d[17];
    const bool rle = type >= 9, grey = type == 3 || type == 11, mapped = type == 1 || type == 9;
    if (!(type == 1 || type == 2 || type == 3 || type == 9 || type == 10 || type == 11) || (mapped && cmap != 1)) {
        err = "unsupported TGA type";
        return false;
    }
    if (grey ? bpp != 8 : mapped ? bpp != 8 : (bpp != 15 && bpp != 16 && bpp != 24 && bpp != 32)) {
        err = "unsupported TGA pixel depth";
        return false;
    }
    if (!dims_ok(w, h, err)) return false;
    // 15/16-bit colours: x RRRRR GGGGG BBBBB, each channel x 255 / 31 (no alpha)
    auto rgb16 = [](const uint8_t* q, uint8_t* o) {
        const int v = q[0] | (q[1] << 8);
        o[0] = (uint8_t)(((v >> 10) & 31) * 255 / 31);
        o[1] = (uint8_t)(((v >> 5) & 31) * 255 / 31);
        o[2] = (uint8_t)((v & 31) * 255 / 31);
        o[3] = 255;
    };
    const int px = (bpp + 7) / 8;
    size_t pos = 18 + (size_t)idlen;
    // colour map (present in any type when cmap == 1): clen entries of cbits.
    // stb_image, which the reference loads through, takes the first-entry
    // field as a count of bytes to skip before the entries of a mapped image
    // and ignores the map of other types; this reader does the same.
    std::vector<uint8_t> colours;                        // RGBA per entry
    if (cmap == 1 && !mapped) {
        pos += (size_t)clen * ((cbits + 7) / 8);         // not used
    } else if (cmap == 1) {
        pos += (size_t)cfirst;
        const int cb = (cbits + 7) / 8;
        if (clen == 0) { err = "bad TGA colour map"; return false; }
        if (!(cbits == 15 || cbits == 16 || cbits == 24 || cbits == 32)) { err = "bad TGA colour map"; return false; }
        if (pos + (size_t)clen * cb > n) { err = "TGA colour map truncated"; return false; }
        colours.assign((size_t)clen * 4, 255);
        for (int i = 0; i < clen; ++i) {
            const uint8_t* q = d + pos + (size_t)i * cb;
            uint8_t* o = colours.data() + (size_t)i * 4;
            if (cb == 2) {
                rgb16(q, o);
            } else {
                o[0] = q[2]; o[1] = q[1]; o[2] = q[0];
                if (cb == 4) o[3] = q[3];
            }
        }
        pos += (size_t)clen * cb;
    }
    // raw data holds every byte; a run-length packet of 1 + px bytes at most 128 pixels
    if ((size_t)w * h * px > (rle ? 128 * n : n)) { err = "TGA data too short"; return false; }
    std::vector<uint8_t> raw((size_t)w * h * px);
    if (!rle) {
        if (pos + raw.size() > n) { err = "TGA data too short"; return false; }
        std::copy(d + pos, d + pos + raw.size(), raw.begin());
    } else {
        size_t o = 0;
        while (o < raw.size()) {
            if (pos >= n) { err = "TGA data too short"; return false; }
            const int c = d[pos++];
            // a packet that runs past the last pixel ends with the image (as
            // stb_image, the reference's loader, reads it)
            const int count = (int)std::min<size_t>((size_t)(c & 0x7F) + 1, (raw.size() - o) / px);
            if (c & 0x80) {                               // one pixel repeated
                if (pos + px > n) { err = "TGA data too short"; return false; }
                for (int i = 0; i < count; ++i, o += px) std::copy(d + pos, d + pos + px, raw.begin() + o);
                pos += px;
            } else {                                      // count literal pixels
                if (pos + (size_t)count * px > n) { err = "TGA data too short"; return false; }
                std::copy(d + pos, d + pos + (size_t)count * px, raw.begin() + o);
                pos += (size_t)count * px;
                o += (size_t)count * px;
            }
        }
    }
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 255);
    const bool top_down = (desc >> 5) & 1;
    for (int y = 0; y < h; ++y) {
        const uint8_t* s = raw.data() + (size_t)(top_down ? y : h - 1 - y) * w * px;
        uint8_t* o = img.rgba.data() + (size_t)y * w * 4;
        for (int x = 0; x < w; ++x, s += px, o += 4) {
            if (grey) { o[0] = o[1] = o[2] = s[0]; continue; }
            if (mapped) {
                // the index is used as stored, an index past the colour map
                // takes entry 0 (stb_image's reading)
                const int i = s[0] < clen ? s[0] : 0;
                memcpy(o, colours.data() + (size_t)i * 4, 4);
                continue;
            }
            if (px == 2) { rgb16(s, o); continue; }
            o[0] = s[2]; o[1] = s[1]; o[2] = s[0];
            if (px == 4) o[3] = s[3];
        }
    }
    return true;
}

// Windows BMP with a BITMAPINFOHEADER (or later): 1/4/8-bit palettes, 16-bit
// (5:5:5 or bit fields), 24-bit BGR and 32-bit BGRA (or bit fields); rows
// bottom-up unless the height is negative, padded to 4 bytes.
bool decode_bmp(const uint8_t* d, size_t n, Image& img, std::string& err) {
    auto u16 = [&](size_t o) { return (uint32_t)d[o] | ((uint32_t)d[o + 1] << 8); };
    auto u32 = [&](size_t o) { return u16(o) | (u16(o + 2) << 16); };
    if (n < 54 || d[0] != 'B' || d[1] != 'M') { err = "not a BMP file"; return false; }
    const uint32_t off = u32(10), hdr = u32(14);
    if (hdr < 40) { err = "unsupported BMP header"; return false; }
    const int w = (int)u32(18), hraw = (int)u32(22), bpp = (int)u16(28), comp = (int)u32(30);
    const bool top_down = hraw < 0;
    const long long h64 = top_down ? -(long long)hraw : (long long)hraw;
    if (!dims_ok(w, h64, err)) return false;
    const int h = (int)h64;
    const bool pal = bpp == 1 || bpp == 4 || bpp == 8;
    if (!(pal || bpp == 16 || bpp == 24 || bpp == 32) ||
        !(comp == 0 || (comp == 3 && (bpp == 16 || bpp == 32)))) {
        err = "unsupported BMP format (1/4/8/16/24/32-bit uncompressed or 16/32-bit bit fields)";
        return false;
    }
    uint32_t mask[4] = {0x00FF0000u, 0x0000FF00u, 0x000000FFu, bpp == 32 ? 0xFF000000u : 0u};
    if (bpp == 16) { mask[0] = 0x7C00u; mask[1] = 0x03E0u; mask[2] = 0x001Fu; mask[3] = 0u; }   // 5:5:5
    if (comp == 3) {
        if (14 + 40 + 12 > n) { err = "BMP masks missing"; return false; }
        for (int c = 0; c < 3; ++c) mask[c] = u32(54 + 4 * c);
        mask[3] = hdr >= 56 && 14 + 56 <= n ? u32(54 + 12) : 0u;
    }
    // palette: after the header (and the masks of a 40-byte header with bit fields), B G R x
    uint8_t palette[256][3] = {};
    int ncolors = 0;
    if (pal) {
        const uint32_t used = u32(46);
        ncolors = used == 0 || used > (1u << bpp) ? 1 << bpp : (int)used;
        const size_t at = 14 + (size_t)hdr;
        if (at + 4 * (size_t)ncolors > n) { err = "BMP palette missing"; return false; }
        for (int i = 0; i < ncolors; ++i)
            for (int c = 0; c < 3; ++c) palette[i][c] = d[at + 4 * i + 2 - c];
    }
    const size_t stride = (((size_t)w * bpp + 31) / 32) * 4;
    if ((size_t)off + stride * h > n) { err = "BMP data too short"; return false; }
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 255);
    // a mask's field widened to 8 bits the way stb_image -- the reference's
    // loader -- widens it: the masked value is moved so the mask's top bit
    // sits at bit 7, its top n bits (n = the mask's bit count) are the field,
    // and the field's bits repeat to fill 8 bits (a 5-bit 11000 reads
    // 11000110); a field of 8 bits or more keeps the 8 below the top bit
    auto channel = [](uint32_t v, uint32_t m) -> uint8_t {
        if (!m) return 255;
        int hb = 31, n = 0;
        while (!((m >> hb) & 1)) --hb;
        for (int i = 0; i < 32; ++i) n += (m >> i) & 1;
        const uint32_t y = (hb >= 7 ? (v & m) >> (hb - 7) : (v & m) << (7 - hb)) & 0xFFu;
        if (n >= 8) return (uint8_t)y;
        const uint32_t x = y >> (8 - n);
        uint32_t acc = 0;
        int bits = 0;
        while (bits < 8) { acc = (acc << n) | x; bits += n; }
        return (uint8_t)(acc >> (bits - 8));
    };
    for (int y = 0; y < h; ++y) {
        const uint8_t* s = d + off + (size_t)(top_down ? y : h - 1 - y) * stride;
        uint8_t* o = img.rgba.data() + (size_t)y * w * 4;
        for (int x = 0; x < w; ++x, o += 4) {
            if (pal) {
                const size_t bit = (size_t)x * bpp;
                const int idx = (s[bit >> 3] >> (8 - bpp - (bit & 7))) & ((1 << bpp) - 1);
                if (idx >= ncolors) { err = "BMP palette index out of range"; return false; }
                o[0] = palette[idx][0]; o[1] = palette[idx][1]; o[2] = palette[idx][2];
            } else if (bpp == 24) {
                o[0] = s[3 * x + 2]; o[1] = s[3 * x + 1]; o[2] = s[3 * x];
            } else {
                const uint32_t v = bpp == 16 ? (uint32_t)s[2 * x] | ((uint32_t)s[2 * x + 1] << 8)
                                             : (uint32_t)s[4 * x] | ((uint32_t)s[4 * x + 1] << 8) |
                                                   ((uint32_t)s[4 * x + 2] << 16) | ((uint32_t)s[4 * x + 3] << 24);
                for (int c = 0; c < 4; ++c) o[c] = channel(v, mask[c]);
            }
        }
    }
    // many 32-bit BI_RGB files leave the fourth byte 0 everywhere: read as
    // opaque (stb_image, the reference's loader, does the same for 40- and
    // 56-byte headers)
    if (bpp == 32 && comp == 0 && (hdr == 40 || hdr == 56)) {
        uint8_t any = 0;
        for (size_t i = 3; i < img.rgba.size(); i += 4) any |= img.rgba[i];
        if (!any)
            for (size_t i = 3; i < img.rgba.size(); i += 4) img.rgba[i] = 255;
    }
    return true;
}

// Baseline and progressive JPEG (ITU-T T.81: SOF0 / SOF1 / SOF2, 8-bit
// samples, Huffman coding; one grey or three YCbCr components with sampling
// factors 1..2; interleaved and single-component scans; spectral selection and
// successive approximation (Annex G); restart intervals).  The scans fill each
// component's quantised coefficients; then every block is dequantised and
// taken through a separable floating-point inverse DCT (+128, rounded,
// clamped), chroma is upsampled by replication and converted with the JFIF
// equations.  Arithmetic-coded, lossless, hierarchical, 12-bit and CMYK files
// are refused.
namespace {

struct JpegHuff {
    uint8_t count[17] = {};                  // codes of each length 1..16
    uint8_t sym[256] = {};
    int mincode[17] = {}, maxcode[18] = {}, valptr[17] = {};
    bool present = false;
    // false when the code lengths over-fill the code space (more codes of a
    // length than the shorter ones leave), which T.81 forbids
    bool build() {
        int code = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            valptr[l] = k;
            mincode[l] = code;
            code += count[l];
            k += count[l];
            if (code > (1 << l)) return false;
            maxcode[l] = count[l] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7FFFFFFF;
        return true;
    }
};

struct JpegBits {
    const uint8_t* d;
    size_t n, pos;
    uint32_t acc = 0;
    int bits = 0;
    bool marker = false;                     // hit a marker: only zero bits follow
    int past = 0;                            // bytes supplied after the data ran out
    int fill_byte() {
        if (marker || pos >= n) { ++past; return 0; }
        uint8_t b = d[pos];
        if (b == 0xFF) {
            const uint8_t nx = pos + 1 < n ? d[pos + 1] : 0;
            if (nx == 0x00) { pos += 2; return 0xFF; }
            marker = true;                   // RSTn or another marker: stop here
            ++past;
            return 0;
        }
        ++pos;
        return b;
    }
    int bit() {
        if (bits == 0) { acc = (uint32_t)fill_byte(); bits = 8; }
        --bits;
        return (int)((acc >> bits) & 1u);
    }
    int get(int k) {
        int v = 0;
        for (int i = 0; i < k; ++i) v = (v << 1) | bit();
        return v;
    }
    void reset() { bits = 0; past = 0; }
};

int jpeg_decode_sym(JpegBits& b, const JpegHuff& h) {
    int code = 0;
    for (int l = 1; l <= 16; ++l) {
        code = (code << 1) | b.bit();
        if (h.count[l] && code <= h.maxcode[l]) return h.sym[h.valptr[l] + code - h.mincode[l]];
    }
    return -1;
}

int jpeg_extend(int v, int t) { return t == 0 ? 0 : (v < (1 << (t - 1)) ? v - (1 << t) + 1 : v); }

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

void jpeg_idct(const float in[64], uint8_t* out, int stride) {
    static float cosv[8][8];
    static bool init = false;
    if (!init) {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                cosv[x][u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0));
        init = true;
    }
    float tmp[64];
    for (int y = 0; y < 8; ++y)                       // rows: over u
        for (int x = 0; x < 8; ++x) {
            float s = 0.0f;
            for (int u = 0; u < 8; ++u) s += cosv[x][u] * in[y * 8 + u];
            tmp[y * 8 + x] = s * 0.5f;
        }
    for (int x = 0; x < 8; ++x)                       // columns: over v
        for (int y = 0; y < 8; ++y) {
            float s = 0.0f;
            for (int v = 0; v < 8; ++v) s += cosv[y][v] * tmp[v * 8 + x];
            const float r = std::floor(s * 0.5f + 128.5f);
            out[y * stride + x] = (uint8_t)(r < 0.0f ? 0 : r > 255.0f ? 255 : r);
        }
}

int16_t clamp16(long long v) { return (int16_t)(v < -32768 ? -32768 : v > 32767 ? 32767 : v); }

// One component: its quantised coefficients, natural order, on the block grid
// of the MCU-padded image (bh x bw blocks of 64).
struct JpegComp {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int bw = 0, bh = 0;          // MCU-padded block grid
    int cbw = 0, cbh = 0;        // blocks a single-component scan covers
    std::vector<int16_t> coef;
    long long pred = 0;          // DC predictor
    bool dc_seen = false;
};

struct JpegScanParams {
    int ss, se, ah, al;
    bool progressive;
};

// One block of a scan (Annex F for sequential, G.1.2 for progressive).
bool jpeg_block(JpegBits& b, const JpegHuff* dc, const JpegHuff* ac, const JpegScanParams& sp, JpegComp& c,
                int16_t* blk, int& eobrun) {
    if (!sp.progressive) {
        const int t = jpeg_decode_sym(b, *dc);
        if (t < 0 || t > 11) return false;
        c.pred += jpeg_extend(b.get(t), t);
        blk[0] = clamp16(c.pred);
        for (int k = 1; k < 64;) {
            const int rs = jpeg_decode_sym(b, *ac);
            if (rs < 0) return false;
            const int r = rs >> 4, sz = rs & 15;
            if (sz == 0) {
                if (r != 15) break;               // EOB
                k += 16;                          // ZRL
                continue;
            }
            k += r;
            if (k > 63) return false;
            blk[kZigzag[k]] = (int16_t)jpeg_extend(b.get(sz), sz);
            ++k;
        }
        return true;
    }
    if (sp.ss == 0) {                               // DC scans
        if (sp.ah == 0) {
            const int t = jpeg_decode_sym(b, *dc);
            if (t < 0 || t > 11) return false;
            c.pred += jpeg_extend(b.get(t), t);
            blk[0] = clamp16(c.pred * (1ll << sp.al));
        } else if (b.bit()) {
            blk[0] = (int16_t)(blk[0] | (1 << sp.al));
        }
        return true;
    }
    if (sp.ah == 0) {                               // AC first scan
        if (eobrun > 0) { --eobrun; return true; }
        for (int k = sp.ss; k <= sp.se;) {
            const int rs = jpeg_decode_sym(b, *ac);
            if (rs < 0) return false;
            const int r = rs >> 4, sz = rs & 15;
            if (sz == 0) {
                if (r < 15) {                       // EOB run
                    eobrun = (1 << r) - 1;
                    if (r) eobrun += b.get(r);
                    break;
                }
                k += 16;                            // ZRL
                continue;
            }
            k += r;
            if (k > sp.se) return false;
            blk[kZigzag[k]] = clamp16((long long)jpeg_extend(b.get(sz), sz) * (1ll << sp.al));
            ++k;
        }
        return true;
    }
    // AC refinement: a correction bit for every coefficient already nonzero,
    // and newly nonzero coefficients of magnitude 1 << al
    const int p1 = 1 << sp.al, m1 = -p1;
    auto refine = [&](int z) {
        if (b.bit() && (blk[z] & p1) == 0) blk[z] = (int16_t)(blk[z] + (blk[z] >= 0 ? p1 : m1));
    };
    int k = sp.ss;
    if (eobrun == 0) {
        for (; k <= sp.se; ++k) {
            const int rs = jpeg_decode_sym(b, *ac);
            if (rs < 0) return false;
            int r = rs >> 4;
            const int sz = rs & 15;
            int val = 0;
            if (sz) {
                if (sz != 1) return false;
                val = b.bit() ? p1 : m1;
            } else if (r != 15) {                   // EOB run: this block's rest is refined below
                eobrun = 1 << r;
                if (r) eobrun += b.get(r);
                break;
            }
            // skip r coefficients that are still zero, refining the nonzero ones on the way
            for (; k <= sp.se; ++k) {
                const int z = kZigzag[k];
                if (blk[z] != 0) {
                    refine(z);
                } else {
                    if (r == 0) break;
                    --r;
                }
            }
            if (val) {
                if (k > sp.se) return false;
                blk[kZigzag[k]] = (int16_t)val;
            }
        }
    }
    if (eobrun > 0) {
        for (; k <= sp.se; ++k)
            if (blk[kZigzag[k]] != 0) refine(kZigzag[k]);
        --eobrun;
    }
    return true;
}

}  // namespace

bool decode_jpeg(const uint8_t* d, size_t n, Image& img, std::string& err) {
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) { err = "not a JPEG file"; return false; }
    uint16_t qt[4][64] = {};
    JpegHuff hdc[4], hac[4];
    std::vector<JpegComp> comps;
    int width = 0, height = 0, restart = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0, scans = 0;
    bool frame = false, progressive = false;
    size_t pos = 2;
    auto u16 = [&](size_t o) { return (int)((d[o] << 8) | d[o + 1]); };
    while (pos + 4 <= n) {
        if (d[pos] != 0xFF) { ++pos; continue; }
        const int m = d[pos + 1];
        if (m == 0xFF) { ++pos; continue; }
        if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) { pos += 2; continue; }
        if (m == 0xD9) break;
        const int len = u16(pos + 2);
        const size_t seg = pos + 4, end = pos + 2 + (size_t)len;
        if (len < 2 || end > n) { err = "JPEG segment past the end"; return false; }
        const size_t need = m == 0xC0 || m == 0xC1 || m == 0xC2 ? 6 : m == 0xDD ? 2 : m == 0xDA ? 1 : 0;
        if (seg + need > end) { err = "JPEG segment too short"; return false; }
        if (m == 0xDB) {                                          // DQT
            for (size_t o = seg; o < end;) {
                const int pq = d[o] >> 4, tq = d[o] & 15;
                ++o;
                if (tq > 3 || o + (pq ? 128 : 64) > end) { err = "bad JPEG quantisation table"; return false; }
                for (int i = 0; i < 64; ++i) qt[tq][kZigzag[i]] = pq ? (uint16_t)u16(o + 2 * i) : d[o + i];
                o += pq ? 128 : 64;
            }
        } else if (m == 0xC4) {                                   // DHT
            for (size_t o = seg; o < end;) {
                const int tc = d[o] >> 4, th = d[o] & 15;
                if (tc > 1 || th > 3 || o + 17 > end) { err = "bad JPEG Huffman table"; return false; }
                JpegHuff& h = tc ? hac[th] : hdc[th];
                int total = 0;
                for (int l = 1; l <= 16; ++l) { h.count[l] = d[o + l]; total += h.count[l]; }
                if (total > 256 || o + 17 + total > end) { err = "bad JPEG Huffman table"; return false; }
                for (int i = 0; i < total; ++i) h.sym[i] = d[o + 17 + i];
                if (!h.build()) { err = "bad JPEG Huffman table"; return false; }
                h.present = true;
                o += 17 + total;
            }
        } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) {         // SOF0 / SOF1 / SOF2
            if (frame) { err = "JPEG with more than one frame"; return false; }
            if (d[seg] != 8) { err = "only 8-bit JPEG is read"; return false; }
            progressive = m == 0xC2;
            height = u16(seg + 1);
            width = u16(seg + 3);
            const int nc = d[seg + 5];
            if (!dims_ok(width, height, err)) return false;
            if ((nc != 1 && nc != 3) || seg + 6 + 3 * (size_t)nc > end) {
                err = "unsupported JPEG frame (grey or YCbCr only)";
                return false;
            }
            for (int i = 0; i < nc; ++i) {
                JpegComp c;
                c.id = d[seg + 6 + 3 * i];
                c.h = d[seg + 7 + 3 * i] >> 4;
                c.v = d[seg + 7 + 3 * i] & 15;
                c.tq = d[seg + 8 + 3 * i] & 3;
                if (c.h < 1 || c.h > 2 || c.v < 1 || c.v > 2) { err = "unsupported JPEG sampling"; return false; }
                hmax = std::max(hmax, c.h);
                vmax = std::max(vmax, c.v);
                comps.push_back(c);
            }
            if (nc == 1) comps[0].h = comps[0].v = hmax = vmax = 1;   // one component: blocks in raster order
            mcux = (width + 8 * hmax - 1) / (8 * hmax);
            mcuy = (height + 8 * vmax - 1) / (8 * vmax);
            for (auto& c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.cbw = ((width * c.h + hmax - 1) / hmax + 7) / 8;
                c.cbh = ((height * c.v + vmax - 1) / vmax + 7) / 8;
            }
            frame = true;
        } else if ((m >= 0xC3 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            err = "lossless, hierarchical or arithmetic-coded JPEG is not read";
            return false;
        } else if (m == 0xDD) {                                   // DRI
            restart = u16(seg);
        } else if (m == 0xDA) {                                   // SOS
            if (!frame) { err = "JPEG scan before the frame header"; return false; }
            if (++scans > 256) { err = "too many JPEG scans"; return false; }
            const int ns = d[seg];
            if (ns < 1 || ns > (int)comps.size() || seg + 4 + 2 * (size_t)ns > end) {
                err = "bad JPEG scan header";
                return false;
            }
            std::vector<JpegComp*> sc;
            for (int i = 0; i < ns; ++i) {
                const int id = d[seg + 1 + 2 * i], t = d[seg + 2 + 2 * i];
                JpegComp* found = nullptr;
                for (auto& c : comps)
                    if (c.id == id) found = &c;
                if (!found) { err = "JPEG scan names an unknown component"; return false; }
                found->td = t >> 4;
                found->ta = t & 15;
                sc.push_back(found);
            }
            const size_t q = seg + 1 + 2 * (size_t)ns;
            const JpegScanParams sp{d[q], d[q + 1], d[q + 2] >> 4, d[q + 2] & 15, progressive};
            if (!progressive ? (sp.ss != 0 || sp.se != 63 || sp.ah || sp.al)
                             : (sp.se > 63 || sp.ss > sp.se || (sp.ss == 0 && sp.se != 0) || (sp.ss > 0 && ns != 1) ||
                                sp.ah > 13 || sp.al > 13)) {
                err = "bad JPEG scan parameters";
                return false;
            }
            const bool dc_first = sp.ss == 0 && sp.ah == 0;
            for (JpegComp* c : sc) {
                if ((dc_first || sp.ss == 0) ? (c->td > 3 || (dc_first && !hdc[c->td].present))
                                             : (c->ta > 3 || !hac[c->ta].present)) {
                    err = "JPEG Huffman table missing";
                    return false;
                }
                if (!progressive && (c->ta > 3 || !hac[c->ta].present)) { err = "JPEG Huffman table missing"; return false; }
                if (c->coef.empty()) {
                    // a component's first scan codes its DC: at least one bit per block (two in a
                    // sequential scan), which bounds the work by the file's size
                    if (!dc_first) { err = "JPEG AC scan before the DC scan"; return false; }
                    const long long blocks = ns == 1 ? (long long)c->cbw * c->cbh : (long long)c->bw * c->bh;
                    if (blocks > 8ll * (long long)(n - end) + 64) { err = "JPEG data too short for its size"; return false; }
                    c->coef.assign((size_t)c->bw * c->bh * 64, 0);
                }
                c->pred = 0;
            }
            JpegBits bits{d, n, end};
            int eobrun = 0, units = 0;
            const long long nunits = ns == 1 ? (long long)sc[0]->cbw * sc[0]->cbh : (long long)mcux * mcuy;
            for (long long u = 0; u < nunits; ++u) {
                if (restart && units > 0 && units % restart == 0) {
                    // the RSTn marker ends the interval: realign, reset predictors and EOB runs
                    bits.reset();
                    while (bits.pos + 1 < n && !(d[bits.pos] == 0xFF && d[bits.pos + 1] >= 0xD0 &&
                                                 d[bits.pos + 1] <= 0xD7))
                        ++bits.pos;
                    bits.pos += 2;
                    bits.marker = false;
                    eobrun = 0;
                    for (JpegComp* c : sc) c->pred = 0;
                }
                ++units;
                for (JpegComp* c : sc) {
                    const int nby = ns == 1 ? 1 : c->v, nbx = ns == 1 ? 1 : c->h;
                    for (int by = 0; by < nby; ++by)
                        for (int bx = 0; bx < nbx; ++bx) {
                            const long long row = ns == 1 ? u / c->cbw : (u / mcux) * c->v + by;
                            const long long col = ns == 1 ? u % c->cbw : (u % mcux) * c->h + bx;
                            int16_t* blk = c->coef.data() + ((size_t)row * c->bw + (size_t)col) * 64;
                            if (!jpeg_block(bits, &hdc[c->td & 3], &hac[c->ta & 3], sp, *c, blk, eobrun)) {
                                err = "corrupt JPEG data";
                                return false;
                            }
                        }
                    if (dc_first) c->dc_seen = true;
                }
                if (bits.past > 8) { err = "JPEG data too short"; return false; }
            }
            // continue after the entropy-coded data, at the next marker that is not RSTn
            size_t p = bits.pos;
            while (p + 1 < n && !(d[p] == 0xFF && d[p + 1] != 0x00 && !(d[p + 1] >= 0xD0 && d[p + 1] <= 0xD7))) ++p;
            pos = p;
            continue;
        }
        pos = end;
    }
    if (!frame || scans == 0) { err = "JPEG has no image scan"; return false; }
    for (auto& c : comps)
        if (!c.dc_seen) { err = "JPEG component without a scan"; return false; }
    // dequantise and inverse-transform every block into the component planes
    std::vector<std::vector<uint8_t>> planes(comps.size());
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        const JpegComp& c = comps[ci];
        const int pw = c.bw * 8;
        planes[ci].assign((size_t)pw * c.bh * 8, 0);
        float blk[64];
        for (int by = 0; by < c.bh; ++by)
            for (int bx = 0; bx < c.bw; ++bx) {
                const int16_t* q = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
                for (int i = 0; i < 64; ++i) blk[i] = (float)q[i] * (float)qt[c.tq][i];
                jpeg_idct(blk, planes[ci].data() + (size_t)by * 8 * pw + bx * 8, pw);
            }
    }
    img.width = width;
    img.height = height;
    img.rgba.assign((size_t)width * height * 4, 255);
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            float v[3];
            for (size_t c = 0; c < comps.size(); ++c) {
                const JpegComp& k = comps[c];
                const int sx = x * k.h / hmax, sy = y * k.v / vmax;   // replication
                v[c] = planes[c][(size_t)sy * k.bw * 8 + sx];
            }
            uint8_t* o = img.rgba.data() + ((size_t)y * width + x) * 4;
            if (comps.size() == 1) {
                o[0] = o[1] = o[2] = (uint8_t)v[0];
                continue;
            }
            const float cb = v[1] - 128.0f, cr = v[2] - 128.0f;
            const float rgb[3] = {v[0] + 1.402f * cr, v[0] - 0.344136f * cb - 0.714136f * cr, v[0] + 1.772f * cb};
            for (int c = 0; c < 3; ++c) {
                const float r = std::floor(rgb[c] + 0.5f);
                o[c] = (uint8_t)(r < 0.0f ? 0 : r > 255.0f ? 255 : r);
            }
        }
    return true;
}

// Photoshop PSD (version 1), the merged image that follows the layer section:
// greyscale or RGB colour mode, 8 or 16 bits per channel (16-bit channels keep
// their high byte), grey(+alpha) or RGB(+alpha) from the first channels (extra
// channels ignored), raw or PackBits run-length planes.  Photoshop mattes the
// merged image's partly transparent pixels against white (c = a x + (1 - a)
// 255); the matte is removed for alpha A in 1..254 with the reference
// loader's arithmetic: FP32 c / a + 255 (1 - 1 / a), a = A / 255, truncated,
// 0 below 0.
bool decode_psd(const uint8_t* d, size_t n, Image& img, std::string& err) {
    auto be16 = [&](size_t o) { return (uint32_t)((d[o] << 8) | d[o + 1]); };
    auto be32 = [&](size_t o) { return (be16(o) << 16) | be16(o + 2); };
    if (n < 26 || memcmp(d, "8BPS", 4) != 0) { err = "not a PSD file"; return false; }
    if (be16(4) != 1) { err = "only version-1 PSD is read"; return false; }
    const int channels = (int)be16(12), depth = (int)be16(22), mode = (int)be16(24);
    const uint32_t h = be32(14), w = be32(18);
    if (mode != 1 && mode != 3) { err = "PSD colour mode not read (greyscale and RGB are)"; return false; }
    if (depth != 8 && depth != 16) { err = "only 8- and 16-bit PSD is read"; return false; }
    if (channels < 1 || channels > 56) { err = "bad PSD channel count"; return false; }
    if (!dims_ok(w, h, err)) return false;
    size_t pos = 26;
    for (int sec = 0; sec < 3; ++sec) {                   // colour mode data, resources, layers
        if (pos + 4 > n) { err = "PSD truncated"; return false; }
        pos += 4 + (size_t)be32(pos);
    }
    if (pos + 2 > n) { err = "PSD truncated"; return false; }
    const uint32_t comp = be16(pos);
    pos += 2;
    const int bps = depth / 8, used = std::min(channels, mode == 3 ? 4 : 2);
    const size_t row = (size_t)w * bps, plane = row * h;
    std::vector<std::vector<uint8_t>> ch(used, std::vector<uint8_t>((size_t)w * h));
    if (comp == 0) {
        if (pos + plane * used > n) { err = "PSD data too short"; return false; }
        for (int c = 0; c < used; ++c)
            for (size_t i = 0; i < (size_t)w * h; ++i) ch[c][i] = d[pos + c * plane + i * bps];
    } else if (comp == 1) {
        const size_t counts = pos, rows = (size_t)channels * h;
        size_t p = pos + 2 * rows;
        if (p > n) { err = "PSD data too short"; return false; }
        std::vector<uint8_t> line(row);
        for (int c = 0; c < used; ++c)
            for (uint32_t y = 0; y < h; ++y) {
                const size_t len = be16(counts + 2 * ((size_t)c * h + y)), stop = p + len;
                if (stop > n) { err = "PSD data too short"; return false; }
                size_t o = 0;
                while (p < stop && o < row) {                 // PackBits
                    const int k = (int8_t)d[p++];
                    if (k >= 0) {
                        const size_t cnt = (size_t)k + 1;
                        if (p + cnt > stop || o + cnt > row) { err = "bad PSD run"; return false; }
                        memcpy(line.data() + o, d + p, cnt);
                        p += cnt;
                        o += cnt;
                    } else if (k != -128) {
                        const size_t cnt = (size_t)(1 - k);
                        if (p >= stop || o + cnt > row) { err = "bad PSD run"; return false; }
                        memset(line.data() + o, d[p++], cnt);
                        o += cnt;
                    }
                }
                if (o != row) { err = "bad PSD run"; return false; }
                p = stop;
                for (uint32_t x = 0; x < w; ++x) ch[c][(size_t)y * w + x] = line[(size_t)x * bps];
            }
    } else {
        err = "PSD compression not read (raw and run-length are)";
        return false;
    }
    img.width = (int)w;
    img.height = (int)h;
    img.rgba.assign((size_t)w * h * 4, 255);
    const bool has_alpha = used == (mode == 3 ? 4 : 2);
    const int nc = mode == 3 ? std::min(used, 3) : 1;
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        uint8_t* o = img.rgba.data() + i * 4;
        for (int c = 0; c < 3; ++c) o[c] = mode == 3 ? (c < nc ? ch[c][i] : 0) : ch[0][i];
        if (!has_alpha) continue;
        const int a = ch[used - 1][i];
        o[3] = (uint8_t)a;
        if (a == 0 || a == 255) continue;
        // stb_image's arithmetic (the reference's loader): FP32, c / a +
        // 255 (1 - 1 / a) with a = A / 255, truncated; below 0 (where stb
        // converts a negative float, which C leaves undefined) reads 0
        const float af = (float)a / 255.0f, ra = 1.0f / af, inv_a = 255.0f * (1.0f - ra);
        for (int c = 0; c < 3; ++c) {
            const float v = (float)o[c] * ra + inv_a;
            o[c] = v <= 0.0f ? 0 : (uint8_t)(int)v;
        }
    }
    return true;
}

// GIF (87a / 89a), the first image: composed on the logical screen, which
// starts as transparent black (0, 0, 0, 0); global or local palette; the
// graphic control extension's transparent index leaves its pixels at the
// screen's (0, 0, 0, 0); interlaced rows in the format's four passes; LZW with
// variable code width up to 12 bits, clear and end codes.
bool decode_gif(const uint8_t* d, size_t n, Image& img, std::string& err) {
    auto le16 = [&](size_t o) { return (int)(d[o] | (d[o + 1] << 8)); };
    if (n < 13 || memcmp(d, "GIF8", 4) != 0 || (d[4] != '7' && d[4] != '9') || d[5] != 'a') {
        err = "not a GIF file";
        return false;
    }
    const int sw = le16(6), sh = le16(8), flags = d[10];
    if (!dims_ok(sw, sh, err)) return false;
    size_t pos = 13;
    uint8_t gpal[768] = {}, lpal[768] = {};
    int gsize = 0, transparent = -1;
    if (flags & 0x80) {
        gsize = 2 << (flags & 7);
        if (pos + 3 * (size_t)gsize > n) { err = "GIF truncated"; return false; }
        memcpy(gpal, d + pos, 3 * (size_t)gsize);
        pos += 3 * (size_t)gsize;
    }
    while (pos < n) {
        const int b = d[pos++];
        if (b == 0x3B) break;                                   // trailer
        if (b == 0x21) {                                        // extension
            if (pos >= n) break;
            const int label = d[pos++];
            bool first = true;
            while (pos < n && d[pos] != 0) {
                const size_t len = d[pos];
                if (pos + 1 + len > n) { err = "GIF truncated"; return false; }
                if (label == 0xF9 && first && len >= 4) transparent = (d[pos + 1] & 1) ? d[pos + 4] : -1;
                first = false;
                pos += 1 + len;
            }
            ++pos;
            continue;
        }
        if (b != 0x2C) { err = "bad GIF block"; return false; }
        if (pos + 9 > n) { err = "GIF truncated"; return false; }
        const int fx = le16(pos), fy = le16(pos + 2), fw = le16(pos + 4), fh = le16(pos + 6), ff = d[pos + 8];
        pos += 9;
        const uint8_t* pal = gpal;
        int psize = gsize;
        if (ff & 0x80) {
            psize = 2 << (ff & 7);
            if (pos + 3 * (size_t)psize > n) { err = "GIF truncated"; return false; }
            memcpy(lpal, d + pos, 3 * (size_t)psize);
            pos += 3 * (size_t)psize;
            pal = lpal;
        }
        if (pos >= n) { err = "GIF truncated"; return false; }
        const int minsize = d[pos++];
        if (minsize < 2 || minsize > 11) { err = "bad GIF code size"; return false; }
        std::vector<uint8_t> data;                               // the sub-blocks, joined
        while (pos < n && d[pos] != 0) {
            const size_t len = d[pos];
            if (pos + 1 + len > n) { err = "GIF truncated"; return false; }
            data.insert(data.end(), d + pos + 1, d + pos + 1 + len);
            pos += 1 + len;
        }
        // LZW: prefix / suffix tables, strings written backwards into a stack
        const size_t npix = (size_t)fw * fh;
        std::vector<uint8_t> idx;
        idx.reserve(npix);
        const int clear = 1 << minsize, stop = clear + 1;
        std::vector<int> prefix(4096, -1);
        std::vector<uint8_t> suffix(4096, 0), stack(4097);
        for (int i = 0; i < clear; ++i) suffix[i] = (uint8_t)i;
        int width = minsize + 1, next = clear + 2, prev = -1;
        uint8_t firstc = 0;
        size_t bitpos = 0;
        while (idx.size() < npix) {
            if (bitpos + width > data.size() * 8) break;
            int code = 0;
            for (int i = 0; i < width; ++i, ++bitpos) code |= ((data[bitpos >> 3] >> (bitpos & 7)) & 1) << i;
            if (code == clear) { width = minsize + 1; next = clear + 2; prev = -1; continue; }
            if (code == stop) break;
            if (prev < 0) {
                if (code >= clear) { err = "corrupt GIF data"; return false; }
                idx.push_back((uint8_t)code);
                firstc = (uint8_t)code;
                prev = code;
                continue;
            }
            int cur = code, sp = 0;
            if (code > next || (code >= clear && code < clear + 2)) { err = "corrupt GIF data"; return false; }
            if (code == next) { stack[sp++] = firstc; cur = prev; }  // the KwKwK case
            while (cur >= clear) {
                if (sp >= 4096) { err = "corrupt GIF data"; return false; }
                stack[sp++] = suffix[cur];
                cur = prefix[cur];
            }
            stack[sp++] = (uint8_t)cur;
            firstc = (uint8_t)cur;
            while (sp > 0 && idx.size() < npix) idx.push_back(stack[--sp]);
            if (next < 4096) {
                prefix[next] = prev;
                suffix[next] = firstc;
                ++next;
                if (next == (1 << width) && width < 12) ++width;
            }
            prev = code;
        }
        idx.resize(npix, 0);                                     // a short stream leaves index 0
        img.width = sw;
        img.height = sh;
        img.rgba.assign((size_t)sw * sh * 4, 0);
        // row order: interlaced frames store rows 0, 8, 16.., 4, 12.., 2, 6.., 1, 3..
        std::vector<int> rows;
        if (ff & 0x40) {
            const int start[4] = {0, 4, 2, 1}, step[4] = {8, 8, 4, 2};
            for (int p = 0; p < 4; ++p)
                for (int y = start[p]; y < fh; y += step[p]) rows.push_back(y);
        } else {
            for (int y = 0; y < fh; ++y) rows.push_back(y);
        }
        for (int r = 0; r < fh; ++r) {
            const int y = fy + rows[r];
            if (y >= sh) continue;
            for (int x = 0; x < fw; ++x) {
                if (fx + x >= sw) continue;
                const int c = idx[(size_t)r * fw + x];
                if (c == transparent || c >= psize) continue;
                uint8_t* o = img.rgba.data() + ((size_t)y * sw + fx + x) * 4;
                o[0] = pal[3 * c];
                o[1] = pal[3 * c + 1];
                o[2] = pal[3 * c + 2];
                o[3] = 255;
            }
        }
        return true;
    }
    err = "GIF has no image";
    return false;
}

// Radiance HDR (RGBE): "#?RADIANCE" / "#?RGBE" header with
// FORMAT=32-bit_rle_rgbe, resolution "-Y h +X w", flat or run-length
// scanlines (the 2 2 hi lo form, channels coded apart).  Texel (m, e) is
// m x 2^(e - 136) (0 when e = 0); the 8-bit image is what an 8-bit load of the
// reference's image library gives: 255 x v^(1/2.2) + 0.5, clamped and
// truncated, alpha 255.
bool decode_hdr(const uint8_t* d, size_t n, Image& img, std::string& err) {
    size_t pos = 0;
    auto line = [&](std::string& out) {
        out.clear();
        while (pos < n && d[pos] != '\n') out.push_back((char)d[pos++]);
        if (pos >= n) return false;
        ++pos;
        return true;
    };
    std::string l;
    if (!line(l) || (l != "#?RADIANCE" && l != "#?RGBE")) { err = "not a Radiance HDR file"; return false; }
    while (true) {
        if (!line(l)) { err = "HDR header truncated"; return false; }
        if (l.empty()) break;
        if (l.rfind("FORMAT=", 0) == 0) {
            if (l != "FORMAT=32-bit_rle_rgbe") { err = "HDR format not read (32-bit_rle_rgbe is)"; return false; }
        }
    }
    if (!line(l)) { err = "HDR resolution missing"; return false; }
    int h = 0, w = 0;
    char ax[3] = {}, ay[3] = {};
    if (sscanf(l.c_str(), "%2s %d %2s %d", ay, &h, ax, &w) != 4 || strcmp(ay, "-Y") != 0 || strcmp(ax, "+X") != 0) {
        err = "HDR orientation not read (-Y h +X w is)";
        return false;
    }
    if (!dims_ok(w, h, err)) return false;
    if ((size_t)w * h > 64 * (n - pos) + 64) { err = "HDR data too short for its size"; return false; }
    std::vector<uint8_t> rgbe((size_t)w * h * 4);
    for (int y = 0; y < h; ++y) {
        uint8_t* row = rgbe.data() + (size_t)y * w * 4;
        if (w >= 8 && w < 32768 && pos + 4 <= n && d[pos] == 2 && d[pos + 1] == 2 && !(d[pos + 2] & 0x80)) {
            if (((d[pos + 2] << 8) | d[pos + 3]) != w) { err = "bad HDR scanline"; return false; }
            pos += 4;
            for (int c = 0; c < 4; ++c)
                for (int x = 0; x < w;) {
                    if (pos >= n) { err = "HDR data too short"; return false; }
                    int k = d[pos++];
                    if (k > 128) {                               // run
                        k -= 128;
                        if (pos >= n || x + k > w) { err = "bad HDR run"; return false; }
                        for (int i = 0; i < k; ++i) row[(size_t)(x + i) * 4 + c] = d[pos];
                        ++pos;
                    } else {                                     // literal
                        if (k == 0 || pos + k > n || x + k > w) { err = "bad HDR run"; return false; }
                        for (int i = 0; i < k; ++i) row[(size_t)(x + i) * 4 + c] = d[pos + i];
                        pos += k;
                    }
                    x += k;
                }
        } else {
            if (pos + (size_t)w * 4 > n) { err = "HDR data too short"; return false; }
            memcpy(row, d + pos, (size_t)w * 4);
            pos += (size_t)w * 4;
        }
    }
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 255);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        const uint8_t* p = rgbe.data() + i * 4;
        const float f = p[3] ? ldexpf(1.0f, (int)p[3] - 136) : 0.0f;
        for (int c = 0; c < 3; ++c) {
            float z = powf((float)p[c] * f, 1.0f / 2.2f) * 255.0f + 0.5f;
            z = z < 0.0f ? 0.0f : z > 255.0f ? 255.0f : z;
            img.rgba[i * 4 + c] = (uint8_t)(int)z;
        }
    }
    return true;
}

// Softimage PIC: a 104-byte header (magic 0x5380F634, "PICT" at 88, width
// and height big-endian at 92), chained channel packets (8-bit channels, a
// mask of red 0x80, green 0x40, blue 0x20, alpha 0x10; uncompressed, pure
// run-length or mixed run-length), then each scanline top to bottom, packet
// by packet.  Channels no packet carries are 255.
bool decode_pic(const uint8_t* d, size_t n, Image& img, std::string& err) {
    if (n < 104 || !(d[0] == 0x53 && d[1] == 0x80 && d[2] == 0xF6 && d[3] == 0x34) || memcmp(d + 88, "PICT", 4) != 0) {
        err = "not a Softimage PIC file";
        return false;
    }
    const int w = (d[92] << 8) | d[93], h = (d[94] << 8) | d[95];
    if (!dims_ok(w, h, err)) return false;
    size_t pos = 104;
    struct Packet { int type, mask; };
    std::vector<Packet> packets;
    int all = 0;
    for (bool chained = true; chained;) {
        if (pos + 4 > n || packets.size() >= 10) { err = "bad PIC packets"; return false; }
        chained = d[pos] != 0;
        if (d[pos + 1] != 8 || d[pos + 2] > 2) { err = "PIC packet not read (8-bit channels are)"; return false; }
        packets.push_back({d[pos + 2], d[pos + 3]});
        all |= d[pos + 3];
        pos += 4;
    }
    if (!(all & 0xF0)) { err = "PIC without colour channels"; return false; }
    // every pixel of every packet needs a byte at least once per 65535 pixels
    if ((size_t)w * h > 65535ull * (n - pos) + 65535) { err = "PIC data too short for its size"; return false; }
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 255);
    auto put = [&](uint8_t* px, int mask, const uint8_t* vals) {   // vals in channel order R G B A
        int k = 0;
        for (int c = 0; c < 4; ++c)
            if (mask & (0x80 >> c)) px[c] = vals[k++];
    };
    for (int y = 0; y < h; ++y) {
        uint8_t* row = img.rgba.data() + (size_t)y * w * 4;
        for (const Packet& p : packets) {
            int nch = 0;
            for (int c = 0; c < 4; ++c) nch += (p.mask >> (7 - c)) & 1;
            uint8_t vals[4];
            auto read_vals = [&]() {
                if (pos + nch > n) return false;
                memcpy(vals, d + pos, nch);
                pos += nch;
                return true;
            };
            for (int x = 0; x < w;) {
                int count = 0;
                bool literal = false;
                if (p.type == 0) {
                    count = 1;
                    literal = true;
                } else {
                    if (pos >= n) { err = "PIC data too short"; return false; }
                    const int c = d[pos++];
                    if (p.type == 1) {
                        count = c;
                    } else if (c < 128) {
                        count = c + 1;
                        literal = true;
                    } else if (c == 128) {
                        if (pos + 2 > n) { err = "PIC data too short"; return false; }
                        count = (d[pos] << 8) | d[pos + 1];
                        pos += 2;
                    } else {
                        count = c - 127;
                    }
                }
                // a pure run-length packet is cut at the end of the row and may
                // be empty (its value is still read); mixed packets may not
                // overrun the row (what stb_image's reader does)
                if (p.type == 1 && count > w - x) count = w - x;
                if (count < 0 || x + count > w || (count == 0 && literal)) { err = "bad PIC run"; return false; }
                if (!literal && !read_vals()) { err = "PIC data too short"; return false; }
                for (int i = 0; i < count; ++i, ++x) {
                    if (literal && !read_vals()) { err = "PIC data too short"; return false; }
                    put(row + (size_t)x * 4, p.mask, vals);
                }
            }
        }
    }
    return true;
}

bool load_image(const std::string& path, Image& img, std::string& err) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) { err = "cannot open " + path; return false; }
    std::vector<uint8_t> data;
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + got);
    fclose(f);
    if (data.size() >= 8 && data[0] == 0x89 && data[1] == 'P') return decode_png(data.data(), data.size(), img, err);
    if (data.size() >= 2 && data[0] == 'P' && data[1] >= '5' && data[1] <= '7')
        return decode_pnm(data.data(), data.size(), img, err);
    if (data.size() >= 2 && data[0] == 'B' && data[1] == 'M') return decode_bmp(data.data(), data.size(), img, err);
    if (data.size() >= 3 && data[0] == 0xFF && data[1] == 0xD8 && data[2] == 0xFF)
        return decode_jpeg(data.data(), data.size(), img, err);
    if (data.size() >= 4 && memcmp(data.data(), "8BPS", 4) == 0) return decode_psd(data.data(), data.size(), img, err);
    if (data.size() >= 4 && memcmp(data.data(), "GIF8", 4) == 0) return decode_gif(data.data(), data.size(), img, err);
    if (data.size() >= 6 && memcmp(data.data(), "#?RGBE", 6) == 0) return decode_hdr(data.data(), data.size(), img, err);
    if (data.size() >= 4 && data[0] == 0x53 && data[1] == 0x80 && data[2] == 0xF6 && data[3] == 0x34)
        return decode_pic(data.data(), data.size(), img, err);
    if (data.size() >= 10 && memcmp(data.data(), "#?RADIANCE", 10) == 0)
        return decode_hdr(data.data(), data.size(), img, err);
    const size_t dot = path.find_last_of('.');
    std::string ext = dot == std::string::npos ? "" : path.substr(dot + 1);
    for (auto& c : ext) c = (char)tolower((unsigned char)c);
    if (ext == "tga") return decode_tga(data.data(), data.size(), img, err);   // TGA has no magic number
    err = "unsupported image format (PNG, JPEG, PSD, GIF, HDR, PIC, PAM/PPM/PGM, BMP and TGA are read)";
    return false;
}

bool save_pam(const std::string& path, const Image& img, std::string& err) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { err = "cannot open " + path; return false; }
    fprintf(f, "P7\nWIDTH %d\nHEIGHT %d\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n", img.width, img.height);
    const bool ok = fwrite(img.rgba.data(), 1, img.rgba.size(), f) == img.rgba.size();
    if (fclose(f) != 0 || !ok) { err = "write failed: " + path; return false; }
    return true;
}

void flip_vertical(Image& img) {
    const size_t row = (size_t)img.width * 4;
    for (int y = 0; y < img.height / 2; ++y)
        std::swap_ranges(img.rgba.begin() + y * row, img.rgba.begin() + (y + 1) * row,
                         img.rgba.begin() + (size_t)(img.height - 1 - y) * row);
}

}  // namespace astc
