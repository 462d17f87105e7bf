// astc_decode.cu -- integer-only ASTC LDR decoder and per-channel SSE
// reduction on sm_103a.  The reference has no decoder; these kernels give the
// library on-device quality checks (PSNR of an encode without a round trip to
// the host).  Decoding follows the ASTC specification: block mode table, ISE
// (trits/quints), colour and weight unquantisation, LDR colour endpoint modes
// 0/1/4/5/6/8/9/10/12/13 with blue contraction, partition hash, dual plane,
// decimated-grid infill, 16-bit interpolation and UNORM8 (top byte) output.
// Error blocks (reserved modes, HDR) decode to magenta.
#include <cuda_runtime.h>
#include <stdint.h>

#include "astc_block_common.cuh"
#include "astc_internal.h"
#include "astc_sse.cuh"
#include "astc_tables.h"

namespace astc {
namespace {

struct alignas(16) DecodeTables {
    uint8_t trit_unpack[256][5];
    uint8_t quint_unpack[128][3];
    uint8_t weight_unq[12][32];
    uint8_t color_unq[kQuantCount][256];
};

constexpr DecodeTables make_decode_tables() {
    DecodeTables d{};
    const IseTables t = make_ise_tables();
    for (int i = 0; i < 256; ++i)
        for (int k = 0; k < 5; ++k) d.trit_unpack[i][k] = t.trit_unpack[i][k];
    for (int i = 0; i < 128; ++i)
        for (int k = 0; k < 3; ++k) d.quint_unpack[i][k] = t.quint_unpack[i][k];
    for (int q = 0; q < 12; ++q)
        for (int v = 0; v < 32; ++v) d.weight_unq[q][v] = t.weight_unq[q][v];
    for (int q = 0; q < kQuantCount; ++q)
        for (int v = 0; v < 256; ++v) d.color_unq[q][v] = t.color_unq[q][v];
    return d;
}

__constant__ DecodeTables c_dec = make_decode_tables();

constexpr int kDecodeThreads = 256;

struct Bits {
    uint32_t w[4];
    __device__ uint32_t read(int pos, int count) const {
        if (count <= 0 || pos >= 128 || pos < 0) return 0;
        const int wi = pos >> 5, sh = pos & 31;
        uint64_t v = w[wi];
        if (wi + 1 < 4) v |= (uint64_t)w[wi + 1] << 32;
        return (uint32_t)(v >> sh) & (count >= 32 ? 0xFFFFFFFFu : ((1u << count) - 1u));
    }
};

// Bits at or past the end of the sequence (pos + its ISE length) read as
// zero: the last trit or quint group is stored cut to the sequence's length,
// and whatever follows in the block (endpoints, a dual-plane selector) is not
// part of it.
struct BoundedBits {
    const Bits& b;
    int end;
    __device__ uint32_t read(int pos, int count) const {
        if (pos >= end) return 0;
        const int n = pos + count > end ? end - pos : count;
        return b.read(pos, n);
    }
};

__device__ void ise_decode(const DecodeTables& T, int quant, int count, const Bits& bits, int pos,
                           uint8_t* out) {
    const RangeShape s = range_shape(quant);
    const BoundedBits b{bits, pos + ise_bit_count(quant, count)};
    if (s.trits) {
        for (int g = 0; g < count; g += 5) {
            uint32_t m[5], tb = 0;
            const int tbits[5] = {2, 2, 1, 2, 1};
            int tsh = 0;
            for (int i = 0; i < 5; ++i) {
                m[i] = b.read(pos, s.bits); pos += s.bits;
                tb |= b.read(pos, tbits[i]) << tsh;
                pos += tbits[i]; tsh += tbits[i];
            }
            for (int i = 0; i < 5 && g + i < count; ++i)
                out[g + i] = (uint8_t)((T.trit_unpack[tb][i] << s.bits) | m[i]);
        }
    } else if (s.quints) {
        for (int g = 0; g < count; g += 3) {
            uint32_t m[3], qb = 0;
            const int qbits[3] = {3, 2, 2};
            int qsh = 0;
            for (int i = 0; i < 3; ++i) {
                m[i] = b.read(pos, s.bits); pos += s.bits;
                qb |= b.read(pos, qbits[i]) << qsh;
                pos += qbits[i]; qsh += qbits[i];
            }
            for (int i = 0; i < 3 && g + i < count; ++i)
                out[g + i] = (uint8_t)((T.quint_unpack[qb][i] << s.bits) | m[i]);
        }
    } else {
        for (int i = 0; i < count; ++i) { out[i] = (uint8_t)b.read(pos, s.bits); pos += s.bits; }
    }
}

__device__ __forceinline__ int clamp255(int v) { return v < 0 ? 0 : v > 255 ? 255 : v; }

__device__ __forceinline__ void bit_transfer_signed(int& a, int& b) {
    b >>= 1;
    b |= a & 0x80;
    a >>= 1;
    a &= 0x3F;
    if (a & 0x20) a -= 0x40;
}

__device__ __forceinline__ void blue_contract(int c[4]) {
    c[0] = (c[0] + c[2]) >> 1;
    c[1] = (c[1] + c[2]) >> 1;
}

__device__ bool unpack_endpoints(int cem, const int* v, int e0[4], int e1[4]) {
    switch (cem) {
    case 0:
        e0[0] = e0[1] = e0[2] = v[0]; e0[3] = 255;
        e1[0] = e1[1] = e1[2] = v[1]; e1[3] = 255;
        return true;
    case 1: {
        const int l0 = (v[0] >> 2) | (v[1] & 0xC0);
        const int l1 = min(l0 + (v[1] & 0x3F), 255);
        e0[0] = e0[1] = e0[2] = l0; e0[3] = 255;
        e1[0] = e1[1] = e1[2] = l1; e1[3] = 255;
        return true;
    }
    case 4:
        e0[0] = e0[1] = e0[2] = v[0]; e0[3] = v[2];
        e1[0] = e1[1] = e1[2] = v[1]; e1[3] = v[3];
        return true;
    case 5: {
        int a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3];
        bit_transfer_signed(a1, a0);
        bit_transfer_signed(a3, a2);
        e0[0] = e0[1] = e0[2] = a0; e0[3] = a2;
        const int l = clamp255(a0 + a1);
        e1[0] = e1[1] = e1[2] = l; e1[3] = clamp255(a2 + a3);
        return true;
    }
    case 6:
        e0[0] = (v[0] * v[3]) >> 8; e0[1] = (v[1] * v[3]) >> 8; e0[2] = (v[2] * v[3]) >> 8; e0[3] = 255;
        e1[0] = v[0]; e1[1] = v[1]; e1[2] = v[2]; e1[3] = 255;
        return true;
    case 8:
    case 12: {
        const int a0 = cem == 12 ? v[6] : 255, a1 = cem == 12 ? v[7] : 255;
        if (v[1] + v[3] + v[5] >= v[0] + v[2] + v[4]) {
            e0[0] = v[0]; e0[1] = v[2]; e0[2] = v[4]; e0[3] = a0;
            e1[0] = v[1]; e1[1] = v[3]; e1[2] = v[5]; e1[3] = a1;
        } else {
            e0[0] = v[1]; e0[1] = v[3]; e0[2] = v[5]; e0[3] = a1;
            e1[0] = v[0]; e1[1] = v[2]; e1[2] = v[4]; e1[3] = a0;
            blue_contract(e0);
            blue_contract(e1);
        }
        return true;
    }
    case 9:
    case 13: {
        int a[8];
        for (int i = 0; i < 8; ++i) a[i] = i < (cem == 13 ? 8 : 6) ? v[i] : 255;
        bit_transfer_signed(a[1], a[0]);
        bit_transfer_signed(a[3], a[2]);
        bit_transfer_signed(a[5], a[4]);
        if (cem == 13) bit_transfer_signed(a[7], a[6]);
        const int al0 = cem == 13 ? a[6] : 255;
        const int al1 = cem == 13 ? clamp255(a[6] + a[7]) : 255;
        if (a[1] + a[3] + a[5] >= 0) {
            e0[0] = a[0]; e0[1] = a[2]; e0[2] = a[4]; e0[3] = al0;
            e1[0] = clamp255(a[0] + a[1]); e1[1] = clamp255(a[2] + a[3]);
            e1[2] = clamp255(a[4] + a[5]); e1[3] = al1;
        } else {
            e0[0] = a[0] + a[1]; e0[1] = a[2] + a[3]; e0[2] = a[4] + a[5]; e0[3] = al1;
            e1[0] = a[0]; e1[1] = a[2]; e1[2] = a[4]; e1[3] = al0;
            blue_contract(e0);
            blue_contract(e1);
            for (int c = 0; c < 4; ++c) { e0[c] = clamp255(e0[c]); e1[c] = clamp255(e1[c]); }
        }
        return true;
    }
    case 10:
        e0[0] = (v[0] * v[3]) >> 8; e0[1] = (v[1] * v[3]) >> 8; e0[2] = (v[2] * v[3]) >> 8; e0[3] = v[4];
        e1[0] = v[0]; e1[1] = v[1]; e1[2] = v[2]; e1[3] = v[5];
        return true;
    default:
        return false;
    }
}

__device__ int select_partition(int seed, int x, int y, int pcount, bool small) {
    if (small) { x <<= 1; y <<= 1; }
    seed += (pcount - 1) * 1024;
    uint32_t p = (uint32_t)seed;
    p ^= p >> 15; p -= p << 17; p += p << 7; p += p << 4;
    p ^= p >> 5;  p += p << 16; p ^= p >> 7; p ^= p >> 3;
    p ^= p << 6;  p ^= p >> 17;
    int s[12];
    for (int i = 0; i < 8; ++i) s[i] = (p >> (4 * i)) & 0xF;
    s[8] = (p >> 18) & 0xF;
    s[9] = (p >> 22) & 0xF;
    s[10] = (p >> 26) & 0xF;
    s[11] = ((p >> 30) | (p << 2)) & 0xF;
    for (int i = 0; i < 12; ++i) s[i] *= s[i];
    int sh1, sh2;
    if (seed & 1) { sh1 = (seed & 2) ? 4 : 5; sh2 = pcount == 3 ? 6 : 5; }
    else { sh1 = pcount == 3 ? 6 : 5; sh2 = (seed & 2) ? 4 : 5; }
    const int sh3 = (seed & 0x10) ? sh1 : sh2;
    s[0] >>= sh1; s[1] >>= sh2; s[2] >>= sh1; s[3] >>= sh2;
    s[4] >>= sh1; s[5] >>= sh2; s[6] >>= sh1; s[7] >>= sh2;
    s[8] >>= sh3; s[9] >>= sh3; s[10] >>= sh3; s[11] >>= sh3;
    // z = 0 for 2-D blocks
    int a = (s[0] * x + s[1] * y + (int)(p >> 14)) & 0x3F;
    int b = (s[2] * x + s[3] * y + (int)(p >> 10)) & 0x3F;
    int c = (s[4] * x + s[5] * y + (int)(p >> 6)) & 0x3F;
    int d = (s[6] * x + s[7] * y + (int)(p >> 2)) & 0x3F;
    if (pcount < 4) d = 0;
    if (pcount < 3) c = 0;
    if (a >= b && a >= c && a >= d) return 0;
    if (b >= c && b >= d) return 1;
    if (c >= d) return 2;
    return 3;
}

struct Mode { int gw, gh, dual, quant, ok; };

__device__ Mode block_mode(int m) {
    Mode r = {0, 0, 0, 0, 0};
    int R, H = (m >> 9) & 1, D = (m >> 10) & 1;
    if ((m & 3) != 0) {
        R = ((m >> 4) & 1) | ((m & 1) << 1) | (((m >> 1) & 1) << 2);
        const int A = (m >> 5) & 3, B = (m >> 7) & 3;
        switch ((m >> 2) & 3) {
        case 0: r.gw = B + 4; r.gh = A + 2; break;
        case 1: r.gw = B + 8; r.gh = A + 2; break;
        case 2: r.gw = A + 2; r.gh = B + 8; break;
        default:
            if (((m >> 8) & 1) == 0) { r.gw = A + 2; r.gh = ((m >> 7) & 1) + 6; }
            else { r.gw = ((m >> 7) & 1) + 2; r.gh = A + 2; }
        }
    } else {
        if (((m >> 2) & 3) == 0) return r;
        R = ((m >> 4) & 1) | (((m >> 2) & 1) << 1) | (((m >> 3) & 1) << 2);
        const int A = (m >> 5) & 3;
        switch ((m >> 7) & 3) {
        case 0: r.gw = 12; r.gh = A + 2; break;
        case 1: r.gw = A + 2; r.gh = 12; break;
        case 3:
            if ((m >> 6) & 1) return r;
            if (((m >> 5) & 1) == 0) { r.gw = 6; r.gh = 10; } else { r.gw = 10; r.gh = 6; }
            break;
        default:
            r.gw = A + 6; r.gh = ((m >> 9) & 3) + 6; H = 0; D = 0;
        }
    }
    r.dual = D;
    r.quant = (R - 2) + 6 * H;
    r.ok = 1;
    return r;
}

__device__ __forceinline__ uint32_t rev32(uint32_t v) { return __brev(v); }

// The blocks the fixed-mode encoder writes (single partition, a 4x4 weight
// grid in QUANT_6 trits with CEM 8 or 12, or in QUANT_12 trits with CEM 8;
// both leave room for QUANT_256 endpoints; no dual plane) decoded with the
// block and grid sizes known at compile time:
// the same arithmetic as the general path below, unrolled into registers.
// Q = kQuant6 (1 bit + trit per weight) or kQuant12 (2 bits + trit).
template <int DIM, int Q, class Sink>
__device__ __forceinline__ void decode_fixed_grid4(const DecodeTables& T, const uint4 raw, bool alpha, bool srgb,
                                                   Sink&& sink) {
    constexpr int B = Q == kQuant6 ? 1 : 2;
    constexpr int GW = 5 * B + 8;
    constexpr int NBITS = ise_bit_count(Q, 16);
    // endpoint bytes from bit 17: r0 r1 g0 g1 b0 b1 [a0 a1]
    const uint64_t lo = ((uint64_t)raw.y << 32) | raw.x;
    const uint64_t ep = (lo >> 17) | ((uint64_t)raw.z << 47);
    int v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (int)((ep >> (8 * i)) & 0xFFu);
    const int a0 = alpha ? v[6] : 255, a1 = alpha ? v[7] : 255;
    int e0[4], e1[4];
    if (v[1] + v[3] + v[5] >= v[0] + v[2] + v[4]) {
        e0[0] = v[0]; e0[1] = v[2]; e0[2] = v[4]; e0[3] = a0;
        e1[0] = v[1]; e1[1] = v[3]; e1[2] = v[5]; e1[3] = a1;
    } else {
        e0[0] = (v[1] + v[5]) >> 1; e0[1] = (v[3] + v[5]) >> 1; e0[2] = v[5]; e0[3] = a1;
        e1[0] = (v[0] + v[4]) >> 1; e1[1] = (v[2] + v[4]) >> 1; e1[2] = v[4]; e1[3] = a0;
    }
    // the weight stream, bit i = block bit 127 - i, cut to its length
    const uint64_t ws = __brevll(((uint64_t)raw.w << 32) | raw.z) & ((1ull << NBITS) - 1ull);
    int wv[16];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        const uint32_t grp = (uint32_t)(ws >> (g * GW));
        constexpr uint32_t M = (1u << B) - 1u;
        const uint32_t m[5] = {grp & M, (grp >> (B + 2)) & M, (grp >> (2 * B + 4)) & M, (grp >> (3 * B + 5)) & M,
                               (grp >> (4 * B + 7)) & M};
        const uint32_t t = ((grp >> B) & 3u) | (((grp >> (2 * B + 2)) & 3u) << 2) | (((grp >> (3 * B + 4)) & 1u) << 4) |
                           (((grp >> (4 * B + 5)) & 3u) << 5) | (((grp >> (5 * B + 7)) & 1u) << 7);
#pragma unroll
        for (int i = 0; i < 5; ++i)
            if (5 * g + i < 16) wv[5 * g + i] = T.weight_unq[Q][(T.trit_unpack[t][i] << B) | m[i]];
    }
    constexpr int ds = (1024 + DIM / 2) / (DIM - 1);
    uint32_t row[DIM];
#pragma unroll
    for (int t = 0; t < DIM; ++t)
#pragma unroll
        for (int s = 0; s < DIM; ++s) {
            const int gs = (ds * s * 3 + 32) >> 6, gt = (ds * t * 3 + 32) >> 6;
            const int js = gs >> 4, fs = gs & 0xF, jt = gt >> 4, ft = gt & 0xF;
            const int w11 = (fs * ft + 8) >> 4, w10 = ft - w11, w01 = fs - w11, w00 = 16 - fs - ft + w11;
            const int v0 = js + jt * 4;
            int acc = wv[v0] * w00;
            if (w01) acc += wv[v0 + 1] * w01;
            if (w10) acc += wv[v0 + 4] * w10;
            if (w11) acc += wv[v0 + 5] * w11;
            const int wt = (acc + 8) >> 4;
            uint32_t px = 0;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int c0 = srgb ? ((e0[c] << 8) | 0x80) : e0[c] * 257;
                const int c1 = srgb ? ((e1[c] << 8) | 0x80) : e1[c] * 257;
                px |= (uint32_t)(((c0 * (64 - wt) + c1 * wt + 32) >> 6) >> 8) << (8 * c);
            }
            row[s] = px;
            if (s == DIM - 1) sink.row(t, row);
        }
}

// Decode one block into `texel(s, t, rgba)`; returns false for an error block.
template <class Sink>
__device__ bool decode_one(const DecodeTables& T, const uint4 raw, int bw, int bh, bool srgb,
                           Sink&& sink) {
    // the fixed-mode encoder's blocks: mode word, one partition, CEM 8 or 12
    const uint32_t head = raw.x & 0x1FFFFu;
    if (bw == bh && (bw == 4 || bw == 6)) {
        const uint32_t mode11 = head & 0x7FFu, cem = head >> 13;
        const bool q6 = mode11 == blockmode_4x4_grid(kQuant6), q12 = mode11 == blockmode_4x4_grid(kQuant12);
        const bool alpha = cem == 12u;
        // QUANT_12 weights leave 53 bits for the colours: QUANT_256 for six
        // values (CEM 8), a smaller range for eight (CEM 12, the general path)
        if ((head & 0x1800u) == 0 && (cem == 8u || cem == 12u) && (q6 || (q12 && !alpha))) {
            if (bw == 4) {
                if (q6) decode_fixed_grid4<4, kQuant6>(T, raw, alpha, srgb, sink);
                else decode_fixed_grid4<4, kQuant12>(T, raw, alpha, srgb, sink);
            } else {
                if (q6) decode_fixed_grid4<6, kQuant6>(T, raw, alpha, srgb, sink);
                else decode_fixed_grid4<6, kQuant12>(T, raw, alpha, srgb, sink);
            }
            return true;
        }
    }
    Bits b = {{raw.x, raw.y, raw.z, raw.w}};
    const int mode = (int)b.read(0, 11);
    if ((mode & 0x1FF) == 0x1FC) {
        if ((mode >> 9) & 1) return false;
        const uint32_t c[4] = {b.read(64, 16) >> 8, b.read(80, 16) >> 8, b.read(96, 16) >> 8,
                               b.read(112, 16) >> 8};
        const uint32_t px = c[0] | (c[1] << 8) | (c[2] << 16) | (c[3] << 24);
        for (int t = 0; t < bh; ++t)
            for (int s = 0; s < bw; ++s) sink(s, t, px);
        return true;
    }
    const Mode bm = block_mode(mode);
    if (!bm.ok || bm.gw > bw || bm.gh > bh) return false;
    const int pcount = (int)b.read(11, 2) + 1;
    const int nw = bm.gw * bm.gh * (bm.dual ? 2 : 1);
    if (nw > 64) return false;
    const int wbits = ise_bit_count(bm.quant, nw);
    if (wbits < 24 || wbits > 96 || (pcount == 4 && bm.dual)) return false;
    int cems[4] = {0, 0, 0, 0};
    int color_start = 17, extra = 0;
    const int below = 128 - wbits;
    if (pcount == 1) {
        cems[0] = (int)b.read(13, 4);
    } else {
        color_start = 29;
        const int f = (int)b.read(23, 6);
        if ((f & 3) == 0) {
            for (int p = 0; p < pcount; ++p) cems[p] = f >> 2;
        } else {
            extra = 3 * pcount - 4;
            const int comb = (f >> 2) | ((int)b.read(below - extra, extra) << 4);
            const int base = (f & 3) - 1;
            for (int p = 0; p < pcount; ++p)
                cems[p] = ((base + ((comb >> p) & 1)) << 2) | ((comb >> (pcount + 2 * p)) & 3);
        }
    }
    const int color_end = below - extra - (bm.dual ? 2 : 0);
    const int plane2 = bm.dual ? (int)b.read(color_end, 2) : -1;
    int nvals = 0;
    for (int p = 0; p < pcount; ++p) nvals += 2 * ((cems[p] >> 2) + 1);
    const int cbits = color_end - color_start;
    if (nvals > 18 || cbits < 0) return false;
    int cq = -1;
    for (int q = kQuant256; q >= 0; --q)
        if (ise_bit_count(q, nvals) <= cbits) { cq = q; break; }
    if (cq < kQuant6) return false;
    uint8_t cv[18];
    ise_decode(T, cq, nvals, b, color_start, cv);
    int ep[4][2][4];
    for (int p = 0, off = 0; p < pcount; ++p) {
        int v[8];
        const int n = 2 * ((cems[p] >> 2) + 1);
        for (int i = 0; i < n; ++i) v[i] = T.color_unq[cq][cv[off + i]];
        off += n;
        if (!unpack_endpoints(cems[p], v, ep[p][0], ep[p][1])) return false;
    }
    Bits rb = {{rev32(raw.w), rev32(raw.z), rev32(raw.y), rev32(raw.x)}};
    uint8_t wv[64];
    ise_decode(T, bm.quant, nw, rb, 0, wv);
    for (int i = 0; i < nw; ++i) wv[i] = T.weight_unq[bm.quant][wv[i]];
    const int planes = bm.dual ? 2 : 1;
    const int ds = (1024 + bw / 2) / (bw - 1), dt = (1024 + bh / 2) / (bh - 1);
    const bool small = bw * bh < 31;
    const int seed = pcount > 1 ? (int)b.read(13, 10) : 0;
    for (int t = 0; t < bh; ++t)
        for (int s = 0; s < bw; ++s) {
            const int gs = (ds * s * (bm.gw - 1) + 32) >> 6;
            const int gt = (dt * t * (bm.gh - 1) + 32) >> 6;
            const int js = gs >> 4, fs = gs & 0xF, jt = gt >> 4, ft = gt & 0xF;
            const int w11 = (fs * ft + 8) >> 4, w10 = ft - w11, w01 = fs - w11;
            const int w00 = 16 - fs - ft + w11;
            const int v0 = js + jt * bm.gw, ng = bm.gw * bm.gh;
            int w[2] = {0, 0};
            for (int pl = 0; pl < planes; ++pl) {
                int acc = (v0 < ng ? wv[v0 * planes + pl] : 0) * w00;
                if (w01) acc += (v0 + 1 < ng ? wv[(v0 + 1) * planes + pl] : 0) * w01;
                if (w10) acc += (v0 + bm.gw < ng ? wv[(v0 + bm.gw) * planes + pl] : 0) * w10;
                if (w11) acc += (v0 + bm.gw + 1 < ng ? wv[(v0 + bm.gw + 1) * planes + pl] : 0) * w11;
                w[pl] = (acc + 8) >> 4;
            }
            const int part = pcount > 1 ? select_partition(seed, s, t, pcount, small) : 0;
            uint32_t px = 0;
            for (int c = 0; c < 4; ++c) {
                const int wt = c == plane2 ? w[1] : w[0];
                const int c0 = srgb ? ((ep[part][0][c] << 8) | 0x80) : ep[part][0][c] * 257;
                const int c1 = srgb ? ((ep[part][1][c] << 8) | 0x80) : ep[part][1][c] * 257;
                px |= (uint32_t)(((c0 * (64 - wt) + c1 * wt + 32) >> 6) >> 8) << (8 * c);
            }
            sink(s, t, px);
        }
    return true;
}

// Writes decoded texels into the RGBA8 image: one at a time, or a block's
// whole row (N texels) in 16-byte (N = 4) or 8-byte (N = 6) stores when the
// block lies inside the image's width and the row's address allows it.
struct TexelSink {
    uint32_t* out;
    int width, height, x0, y0;
    bool full_width;
    __device__ __forceinline__ void operator()(int s, int t, uint32_t px) const {
        const int x = x0 + s, y = y0 + t;
        if (x < width && y < height) out[(size_t)y * width + x] = px;
    }
    template <int N>
    __device__ __forceinline__ void row(int t, const uint32_t (&px)[N]) const {
        const int y = y0 + t;
        if (y >= height) return;
        uint32_t* dst = out + (size_t)y * width + x0;
        const uintptr_t a = reinterpret_cast<uintptr_t>(dst);
        if (full_width && N == 4 && a % 16 == 0) {
            *reinterpret_cast<uint4*>(dst) = make_uint4(px[0], px[1], px[2], px[3 % N]);
        } else if (full_width && N % 2 == 0 && a % 8 == 0) {
#pragma unroll
            for (int k = 0; k < N; k += 2) *reinterpret_cast<uint2*>(dst + k) = make_uint2(px[k], px[k + 1]);
        } else {
#pragma unroll
            for (int s = 0; s < N; ++s) (*this)(s, t, px[s]);
        }
    }
};

__global__ void __launch_bounds__(kDecodeThreads)
astc_decode_ldr(const uint4* __restrict__ blocks, int width, int height, int bw, int bh, int nbx,
                long long nblocks, int srgb, uint32_t* __restrict__ out) {
    __shared__ DecodeTables s_tab;
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&c_dec);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&s_tab);
        for (int i = threadIdx.x; i < (int)(sizeof(DecodeTables) / 4); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    pdl_wait_prior();
    pdl_allow_next();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nblocks) return;
    const int by = (int)(i / nbx), bx = (int)(i - (long long)by * nbx);
    const int x0 = bx * bw, y0 = by * bh;
    TexelSink sink{out, width, height, x0, y0, x0 + bw <= width};
    if (!decode_one(s_tab, blocks[i], bw, bh, srgb != 0, sink)) {
        for (int t = 0; t < bh; ++t)
            for (int s = 0; s < bw; ++s) sink(s, t, 0xFFFF00FFu);    // magenta
    }
}

// Per-channel sum of squared differences; one 64-bit atomic per warp.
__global__ void __launch_bounds__(256)
astc_sse_rgba(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, size_t n,
              unsigned long long* __restrict__ sse) {
    SseAcc acc;
    sse_range(a, b, 0, n, (size_t)blockIdx.x * blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x, acc);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        unsigned long long v = acc.hi[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(sse + c, v);
    }
}

// Squared error of two normal maps in the -norm layout, on the reconstructed
// unit normals: x, y = code * 2/255 - 1 from R and G, z = sqrt(max(0, 1 - x^2
// - y^2)); each component's difference is scaled by 127.5 (the [-1, 1] range
// mapped onto 0..255) so PSNR takes the usual 8-bit peak.  FP64 accumulation.
__device__ __forceinline__ void normal_of(uint32_t px, float n[3]) {
    n[0] = (float)(px & 0xFF) * (2.0f / 255.0f) - 1.0f;
    n[1] = (float)((px >> 8) & 0xFF) * (2.0f / 255.0f) - 1.0f;
    n[2] = sqrtf(fmaxf(0.0f, 1.0f - n[0] * n[0] - n[1] * n[1]));
}

__global__ void __launch_bounds__(256)
astc_normal_sse(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, size_t n,
                double* __restrict__ sse) {
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float p[3], q[3];
        normal_of(__ldg(a + i), p);
        normal_of(__ldg(b + i), q);
        float t = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float d = (p[c] - q[c]) * 127.5f;
            t += d * d;
        }
        acc += (double)t;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(sse, acc);
}

}  // namespace

cudaError_t launch_normal_sse(const uint8_t* a, const uint8_t* b, size_t texels, double* d_sse,
                              cudaStream_t stream) {
    if (texels == 0) return cudaSuccess;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = ((long long)texels + 255) / 256;
    const long long cap = (long long)sms * 8;
    if (grid > cap) grid = cap;
    astc_normal_sse<<<(unsigned)grid, 256, 0, stream>>>(reinterpret_cast<const uint32_t*>(a),
                                                        reinterpret_cast<const uint32_t*>(b), texels, d_sse);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

cudaError_t launch_decode(const uint8_t* blocks, int width, int height, int bw, int bh, int srgb,
                          uint8_t* out, cudaStream_t stream) {
    const int nbx = (width + bw - 1) / bw;
    const long long nb = (long long)nbx * ((height + bh - 1) / bh);
    const long long grid = (nb + kDecodeThreads - 1) / kDecodeThreads;
    const cudaError_t e = launch_pdl(astc_decode_ldr, (unsigned)grid, kDecodeThreads, 0, stream,
                                     reinterpret_cast<const uint4*>(blocks), width, height, bw, bh, nbx, nb, srgb,
                                     reinterpret_cast<uint32_t*>(out));
    if (e == cudaSuccess) count_launches(1);
    return e;
}

cudaError_t launch_sse(const uint8_t* a, const uint8_t* b, size_t texels, unsigned long long* d_sse,
                       cudaStream_t stream) {
    if (texels == 0) return cudaSuccess;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = ((long long)texels + 2047) / 2048;      // at least 8 texels per thread
    const long long cap = (long long)sms * 8;
    if (grid > cap) grid = cap;
    astc_sse_rgba<<<(unsigned)grid, 256, 0, stream>>>(reinterpret_cast<const uint32_t*>(a),
                                                      reinterpret_cast<const uint32_t*>(b), texels, d_sse);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

}  // namespace astc
