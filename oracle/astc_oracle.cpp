/*
 * astc_oracle.cpp -- CPU oracle for the ASTC block encoder.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA encoder is compared with.
 * The product library never links or loads this file.
 *
 * What it restates (niepp/astc_encoder, file:line):
 *   texel fetch            ASTC_Encode.hlsl:561-580  (OOB Load = 0, normal map
 *                                                      b=a=1, then x255)
 *   encode_block           ASTC_Encode.hlsl:510-550
 *   PCA / mean / cov       ASTC_Encode.hlsl:139-168
 *   eigen_vector           ASTC_Encode.hlsl:93-106
 *   find_min_max           ASTC_Encode.hlsl:108-137
 *   encode_color           ASTC_Encode.hlsl:233-245, endpoint_ise 475-489
 *   weights                ASTC_Encode.hlsl:256-260, 268-314, 316-393, 491-508
 *   assemble_blockmode     ASTC_Encode.hlsl:446-473
 *   assemble_block         ASTC_Encode.hlsl:400-444
 *   ISE                    ASTC_IntegerSequenceEncoding.hlsl:5-276
 *   scramble tables        ASTC_Table.hlsl:4-66
 *   max_accumulation_pixel_direction  ASTC_Encode.hlsl:170-227 (the shader's
 *                          unused alternative to the PCA, opts.axis = 1)
 *   search mode            the choose_best_quantmethod the shader sketches at
 *                          ASTC_Encode.hlsl:524-526 (opts.quality = 1): every
 *                          4x4-grid weight range with the endpoint range the
 *                          decoder derives, scored by the spec decode;
 *                          quality 2 adds the other fit and dual-plane
 *                          blocks, quality 3 two-partition blocks (modes
 *                          the shader leaves out: its dual-plane bit is 0,
 *                          ASTC_Encode.hlsl:446-473; its partition layout a
 *                          commented-out stub, 422-431)
 *
 * The lookup tables are GENERATED here from the ASTC specification's
 * definitions (trit/quint decode, weight unquantisation), never copied; the
 * test suite compares them element-wise with the reference's arrays.
 *
 * FP32 arithmetic model (the shader's HLSL semantics, pinned once):
 *   - round()        = round half to even (rintf), HLSL round / DXBC round_ne
 *   - a*b+c (mad)    = ORACLE_FUSED_MAD ? fmaf(a,b,c) : (a*b)+c
 *   - dot(a,b)       = a.x*b.x, then mad over y, z, w in that order
 *   - length(v)      = sqrt(dot(v,v))        (correctly rounded sqrt)
 *   - normalize(v)   = v * (1 / sqrt(dot(v,v)))
 *   - x / N (const)  = ORACLE_CONST_DIV_AS_MUL ? x * (1/N) : x / N
 *   - 1.0f / x       = correctly rounded division
 *   - min/max/clamp  = fminf/fmaxf (no NaN can reach them)
 *   - UNORM8 fetch   = c / 255 * 255 (exact: equals c for all 256 codes)
 *   - sRGB fetch     = float(srgb_to_linear_f64(c / 255)) * 255
 * Build with -ffp-contract=off so the compiler fuses nothing on its own.
 * The default model was chosen by the identical-block count against the
 * reference's own output textures/leaf.astc (see the golden tests).
 */
#include "astc_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_FUSED_MAD
#define ORACLE_FUSED_MAD 1
#endif
#ifndef ORACLE_CONST_DIV_AS_MUL
#define ORACLE_CONST_DIV_AS_MUL 1
#endif

namespace {

// ---------------------------------------------------------------------------
// quant methods (ASTC_Encode.hlsl:47-68)
// ---------------------------------------------------------------------------
enum {
    QUANT_2 = 0, QUANT_3, QUANT_4, QUANT_5, QUANT_6, QUANT_8, QUANT_10, QUANT_12,
    QUANT_16, QUANT_20, QUANT_24, QUANT_32, QUANT_40, QUANT_48, QUANT_64, QUANT_80,
    QUANT_96, QUANT_128, QUANT_160, QUANT_192, QUANT_256, QUANT_MAX
};
const int kQuantLevels[QUANT_MAX] = {2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32,
                                     40, 48, 64, 80, 96, 128, 160, 192, 256};

// ---------------------------------------------------------------------------
// Tables generated from the specification
// ---------------------------------------------------------------------------
struct Tables {
    int btq[QUANT_MAX][3];       // bits, trits, quints per range
    int trits_enc[243];          // 5 trits -> 8-bit T
    int trits_dec[256][5];       // 8-bit T -> 5 trits
    int quints_enc[125];         // 3 quints -> 7-bit Q
    int quints_dec[128][3];      // 7-bit Q -> 3 quints
    int scramble[12][32];        // linear weight index -> ISE symbol
    int unscramble[12][32];      // ISE symbol -> linear weight index
    int wunq[12][32];            // ISE symbol -> weight 0..64
    int cunq[QUANT_MAX][256];    // ISE symbol -> colour 0..255
    float srgb_lut[256];         // float(srgb->linear) (not yet x255)
    double srgb_lut64[256];
    Tables();
};

inline int bit(int x, int i) { return (x >> i) & 1; }

// Spec trit block decode: 8 bits T -> t0..t4.
void decode_trit_block(int T, int t[5]) {
    int C;
    if (((T >> 2) & 7) == 7) {
        C = (((T >> 5) & 7) << 2) | (T & 3);
        t[4] = 2; t[3] = 2;
    } else {
        C = T & 31;
        if (((T >> 5) & 3) == 3) { t[4] = 2; t[3] = bit(T, 7); }
        else { t[4] = bit(T, 7); t[3] = (T >> 5) & 3; }
    }
    if ((C & 3) == 3) {
        t[2] = 2; t[1] = bit(C, 4);
        t[0] = (bit(C, 3) << 1) | (bit(C, 2) & ~bit(C, 3) & 1);
    } else if (((C >> 2) & 3) == 3) {
        t[2] = 2; t[1] = 2; t[0] = C & 3;
    } else {
        t[2] = bit(C, 4); t[1] = (C >> 2) & 3;
        t[0] = (bit(C, 1) << 1) | (bit(C, 0) & ~bit(C, 1) & 1);
    }
}

// Spec quint block decode: 7 bits Q -> q0..q2.
void decode_quint_block(int Q, int q[3]) {
    if (((Q >> 1) & 3) == 3 && ((Q >> 5) & 3) == 0) {
        q[2] = (bit(Q, 0) << 2) | ((bit(Q, 4) & ~bit(Q, 0) & 1) << 1) |
               (bit(Q, 3) & ~bit(Q, 0) & 1);
        q[1] = 4; q[0] = 4;
        return;
    }
    int C;
    if (((Q >> 1) & 3) == 3) {
        q[2] = 4;
        C = (((Q >> 3) & 3) << 3) | (((~Q >> 5) & 3) << 1) | bit(Q, 0);
    } else {
        q[2] = (Q >> 5) & 3;
        C = Q & 31;
    }
    if ((C & 7) == 5) { q[1] = 4; q[0] = (C >> 3) & 3; }
    else { q[1] = (C >> 3) & 3; q[0] = C & 7; }
}

// Spec weight unquantisation of ISE symbol v (0..levels-1) -> 0..64.
int spec_unquant_weight(int quant, int v) {
    const int levels = kQuantLevels[quant];
    (void)levels;
    int bits = 0, trits = 0, quints = 0;
    int l = kQuantLevels[quant];
    while ((l & 1) == 0) { l >>= 1; ++bits; }
    if (l == 3) trits = 1; else if (l == 5) quints = 1;
    int r;
    if (!trits && !quints) {
        // bit replication to 6 bits
        r = 0; int have = 0;
        while (have < 6) { r = (r << bits) | v; have += bits; }
        r >>= (have - 6);
    } else if (bits == 0) {
        int D = v;
        r = trits ? (D == 0 ? 0 : D == 1 ? 32 : 63)
                  : (D == 0 ? 0 : D == 1 ? 16 : D == 2 ? 32 : D == 3 ? 47 : 63);
    } else {
        const int D = v >> bits;
        const int m = v & ((1 << bits) - 1);
        const int A = (m & 1) ? 0x7F : 0;
        const int b1 = bit(m, 1), b2 = bit(m, 2);
        int B = 0, C = 0;
        if (trits) {
            if (bits == 1) { C = 50; B = 0; }
            else if (bits == 2) { C = 23; B = (b1 << 6) | (b1 << 2) | b1; }
            else { C = 11; B = (b2 << 6) | (b1 << 5) | (b2 << 1) | b1; }   // bits == 3
        } else {
            if (bits == 1) { C = 28; B = 0; }
            else { C = 13; B = (b1 << 6) | (b1 << 1) | b1; }                 // bits == 2
        }
        int T = D * C + B;
        T ^= A;
        r = (A & 0x20) | (T >> 2);
    }
    if (r > 32) r += 1;
    return r;
}

// Spec colour unquantisation of ISE symbol v -> 0..255.
int spec_unquant_color(int quant, int v) {
    int bits = 0, trits = 0, quints = 0;
    int l = kQuantLevels[quant];
    while ((l & 1) == 0) { l >>= 1; ++bits; }
    if (l == 3) trits = 1; else if (l == 5) quints = 1;
    if (!trits && !quints) {
        int r = 0, have = 0;
        while (have < 8) { r = (r << bits) | v; have += bits; }
        return r >> (have - 8);
    }
    const int D = v >> bits;
    const int m = v & ((1 << bits) - 1);
    const int A = (m & 1) ? 0x1FF : 0;
    const int b = bit(m, 1), c = bit(m, 2), d = bit(m, 3), e = bit(m, 4), f = bit(m, 5);
    int B = 0, C = 0;
    if (trits) {
        switch (bits) {
        case 1: C = 204; B = 0; break;
        case 2: C = 93;  B = (b << 8) | (b << 4) | (b << 2) | (b << 1); break;
        case 3: C = 44;  B = (c << 8) | (b << 7) | (c << 3) | (b << 2) | (c << 1) | b; break;
        case 4: C = 22;  B = (d << 8) | (c << 7) | (b << 6) | (d << 2) | (c << 1) | b; break;
        case 5: C = 11;  B = (e << 8) | (d << 7) | (c << 6) | (b << 5) | (e << 1) | d; break;
        default: C = 5;  B = (f << 8) | (e << 7) | (d << 6) | (c << 5) | (b << 4) | f; break;
        }
    } else {
        switch (bits) {
        case 1: C = 113; B = 0; break;
        case 2: C = 54;  B = (b << 8) | (b << 3) | (b << 2); break;
        case 3: C = 26;  B = (c << 8) | (b << 7) | (c << 2) | (b << 1) | c; break;
        case 4: C = 13;  B = (d << 8) | (c << 7) | (b << 6) | (d << 1) | c; break;
        default: C = 6;  B = (e << 8) | (d << 7) | (c << 6) | (b << 5) | e; break;
        }
    }
    int T = D * C + B;
    T ^= A;
    return (A & 0x80) | (T >> 2);
}

double srgb_to_linear_f64(double x) {
    return x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4);
}

Tables::Tables() {
    for (int q = 0; q < QUANT_MAX; ++q) {
        int l = kQuantLevels[q], b = 0;
        while ((l & 1) == 0) { l >>= 1; ++b; }
        btq[q][0] = b; btq[q][1] = (l == 3); btq[q][2] = (l == 5);
    }
    // Encoding tables: the inverse of the spec decode.  Where several codes
    // decode to the same tuple, the largest code is taken (this is the
    // choice the reference's integer_from_trits / integer_from_quints make).
    for (int T = 0; T < 256; ++T) {
        int t[5];
        decode_trit_block(T, t);
        for (int i = 0; i < 5; ++i) trits_dec[T][i] = t[i];
        trits_enc[t[4] * 81 + t[3] * 27 + t[2] * 9 + t[1] * 3 + t[0]] = T;
    }
    for (int Q = 0; Q < 128; ++Q) {
        int q[3];
        decode_quint_block(Q, q);
        for (int i = 0; i < 3; ++i) quints_dec[Q][i] = q[i];
        quints_enc[q[2] * 25 + q[1] * 5 + q[0]] = Q;
    }
    // Weight scramble: order the ISE symbols of each weight range by their
    // unquantised value; scramble[i] is the symbol of the i-th smallest.
    std::memset(scramble, 0, sizeof(scramble));
    std::memset(unscramble, 0, sizeof(unscramble));
    std::memset(wunq, 0, sizeof(wunq));
    for (int q = 0; q < 12; ++q) {
        const int n = kQuantLevels[q];
        int vals[32], order[32];
        for (int v = 0; v < n; ++v) { vals[v] = spec_unquant_weight(q, v); order[v] = v; wunq[q][v] = vals[v]; }
        for (int i = 1; i < n; ++i)            // insertion sort, stable
            for (int j = i; j > 0 && vals[order[j - 1]] > vals[order[j]]; --j) {
                int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
            }
        for (int i = 0; i < n; ++i) { scramble[q][i] = order[i]; unscramble[q][order[i]] = i; }
    }
    for (int q = 0; q < QUANT_MAX; ++q)
        for (int v = 0; v < 256; ++v)
            cunq[q][v] = v < kQuantLevels[q] ? spec_unquant_color(q, v) : 0;
    for (int c = 0; c < 256; ++c) {
        srgb_lut64[c] = srgb_to_linear_f64(c / 255.0);
        srgb_lut[c] = (float)srgb_lut64[c];
    }
}

const Tables& tables() {
    static const Tables t;
    return t;
}

// ---------------------------------------------------------------------------
// 128-bit little-endian bit writer (ASTC_IntegerSequenceEncoding.hlsl:98-119)
// ---------------------------------------------------------------------------
struct Bits128 {
    uint32_t w[4];
};

// ORs the low `count` bits of `number` at bit offset `pos` (number < 2^count,
// count <= 8), advancing pos -- orbits8_ptr.
inline void or_bits(Bits128& o, uint32_t& pos, uint32_t number, uint32_t count) {
    const uint32_t newpos = pos + count;
    const uint32_t nidx = newpos >> 5, uidx = pos >> 5, bidx = pos & 31;
    if (uidx < 4) o.w[uidx] |= number << bidx;
    if (nidx > uidx && uidx + 1 < 4) o.w[uidx + 1] |= number >> (32 - bidx);
    pos = newpos;
}

inline uint32_t read_bits(const uint8_t* p, int pos, int count) {
    uint32_t v = 0;
    for (int i = 0; i < count; ++i) {
        const int b = pos + i;
        if (b >= 0 && b < 128) v |= (uint32_t)((p[b >> 3] >> (b & 7)) & 1) << i;
    }
    return v;
}

// encode_trits (ISE:142-176): 5 values, b bits each, one packed trit byte.
void encode_trits(uint32_t b, const uint32_t v[5], Bits128& o, uint32_t& pos) {
    const Tables& tb = tables();
    const uint32_t mask = (1u << b) - 1;
    uint32_t t[5], m[5];
    for (int i = 0; i < 5; ++i) { m[i] = v[i] & mask; t[i] = (v[i] >> b) & 0xFF; }
    const uint32_t T = tb.trits_enc[t[4] * 81 + t[3] * 27 + t[2] * 9 + t[1] * 3 + t[0]];
    or_bits(o, pos, m[0], b); or_bits(o, pos, T & 3, 2);
    or_bits(o, pos, m[1], b); or_bits(o, pos, (T >> 2) & 3, 2);
    or_bits(o, pos, m[2], b); or_bits(o, pos, (T >> 4) & 1, 1);
    or_bits(o, pos, m[3], b); or_bits(o, pos, (T >> 5) & 3, 2);
    or_bits(o, pos, m[4], b); or_bits(o, pos, (T >> 7) & 1, 1);
}

// encode_quints (ISE:181-205): 3 values, b bits each, one packed quint.
void encode_quints(uint32_t b, const uint32_t v[3], Bits128& o, uint32_t& pos) {
    const Tables& tb = tables();
    const uint32_t mask = (1u << b) - 1;
    uint32_t q[3], m[3];
    for (int i = 0; i < 3; ++i) { m[i] = v[i] & mask; q[i] = (v[i] >> b) & 0xFF; }
    const uint32_t Q = tb.quints_enc[q[2] * 25 + q[1] * 5 + q[0]];
    or_bits(o, pos, m[0], b); or_bits(o, pos, Q & 7, 3);
    or_bits(o, pos, m[1], b); or_bits(o, pos, (Q >> 3) & 3, 2);
    or_bits(o, pos, m[2], b); or_bits(o, pos, (Q >> 5) & 3, 2);
}

// bise_endpoints / bise_weights (ISE:207-276) for any count: groups of 5
// (trits) or 3 (quints) padded with zeros, or plain b-bit fields.
void ise_encode(int quant, int count, const uint32_t* values, Bits128& o) {
    const Tables& tb = tables();
    const uint32_t b = tb.btq[quant][0];
    uint32_t pos = 0;
    if (tb.btq[quant][1]) {
        for (int g = 0; g < count; g += 5) {
            uint32_t v[5];
            for (int i = 0; i < 5; ++i) v[i] = g + i < count ? values[g + i] : 0;
            encode_trits(b, v, o, pos);
        }
    } else if (tb.btq[quant][2]) {
        for (int g = 0; g < count; g += 3) {
            uint32_t v[3];
            for (int i = 0; i < 3; ++i) v[i] = g + i < count ? values[g + i] : 0;
            encode_quints(b, v, o, pos);
        }
    } else {
        for (int i = 0; i < count; ++i) or_bits(o, pos, values[i], b);
    }
}

// compute_ise_bitcount (ISE:76-93)
int ise_bits(int quant, int count) {
    const Tables& tb = tables();
    const int b = tb.btq[quant][0];
    if (tb.btq[quant][1]) return ((8 + 5 * b) * count + 4) / 5;
    if (tb.btq[quant][2]) return ((7 + 3 * b) * count + 2) / 3;
    return count * b;
}

// Spec ISE decode from a little-endian bit stream starting at bit `pos`.
// Bits at or past the end of the sequence (pos + ise_bits) read as zero: the
// last trit or quint group of a sequence is stored cut to the sequence's
// length, and whatever follows in the block (endpoints, a dual-plane
// selector) is not part of it.
void ise_decode(int quant, int count, const uint8_t* p, int pos, uint32_t* out) {
    const Tables& tb = tables();
    const int b = tb.btq[quant][0];
    const int end = pos + ise_bits(quant, count);
    auto read_bits = [&](const uint8_t* q, int at, int n) -> uint32_t {
        uint32_t v = 0;
        for (int i = 0; i < n; ++i) {
            const int bit = at + i;
            if (bit >= 0 && bit < 128 && bit < end) v |= (uint32_t)((q[bit >> 3] >> (bit & 7)) & 1) << i;
        }
        return v;
    };
    if (tb.btq[quant][1]) {
        for (int g = 0; g < count; g += 5) {
            uint32_t m[5] = {0, 0, 0, 0, 0};
            static const int tbits[5] = {2, 2, 1, 2, 1};
            uint32_t T = 0;
            int tshift = 0;
            for (int i = 0; i < 5; ++i) {
                m[i] = read_bits(p, pos, b); pos += b;
                T |= read_bits(p, pos, tbits[i]) << tshift;
                pos += tbits[i]; tshift += tbits[i];
            }
            for (int i = 0; i < 5 && g + i < count; ++i)
                out[g + i] = ((uint32_t)tb.trits_dec[T][i] << b) | m[i];
        }
    } else if (tb.btq[quant][2]) {
        for (int g = 0; g < count; g += 3) {
            uint32_t m[3] = {0, 0, 0};
            static const int qbits[3] = {3, 2, 2};
            uint32_t Q = 0;
            int qshift = 0;
            for (int i = 0; i < 3; ++i) {
                m[i] = read_bits(p, pos, b); pos += b;
                Q |= read_bits(p, pos, qbits[i]) << qshift;
                pos += qbits[i]; qshift += qbits[i];
            }
            for (int i = 0; i < 3 && g + i < count; ++i)
                out[g + i] = ((uint32_t)tb.quints_dec[Q][i] << b) | m[i];
        }
    } else {
        for (int i = 0; i < count; ++i) { out[i] = read_bits(p, pos, b); pos += b; }
    }
}

inline uint32_t reverse_byte(uint32_t p) {                 // ISE:131-137
    p = ((p & 0xF) << 4) | ((p >> 4) & 0xF);
    p = ((p & 0x33) << 2) | ((p >> 2) & 0x33);
    p = ((p & 0x55) << 1) | ((p >> 1) & 0x55);
    return p;
}

inline uint32_t reverse_word(uint32_t v) {
    return (reverse_byte(v & 0xFF) << 24) | (reverse_byte((v >> 8) & 0xFF) << 16) |
           (reverse_byte((v >> 16) & 0xFF) << 8) | reverse_byte((v >> 24) & 0xFF);
}

// assemble_blockmode (ASTC_Encode.hlsl:446-473), 4x4 weight grid.
uint32_t assemble_blockmode(uint32_t wq) {
    const uint32_t a = (4 - 2) & 3, b = (4 - 4) & 3, d = 0;
    const uint32_t h = wq < 6 ? 0 : 1, r = (wq % 6) + 2;
    uint32_t m = (r >> 1) & 3;
    m |= (r & 1) << 4;
    m |= (a & 3) << 5;
    m |= (b & 3) << 7;
    m |= h << 9;
    m |= d << 10;
    return m;
}

// assemble_block (ASTC_Encode.hlsl:400-444), single partition.
void assemble_block(uint32_t mode, uint32_t cem, const Bits128& ep, const Bits128& wt,
                    uint8_t out[16]) {
    uint32_t blk[4] = {0, 0, 0, 0};
    blk[3] |= reverse_word(wt.w[0]);
    blk[2] |= reverse_word(wt.w[1]);
    blk[1] |= reverse_word(wt.w[2]);
    blk[0] = mode;
    blk[0] |= (cem & 0xF) << 13;
    blk[0] |= (ep.w[0] & 0x7FFF) << 17;
    blk[1] = (ep.w[0] >> 15) & 0x1FFFF;     // '=' as in the shader (line 438)
    blk[1] |= (ep.w[1] & 0x7FFF) << 17;
    blk[2] |= (ep.w[1] >> 15) & 0x1FFFF;
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 4; ++k) out[i * 4 + k] = (uint8_t)(blk[i] >> (8 * k));
}

// Integer half of encode_block: symbolic endpoints + weights -> 16 bytes.
void assemble_symbolic(const uint32_t ep_q[8], const uint32_t qw[16], bool alpha,
                       uint8_t out[16]) {
    const Tables& tb = tables();
    const uint32_t wq = alpha ? QUANT_6 : QUANT_12;
    Bits128 ep = {{0, 0, 0, 0}}, wt = {{0, 0, 0, 0}};
    uint32_t epv[8];
    for (int i = 0; i < 8; ++i) epv[i] = ep_q[i];
    if (!alpha) { epv[6] = 0; epv[7] = 0; }                 // lines 480-483
    ise_encode(QUANT_256, alpha ? 8 : 6, epv, ep);
    uint32_t sw[16];
    for (int i = 0; i < 16; ++i) sw[i] = (uint32_t)tb.scramble[wq][qw[i]];
    ise_encode((int)wq, 16, sw, wt);
    assemble_block(assemble_blockmode(wq), alpha ? 12u : 8u, ep, wt, out);
}

// ---------------------------------------------------------------------------
// Integer helpers of the search mode (ASTC specification rules)
// ---------------------------------------------------------------------------
// Endpoint quant method of a block with a 4x4 weight grid of quant method wq
// and nvals endpoint values: the decoder takes the largest range whose ISE
// fits in the bits between the header (17 bits for one partition, 29 for
// several with one shared CEM) and the weights (and the block is illegal
// below QUANT_6 or outside 24..96 weight bits).
int endpoint_quant(int wq, int nvals, int header_bits = 17, int nweights = 16) {
    if (wq < QUANT_2 || wq > QUANT_32) return -1;
    const int wbits = ise_bits(wq, nweights);
    if (wbits < 24 || wbits > 96) return -1;
    const int avail = 128 - header_bits - wbits;
    for (int q = QUANT_256; q >= QUANT_6; --q)
        if (ise_bits(q, nvals) <= avail) return q;
    return -1;
}

// The ISE symbol of colour range cq whose unquantised value is nearest v
// (ties: the smaller value); *unq receives that value.
int nearest_color(int cq, int v, int* unq) {
    const Tables& tb = tables();
    int best = 0, bu = tb.cunq[cq][0], bd = std::abs(bu - v);
    for (int s = 1; s < kQuantLevels[cq]; ++s) {
        const int u = tb.cunq[cq][s], d = std::abs(u - v);
        if (d < bd || (d == bd && u < bu)) { best = s; bu = u; bd = d; }
    }
    *unq = bu;
    return best;
}

// One UNORM8 channel of the spec LDR decode: endpoints expanded to 16 bits
// (x257, or x256 + 0x80 for sRGB), interpolated at weight w of 64, top byte.
int decode_channel(int e0, int e1, int w, bool srgb) {
    const int c0 = srgb ? ((e0 << 8) | 0x80) : e0 * 257;
    const int c1 = srgb ? ((e1 << 8) | 0x80) : e1 * 257;
    return ((c0 * (64 - w) + c1 * w + 32) >> 6) >> 8;
}

// Spec bilinear infill of a 4x4 weight grid at texel (s, t) of a 6x6 block.
int infill_6x6(const int wv[16], int s, int t) {
    const int ds = (1024 + 3) / 5;
    const int gs = (ds * s * 3 + 32) >> 6, gt = (ds * t * 3 + 32) >> 6;
    const int js = gs >> 4, fs = gs & 15, jt = gt >> 4, ft = gt & 15;
    const int w11 = (fs * ft + 8) >> 4, w10 = ft - w11, w01 = fs - w11, w00 = 16 - fs - ft + w11;
    const int v0 = js + 4 * jt;
    int acc = wv[v0] * w00;
    if (w01) acc += wv[v0 + 1] * w01;
    if (w10) acc += wv[v0 + 4] * w10;
    if (w11) acc += wv[v0 + 5] * w11;
    return (acc + 8) >> 4;
}

// A block with a 4x4 weight grid of any range: the header (mode, partition
// fields, CEM) in bits 0..hbits-1, the endpoint ISE from bit hbits up, the
// weight ISE bit-reversed from bit 127 down (every field ORed, each cut to
// its ISE length).
void assemble_fields(uint32_t head, int hbits, uint32_t wq, uint32_t cq, const uint32_t* ev, int nvals,
                     const uint32_t* sw, uint8_t out[16]) {
    Bits128 ep = {{0, 0, 0, 0}}, wt = {{0, 0, 0, 0}};
    ise_encode((int)cq, nvals, ev, ep);
    ise_encode((int)wq, 16, sw, wt);
    const int ebits = ise_bits((int)cq, nvals), wbits = ise_bits((int)wq, 16);
    std::memset(out, 0, 16);
    auto set = [&](int pos) { out[pos >> 3] = (uint8_t)(out[pos >> 3] | (1u << (pos & 7))); };
    for (int i = 0; i < hbits; ++i)
        if ((head >> i) & 1) set(i);
    for (int i = 0; i < ebits; ++i)
        if ((ep.w[i >> 5] >> (i & 31)) & 1) set(hbits + i);
    for (int i = 0; i < wbits; ++i)
        if ((wt.w[i >> 5] >> (i & 31)) & 1) set(127 - i);
}

// Single partition: mode [10:0], CEM [16:13], endpoints from bit 17.
void assemble_general(uint32_t wq, uint32_t cq, uint32_t cem, const uint32_t* ev, int nvals,
                      const uint32_t* sw, uint8_t out[16]) {
    assemble_fields(assemble_blockmode(wq) | ((cem & 0xF) << 13), 17, wq, cq, ev, nvals, sw, out);
}

// pcount (2 or 3) partitions sharing one CEM: mode [10:0], partition count -
// 1 at [12:11], partition index [22:13], CEM field [28:23] = CEM << 2 (the
// low two bits 00 mean "every partition uses this CEM"), endpoints from bit
// 29, partition 0's first.
void assemble_partitions(uint32_t pcount, uint32_t wq, uint32_t cq, uint32_t cem, uint32_t seed,
                         const uint32_t* ev, int nvals, const uint32_t* sw, uint8_t out[16]) {
    const uint32_t head = assemble_blockmode(wq) | ((pcount - 1) << 11) | ((seed & 0x3FF) << 13) |
                          ((cem & 0xF) << 25);
    assemble_fields(head, 29, wq, cq, ev, nvals, sw, out);
}

// Single partition, dual plane: mode [10:0] with D (bit 10) set, CEM [16:13],
// endpoints from bit 17, the 2-bit plane-2 component selector right below
// the weights, 32 weights (plane 1, plane 2 per grid point) bit-reversed from
// bit 127 down.
void assemble_dual_plane(uint32_t wq, uint32_t cq, uint32_t cem, uint32_t pc, const uint32_t* ev, int nvals,
                         const uint32_t* sw, uint8_t out[16]) {
    Bits128 ep = {{0, 0, 0, 0}}, wt = {{0, 0, 0, 0}};
    ise_encode((int)cq, nvals, ev, ep);
    ise_encode((int)wq, 32, sw, wt);
    const int ebits = ise_bits((int)cq, nvals), wbits = ise_bits((int)wq, 32);
    std::memset(out, 0, 16);
    auto set = [&](int pos) { out[pos >> 3] = (uint8_t)(out[pos >> 3] | (1u << (pos & 7))); };
    const uint32_t head = assemble_blockmode(wq) | (1u << 10) | ((cem & 0xF) << 13);
    for (int i = 0; i < 17; ++i)
        if ((head >> i) & 1) set(i);
    for (int i = 0; i < ebits; ++i)
        if ((ep.w[i >> 5] >> (i & 31)) & 1) set(17 + i);
    const int sel = 128 - wbits - 2;
    if (pc & 1) set(sel);
    if (pc & 2) set(sel + 1);
    for (int i = 0; i < wbits; ++i)
        if ((wt.w[i >> 5] >> (i & 31)) & 1) set(127 - i);
}

// Two-partition patterns (the spec's partition hash, defined with the
// decoder below): bit i = texel i (row-major) lies in partition 1.
const uint64_t* partition_masks(int dim);

// Three-partition pattern classes of a block size: one per distinct way the
// partition index splits the block's texels into three non-empty sets (two
// indices that split alike up to the partitions' order are one class, kept
// as the smaller index), in index order; m1 / m2 = texels in partitions 1 / 2.
struct ThreeClass { int seed; uint64_t m1, m2; };
const std::vector<ThreeClass>& three_partition_classes(int dim);

inline int popcount64(uint64_t v) {
    int c = 0;
    while (v) { v &= v - 1; ++c; }
    return c;
}

// ---------------------------------------------------------------------------
// Arithmetic policies: FP32 (the pinned model), FP64 twin, FP32 op counter
// ---------------------------------------------------------------------------
struct F32 {
    typedef float T;
    static float lit(float f, double) { return f; }
    static float add(float a, float b) { return a + b; }
    static float sub(float a, float b) { return a - b; }
    static float mul(float a, float b) { return a * b; }
    static float mad(float a, float b, float c) {
#if ORACLE_FUSED_MAD
        return std::fmaf(a, b, c);
#else
        return a * b + c;
#endif
    }
    static float div(float a, float b) { return a / b; }
    static float sqrt(float a) { return std::sqrt(a); }
    static float rint(float a) { return std::rint(a); }
    static float min(float a, float b) { return std::fmin(a, b); }
    static float max(float a, float b) { return std::fmax(a, b); }
    static float srgb(int c) { return tables().srgb_lut[c]; }
};

struct F64 {
    typedef double T;
    static double lit(float, double d) { return d; }
    static double add(double a, double b) { return a + b; }
    static double sub(double a, double b) { return a - b; }
    static double mul(double a, double b) { return a * b; }
    static double mad(double a, double b, double c) {
#if ORACLE_FUSED_MAD
        return std::fma(a, b, c);
#else
        return a * b + c;
#endif
    }
    static double div(double a, double b) { return a / b; }
    static double sqrt(double a) { return std::sqrt(a); }
    static double rint(double a) { return std::rint(a); }
    static double min(double a, double b) { return std::fmin(a, b); }
    static double max(double a, double b) { return std::fmax(a, b); }
    static double srgb(int c) { return tables().srgb_lut64[c]; }
};

thread_local double g_flops = 0.0;
struct F32Count : F32 {
    static float add(float a, float b) { g_flops += 1; return F32::add(a, b); }
    static float sub(float a, float b) { g_flops += 1; return F32::sub(a, b); }
    static float mul(float a, float b) { g_flops += 1; return F32::mul(a, b); }
    static float mad(float a, float b, float c) { g_flops += 2; return F32::mad(a, b, c); }
    static float div(float a, float b) { g_flops += 1; return F32::div(a, b); }
    static float sqrt(float a) { g_flops += 1; return F32::sqrt(a); }
};

// ---------------------------------------------------------------------------
// The FP pipeline (templated on the arithmetic policy)
// ---------------------------------------------------------------------------
// Optional record of the fixed-mode pipeline's intermediate values (FP32 runs
// only; filled when a non-null pointer is passed).
typedef oracle_trace Trace;

template <class T>
inline void trace_put(float* dst, const T* src, int n) {
    for (int i = 0; i < n; ++i) dst[i] = (float)src[i];
}

template <class P>
struct Pipe {
    typedef typename P::T T;

    static T dot4(const T a[4], const T b[4]) {
        T d = P::mul(a[0], b[0]);
        d = P::mad(a[1], b[1], d);
        d = P::mad(a[2], b[2], d);
        d = P::mad(a[3], b[3], d);
        return d;
    }
    static T length(const T v[4]) { return P::sqrt(dot4(v, v)); }
    static void normalize(T v[4]) {
        const T r = P::div(P::lit(1.0f, 1.0), P::sqrt(dot4(v, v)));
        for (int i = 0; i < 4; ++i) v[i] = P::mul(v[i], r);
    }
    static T div_const(T x, int n) {
#if ORACLE_CONST_DIV_AS_MUL
        return P::mul(x, P::div(P::lit(1.0f, 1.0), (T)n));
#else
        return P::div(x, (T)n);
#endif
    }

    // eigen_vector (ASTC_Encode.hlsl:93-106)
    static void eigen_vector(const T m[4][4], T v[4], Trace* tr = nullptr) {
        v[0] = P::lit(0.26726f, 0.26726); v[1] = P::lit(0.80178f, 0.80178);
        v[2] = P::lit(0.53452f, 0.53452); v[3] = 0;
        if (tr) v[3] = (T)tr->start_w;      // a trace may seed the start vector's alpha
        if (tr) { tr->early_exit = 0; tr->min_len = 1e31f; }
        for (int it = 0; it < 8; ++it) {
            T t[4];
            for (int r = 0; r < 4; ++r) t[r] = dot4(m[r], v);
            for (int r = 0; r < 4; ++r) v[r] = t[r];
            const T len = length(v);
            if (tr && (float)len < tr->min_len) tr->min_len = (float)len;
            if (len < P::lit(1e-5f, 1e-5)) {
                if (tr) tr->early_exit = 1 + it;
                return;
            }
            for (int r = 0; r < 4; ++r) t[r] = dot4(m[r], v);
            for (int r = 0; r < 4; ++r) v[r] = t[r];
            normalize(v);
        }
    }

    // find_min_max (ASTC_Encode.hlsl:108-137), over the texels in `sel`
    static void find_min_max(const T (*tex)[4], int n, const T mean[4], const T k[4],
                             bool alpha, T e0[4], T e1[4], uint64_t sel = ~0ull,
                             Trace* tr = nullptr) {
        T a = P::lit(1e31f, 1e31), b = P::lit(-1e31f, -1e31);
        for (int i = 0; i < n; ++i) {
            if (!((sel >> i) & 1)) continue;
            T d[4];
            for (int c = 0; c < 4; ++c) d[c] = P::sub(tex[i][c], mean[c]);
            const T t = dot4(d, k);
            a = P::min(a, t);
            b = P::max(b, t);
        }
        for (int c = 0; c < 4; ++c) {
            e0[c] = P::min(P::max(P::mad(k[c], a, mean[c]), (T)0), P::lit(255.0f, 255.0));
            e1[c] = P::min(P::max(P::mad(k[c], b, mean[c]), (T)0), P::lit(255.0f, 255.0));
        }
        const T s0 = P::add(P::add(P::rint(e0[0]), P::rint(e0[1])), P::rint(e0[2]));
        const T s1 = P::add(P::add(P::rint(e1[0]), P::rint(e1[1])), P::rint(e1[2]));
        if (tr) {
            tr->tmin = (float)a; tr->tmax = (float)b;
            trace_put(tr->e0_fit, e0, 4); trace_put(tr->e1_fit, e1, 4);
            tr->s0 = (float)s0; tr->s1 = (float)s1; tr->swapped = s0 > s1;
        }
        if (s0 > s1)
            for (int c = 0; c < 4; ++c) { T t = e0[c]; e0[c] = e1[c]; e1[c] = t; }
        if (!alpha) { e0[3] = P::lit(255.0f, 255.0); e1[3] = P::lit(255.0f, 255.0); }
    }

    // the mean and covariance of principal_component_analysis
    // (ASTC_Encode.hlsl:139-162)
    static void covariance(const T (*tex)[4], int n, T mean[4], T cov[4][4]) {
        for (int c = 0; c < 4; ++c) mean[c] = 0;
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 4; ++c) mean[c] = P::add(mean[c], tex[i][c]);
        for (int c = 0; c < 4; ++c) mean[c] = div_const(mean[c], n);
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) cov[i][j] = 0;
        for (int k = 0; k < n; ++k) {
            T d[4];
            for (int c = 0; c < 4; ++c) d[c] = P::sub(tex[k][c], mean[c]);
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) cov[i][j] = P::mad(d[i], d[j], cov[i][j]);
        }
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) cov[i][j] = div_const(cov[i][j], n - 1);
    }

    // principal_component_analysis (ASTC_Encode.hlsl:139-168)
    static void pca(const T (*tex)[4], int n, bool alpha, T e0[4], T e1[4], Trace* tr = nullptr) {
        T mean[4], cov[4][4];
        covariance(tex, n, mean, cov);
        T k[4];
        eigen_vector(cov, k, tr);
        if (tr) {
            trace_put(tr->mean, mean, 4);
            for (int i = 0; i < 4; ++i) trace_put(tr->cov + 4 * i, cov[i], 4);
            trace_put(tr->axis, k, 4);
        }
        find_min_max(tex, n, mean, k, alpha, e0, e1, ~0ull, tr);
    }

    // max_accumulation_pixel_direction (ASTC_Encode.hlsl:170-227): the axis is
    // the largest of four sums -- of the deviations of the texels whose red,
    // green, blue (or, with alpha, alpha) lies above the mean.
    static void max_accumulation(const T (*tex)[4], int n, bool alpha, T e0[4], T e1[4]) {
        T mean[4] = {0, 0, 0, 0};
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 4; ++c) mean[c] = P::add(mean[c], tex[i][c]);
        for (int c = 0; c < 4; ++c) mean[c] = div_const(mean[c], n);
        T sum[4][4];
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 4; ++c) sum[a][c] = 0;
        for (int i = 0; i < n; ++i) {
            T d[4];
            for (int c = 0; c < 4; ++c) d[c] = P::sub(tex[i][c], mean[c]);
            for (int a = 0; a < 4; ++a)                   // sum += (dt.a > 0) ? dt : 0
                for (int c = 0; c < 4; ++c) sum[a][c] = P::add(sum[a][c], d[a] > 0 ? d[c] : (T)0);
        }
        T k[4];
        for (int c = 0; c < 4; ++c) k[c] = sum[0][c];
        T maxdot = dot4(sum[0], sum[0]);
        for (int a = 1; a < (alpha ? 4 : 3); ++a) {       // strict >, in r g b a order
            const T d = dot4(sum[a], sum[a]);
            if (d > maxdot) {
                maxdot = d;
                for (int c = 0; c < 4; ++c) k[c] = sum[a][c];
            }
        }
        if (!(length(k) < P::lit(1e-5f, 1e-5))) normalize(k);   // safe normalize
        find_min_max(tex, n, mean, k, alpha, e0, e1);
    }

    static void fit(const T (*tex)[4], int n, bool alpha, int axis, T e0[4], T e1[4]) {
        if (axis == 1) max_accumulation(tex, n, alpha, e0, e1);
        else pca(tex, n, alpha, e0, e1);
    }

    // idx_grids / wt_grids (ASTC_Encode.hlsl:268-304): the 4x4 weight grid of
    // a 6x6 block samples 2x2 texel taps at fixed bilinear weights.
    static void grid_taps(int g, int idx[4], T wt[4]) {
        const int gx = g & 3, gy = g >> 2;
        const int x0 = gx < 2 ? gx : gx + 1;           // texel columns 0,1,3,4
        const int y0 = gy < 2 ? gy : gy + 1;
        idx[0] = y0 * 6 + x0; idx[1] = idx[0] + 1; idx[2] = idx[0] + 6; idx[3] = idx[0] + 7;
        // near tap gets 4/9 along an axis where the grid point sits 1/3 from
        // it; grid columns 0 and 2 lean left, 1 and 3 lean right.
        const bool xl = (gx & 1) == 0, yl = (gy & 1) == 0;
        const T hi = P::lit(0.444f, 0.444), mid = P::lit(0.222f, 0.222), lo = P::lit(0.111f, 0.111);
        // corner order (x0,y0), (x1,y0), (x0,y1), (x1,y1)
        const bool nearx[4] = {xl, !xl, xl, !xl};
        const bool neary[4] = {yl, yl, !yl, !yl};
        for (int c = 0; c < 4; ++c)
            wt[c] = (nearx[c] && neary[c]) ? hi : (nearx[c] || neary[c]) ? mid : lo;
    }

    // the colour at weight-grid point g: the texel itself (4x4) or the 2x2
    // bilinear sample of sample_texel (ASTC_Encode.hlsl:307-314, 6x6)
    static void grid_sample(const T (*tex)[4], int dim, int g, T s[4]) {
        if (dim == 6) {
            int idx[4]; T cw[4];
            grid_taps(g, idx, cw);
            for (int c = 0; c < 4; ++c) {
                T acc = P::mul(tex[idx[0]][c], cw[0]);
                acc = P::mad(tex[idx[1]][c], cw[1], acc);
                acc = P::mad(tex[idx[2]][c], cw[2], acc);
                acc = P::mad(tex[idx[3]][c], cw[3], acc);
                s[c] = acc;
            }
        } else {
            for (int c = 0; c < 4; ++c) s[c] = tex[g][c];
        }
    }

    // calculate_normal_weights + quantize_weights (ASTC_Encode.hlsl:316-393)
    static void weights(const T (*tex)[4], int dim, const T e0[4], const T e1[4],
                        uint32_t range, uint32_t qw[16], Trace* tr = nullptr) {
        T k[4];
        for (int c = 0; c < 4; ++c) k[c] = P::sub(e1[c], e0[c]);
        T w[16];
        if (tr) { tr->wlen = (float)length(k); tr->minw = tr->maxw = tr->inv = 0; }
        if (length(k) < P::lit(1e-5f, 1e-5)) {
            for (int i = 0; i < 16; ++i) w[i] = 0;
        } else {
            normalize(k);
            T minw = P::lit(1e31f, 1e31), maxw = P::lit(-1e31f, -1e31);
            for (int i = 0; i < 16; ++i) {
                T s[4];
                grid_sample(tex, dim, i, s);
                T d[4];
                for (int c = 0; c < 4; ++c) d[c] = P::sub(s[c], e0[c]);
                const T x = dot4(k, d);
                minw = P::min(x, minw);
                maxw = P::max(x, maxw);
                w[i] = x;
            }
            T inv = P::sub(maxw, minw);
            inv = P::max(P::lit(1e-5f, 1e-5), inv);
            inv = P::div(P::lit(1.0f, 1.0), inv);
            if (tr) {
                trace_put(tr->wproj, w, 16);
                tr->minw = (float)minw; tr->maxw = (float)maxw; tr->inv = (float)inv;
            }
            for (int i = 0; i < 16; ++i) w[i] = P::mul(P::sub(w[i], minw), inv);
        }
        const T rf = (T)range;
        for (int i = 0; i < 16; ++i) {
            if (tr) tr->wR[i] = (float)P::mul(w[i], rf);
            const T r = P::rint(P::mul(w[i], rf));
            uint32_t q = r <= 0 ? 0u : (uint32_t)r;
            qw[i] = q > range ? range : q;
        }
    }

    // encode_block (ASTC_Encode.hlsl:510-550) after the endpoint fit
    static void fixed_mode(const T (*tex)[4], int dim, bool alpha, const T e0[4], const T e1[4],
                           uint32_t ep_q[8], uint32_t qw[16], uint8_t out[16]) {
        for (int c = 0; c < 4; ++c) {                       // encode_color 233-245
            ep_q[2 * c] = (uint32_t)P::rint(e0[c]);
            ep_q[2 * c + 1] = (uint32_t)P::rint(e1[c]);
        }
        const uint32_t range = alpha ? 5u : 11u;            // weight_range - 1
        weights(tex, dim, e0, e1, range, qw);
        assemble_symbolic(ep_q, qw, alpha, out);
    }

    // encode_block (ASTC_Encode.hlsl:510-550); axis 1 swaps in the
    // alternative fit the shader leaves commented out at line 515
    static void encode(const T (*tex)[4], int dim, bool alpha, uint32_t ep_q[8],
                       uint32_t qw[16], uint8_t out[16], int axis = 0) {
        T e0[4], e1[4];
        fit(tex, dim * dim, alpha, axis, e0, e1);
        fixed_mode(tex, dim, alpha, e0, e1, ep_q, qw, out);
    }

    // ---- search mode -----------------------------------------------------
    // Squared error of a decoded single-partition block with endpoints E0/E1
    // (0..255) and grid weights wv (0..64) against the texels rounded to
    // bytes in the fit space (tb: UNORM codes as they are, sRGB codes
    // linearised x255 and rounded), channels r g b (a).  Exact integers.
    static uint32_t block_error(const int (*tb)[4], int dim, int nch, bool srgb, const int E0[4],
                                const int E1[4], const int wv[16]) {
        uint32_t err = 0;
        for (int i = 0; i < dim * dim; ++i) {
            const int w = dim == 4 ? wv[i] : infill_6x6(wv, i % 6, i / 6);
            for (int c = 0; c < nch; ++c) {
                const int d = decode_channel(E0[c], E1[c], w, srgb) - tb[i][c];
                err += (uint32_t)(d * d);
            }
        }
        return err;
    }

    // One search candidate: weight range wq, endpoint range cq, endpoints
    // snapped to the nearest representable values (dark one first, so the
    // decoder neither swaps nor blue-contracts), weights projected onto the
    // decoded endpoints and rounded to the range.
    struct Trial {
        int wq, cq;
        int sym0[4], sym1[4], E0[4], E1[4];
        uint32_t q[16];
    };
    static void trial(const T (*s)[4], const T e0[4], const T e1[4], bool alpha, int wq, Trial& tr) {
        const int nch = alpha ? 4 : 3;
        tr.wq = wq;
        tr.cq = endpoint_quant(wq, alpha ? 8 : 6);
        for (int c = 0; c < 4; ++c) { tr.sym0[c] = tr.sym1[c] = 0; tr.E0[c] = tr.E1[c] = 255; }
        for (int c = 0; c < nch; ++c) {
            tr.sym0[c] = nearest_color(tr.cq, (int)P::rint(e0[c]), &tr.E0[c]);
            tr.sym1[c] = nearest_color(tr.cq, (int)P::rint(e1[c]), &tr.E1[c]);
        }
        if (tr.E1[0] + tr.E1[1] + tr.E1[2] < tr.E0[0] + tr.E0[1] + tr.E0[2])
            for (int c = 0; c < 4; ++c) {
                std::swap(tr.sym0[c], tr.sym1[c]);
                std::swap(tr.E0[c], tr.E1[c]);
            }
        T d[4];
        for (int c = 0; c < 4; ++c) d[c] = (T)(tr.E1[c] - tr.E0[c]);
        const T dd = dot4(d, d);
        const uint32_t R = (uint32_t)kQuantLevels[wq] - 1;
        if (dd == 0) {
            for (int g = 0; g < 16; ++g) tr.q[g] = 0;
            return;
        }
        const T r = P::div(P::lit(1.0f, 1.0), dd);
        for (int g = 0; g < 16; ++g) {
            T diff[4];
            for (int c = 0; c < 4; ++c) diff[c] = P::sub(s[g][c], (T)tr.E0[c]);
            T w = P::mul(dot4(diff, d), r);
            w = P::min(P::max(w, (T)0), P::lit(1.0f, 1.0));
            tr.q[g] = (uint32_t)P::rint(P::mul(w, (T)R));
        }
    }

    static void trial_weights(int wq, const uint32_t q[16], int wv[16]) {
        const Tables& tb = tables();
        for (int g = 0; g < 16; ++g) wv[g] = tb.wunq[wq][tb.scramble[wq][q[g]]];
    }

    // The fixed-mode block, then (ranges) every weight range QUANT_3..QUANT_32
    // with its endpoint range; the first candidate with the least error is
    // kept.  axis 2 fits both ways and keeps the fit whose fixed-mode block has
    // the smaller error (the PCA on ties); dual adds dual-plane candidates,
    // partitions 1 / 2 two- / two- and three-partition candidates.
    static void search(const T (*tex)[4], int dim, bool alpha, bool srgb, int axis, uint8_t out[16],
                       int* chosen, uint32_t* best_err, uint32_t* fixed_err, int partitions, bool ranges,
                       bool dual) {
        const int nch = alpha ? 4 : 3;
        int tb[36][4];
        for (int i = 0; i < dim * dim; ++i)
            for (int c = 0; c < 4; ++c) tb[i][c] = (int)P::rint(tex[i][c]);
        T e0[4] = {0, 0, 0, 0}, e1[4] = {0, 0, 0, 0};
        uint32_t ep_q[8] = {}, qw[16] = {}, best = 0;
        const int a_first = axis == 2 ? 0 : axis, a_last = axis == 2 ? 1 : axis;
        for (int a = a_first; a <= a_last; ++a) {
            T f0[4], f1[4];
            uint32_t fe[8], fw[16];
            uint8_t fb[16];
            fit(tex, dim * dim, alpha, a, f0, f1);
            fixed_mode(tex, dim, alpha, f0, f1, fe, fw, fb);
            int E0[4], E1[4], wv[16];
            for (int c = 0; c < 4; ++c) { E0[c] = (int)fe[2 * c]; E1[c] = (int)fe[2 * c + 1]; }
            trial_weights(alpha ? QUANT_6 : QUANT_12, fw, wv);
            const uint32_t err = block_error(tb, dim, nch, srgb, E0, E1, wv);
            if (a == a_first || err < best) {
                best = err;
                for (int c = 0; c < 4; ++c) { e0[c] = f0[c]; e1[c] = f1[c]; }
                std::memcpy(ep_q, fe, sizeof(ep_q));
                std::memcpy(qw, fw, sizeof(qw));
                std::memcpy(out, fb, 16);
            }
        }
        int wv[16];
        *fixed_err = best;
        *chosen = -1;
        if (!ranges) {
            *best_err = best;
            return;
        }
        T s[16][4];
        for (int g = 0; g < 16; ++g) grid_sample(tex, dim, g, s[g]);
        Trial keep = {};
        for (int wq = QUANT_3; wq <= QUANT_32; ++wq) {
            if (endpoint_quant(wq, alpha ? 8 : 6) < 0) continue;
            Trial tr;
            trial(s, e0, e1, alpha, wq, tr);
            trial_weights(wq, tr.q, wv);
            const uint32_t err = block_error(tb, dim, nch, srgb, tr.E0, tr.E1, wv);
            if (err < best) { best = err; *chosen = wq; keep = tr; }
        }
        if (*chosen >= 0) assemble_trial(keep, alpha, out);
        if (dual) {
            // dual-plane blocks (THOROUGH and above)
            uint8_t dblk[16];
            int dch = -1;
            const uint32_t derr = dual_plane(tex, tb, dim, alpha, srgb, dblk, &dch);
            if (derr < best) {
                best = derr;
                *chosen = dch;
                std::memcpy(out, dblk, 16);
            }
        }
        if (partitions >= 1) {
            // two partitions, split along the kept fit's fixed-mode endpoints
            int PE0[4], PE1[4];
            for (int c = 0; c < 4; ++c) { PE0[c] = (int)ep_q[2 * c]; PE1[c] = (int)ep_q[2 * c + 1]; }
            uint8_t pblk[16];
            int pch = -1;
            const uint32_t perr = two_partitions(tex, tb, dim, alpha, srgb, PE0, PE1, pblk, &pch);
            if (perr < best) {
                best = perr;
                *chosen = pch;
                std::memcpy(out, pblk, 16);
            }
        }
        if (partitions >= 2 && best > 0) {
            // three partitions (no candidate can beat an exact block)
            uint8_t tblk[16];
            int tch = -1;
            const uint32_t terr = three_partitions(tex, tb, dim, alpha, srgb, tblk, &tch);
            if (terr < best) {
                best = terr;
                *chosen = tch;
                std::memcpy(out, tblk, 16);
            }
        }
        *best_err = best;
    }

    // ---- two partitions (quality 3) ----------------------------------------
    // The fit of one partition: mean (correctly rounded division by its texel
    // count), covariance / max(count - 1, 1), the shader's power iteration,
    // and find_min_max over the partition's texels.
    static void fit_partition(const T (*tex)[4], int n, uint64_t sel, bool alpha, T e0[4], T e1[4]) {
        const int cnt = popcount64(sel);
        T mean[4] = {0, 0, 0, 0};
        for (int i = 0; i < n; ++i)
            if ((sel >> i) & 1)
                for (int c = 0; c < 4; ++c) mean[c] = P::add(mean[c], tex[i][c]);
        for (int c = 0; c < 4; ++c) mean[c] = P::div(mean[c], (T)cnt);
        T cov[4][4];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) cov[i][j] = 0;
        for (int t = 0; t < n; ++t) {
            if (!((sel >> t) & 1)) continue;
            T d[4];
            for (int c = 0; c < 4; ++c) d[c] = P::sub(tex[t][c], mean[c]);
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) cov[i][j] = P::mad(d[i], d[j], cov[i][j]);
        }
        const T den = (T)(cnt > 1 ? cnt - 1 : 1);
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) cov[i][j] = P::div(cov[i][j], den);
        T k[4];
        eigen_vector(cov, k);
        find_min_max(tex, n, mean, k, alpha, e0, e1, sel);
    }

    // Two-partition candidates from fixed-mode endpoints E0/E1 (rounded): the
    // texels beyond the endpoints' midpoint form the ideal split; the
    // partition index whose pattern (or its complement) differs from it in the
    // fewest texels is taken (the smallest index on ties, one-partition
    // patterns skipped); each partition is fitted on its own; every weight
    // range whose endpoint range (12 or 16 values after the 29-bit header) is
    // legal is scored.  Returns the best error (UINT32_MAX if none) and its
    // block in out.
    static uint32_t two_partitions(const T (*tex)[4], const int (*tb)[4], int dim, bool alpha, bool srgb,
                                   const int E0[4], const int E1[4], uint8_t out[16], int* chosen) {
        const Tables& tbl = tables();
        const int n = dim * dim, nch = alpha ? 4 : 3, nv = alpha ? 8 : 6;
        const uint64_t full = n == 64 ? ~0ull : ((1ull << n) - 1);
        T d[4];
        for (int c = 0; c < 4; ++c) d[c] = (T)(E1[c] - E0[c]);
        const T dd = dot4(d, d);
        if (dd == 0) return UINT32_MAX;
        uint64_t ideal = 0;
        for (int i = 0; i < n; ++i) {
            T diff[4];
            for (int c = 0; c < 4; ++c) diff[c] = P::sub(tex[i][c], (T)E0[c]);
            const T x = dot4(diff, d);
            if (P::add(x, x) > dd) ideal |= 1ull << i;
        }
        if (ideal == 0 || ideal == full) return UINT32_MAX;
        const uint64_t* pm = partition_masks(dim);
        int seed = -1, best_m = n + 1;
        for (int s = 0; s < 1024; ++s) {
            if (pm[s] == 0 || pm[s] == full) continue;
            int m = popcount64(pm[s] ^ ideal);
            if (n - m < m) m = n - m;
            if (m < best_m) { best_m = m; seed = s; }
        }
        const uint64_t sel1 = pm[seed], sel0 = full & ~sel1;
        T pe0[2][4], pe1[2][4];
        fit_partition(tex, n, sel0, alpha, pe0[0], pe1[0]);
        fit_partition(tex, n, sel1, alpha, pe0[1], pe1[1]);
        uint32_t best = UINT32_MAX;
        for (int wq = QUANT_3; wq <= QUANT_32; ++wq) {
            const int cq = endpoint_quant(wq, 2 * nv, 29);
            if (cq < 0) continue;
            // snapped endpoints per partition, darker first
            int sym0[2][4], sym1[2][4], Q0[2][4], Q1[2][4];
            for (int p = 0; p < 2; ++p) {
                for (int c = 0; c < 4; ++c) { sym0[p][c] = sym1[p][c] = 0; Q0[p][c] = Q1[p][c] = 255; }
                for (int c = 0; c < nch; ++c) {
                    sym0[p][c] = nearest_color(cq, (int)P::rint(pe0[p][c]), &Q0[p][c]);
                    sym1[p][c] = nearest_color(cq, (int)P::rint(pe1[p][c]), &Q1[p][c]);
                }
                if (Q1[p][0] + Q1[p][1] + Q1[p][2] < Q0[p][0] + Q0[p][1] + Q0[p][2])
                    for (int c = 0; c < 4; ++c) {
                        std::swap(sym0[p][c], sym1[p][c]);
                        std::swap(Q0[p][c], Q1[p][c]);
                    }
            }
            // per-texel weights on the texel's own partition, clamped to [0, 1]
            T pd[2][4], r[2];
            bool flat[2];
            for (int p = 0; p < 2; ++p) {
                for (int c = 0; c < 4; ++c) pd[p][c] = (T)(Q1[p][c] - Q0[p][c]);
                const T pdd = dot4(pd[p], pd[p]);
                flat[p] = pdd == 0;
                r[p] = flat[p] ? (T)0 : P::div(P::lit(1.0f, 1.0), pdd);
            }
            T wt[36];
            for (int i = 0; i < n; ++i) {
                const int p = (int)((sel1 >> i) & 1);
                if (flat[p]) { wt[i] = 0; continue; }
                T diff[4];
                for (int c = 0; c < 4; ++c) diff[c] = P::sub(tex[i][c], (T)Q0[p][c]);
                const T w = P::mul(dot4(diff, pd[p]), r[p]);
                wt[i] = P::min(P::max(w, (T)0), P::lit(1.0f, 1.0));
            }
            // grid weights: the texel weights (4x4) or their 2x2 bilinear
            // sample with the shader's taps (6x6), rounded to the range
            const uint32_t R = (uint32_t)kQuantLevels[wq] - 1;
            uint32_t q[16];
            for (int g = 0; g < 16; ++g) {
                T w = wt[g];
                if (dim == 6) {
                    int idx[4]; T cw[4];
                    grid_taps(g, idx, cw);
                    w = P::mul(wt[idx[0]], cw[0]);
                    w = P::mad(wt[idx[1]], cw[1], w);
                    w = P::mad(wt[idx[2]], cw[2], w);
                    w = P::mad(wt[idx[3]], cw[3], w);
                }
                const uint32_t v = (uint32_t)P::rint(P::mul(w, (T)R));
                q[g] = v > R ? R : v;
            }
            int wv[16];
            trial_weights(wq, q, wv);
            uint32_t err = 0;
            for (int i = 0; i < n; ++i) {
                const int p = (int)((sel1 >> i) & 1);
                const int w = dim == 4 ? wv[i] : infill_6x6(wv, i % 6, i / 6);
                for (int c = 0; c < nch; ++c) {
                    const int e = decode_channel(Q0[p][c], Q1[p][c], w, srgb) - tb[i][c];
                    err += (uint32_t)(e * e);
                }
            }
            if (err < best) {
                best = err;
                *chosen = 100 + wq;
                uint32_t ev[16], sw[16];
                for (int p = 0; p < 2; ++p)
                    for (int c = 0; c < nv / 2; ++c) {
                        ev[p * nv + 2 * c] = (uint32_t)sym0[p][c];
                        ev[p * nv + 2 * c + 1] = (uint32_t)sym1[p][c];
                    }
                for (int g = 0; g < 16; ++g) sw[g] = (uint32_t)tbl.scramble[wq][q[g]];
                assemble_partitions(2, (uint32_t)wq, (uint32_t)cq, alpha ? 12u : 8u, (uint32_t)seed, ev, 2 * nv,
                                    sw, out);
            }
        }
        return best;
    }

    // ---- three partitions (quality 4) --------------------------------------
    // Integer labels of the texels (rounded bytes, nch channels): k0 = the
    // texel farthest from texel 0, k1 the one farthest from k0, k2 the one
    // farthest from both (first on ties); every texel takes the nearest of
    // the three (lowest on ties).  Returns false if a label is left empty.
    static int byte_dist(const int* a, const int* b, int nch) {
        int d = 0;
        for (int c = 0; c < nch; ++c) d += (a[c] - b[c]) * (a[c] - b[c]);
        return d;
    }
    static bool three_labels(const int (*tb)[4], int n, int nch, uint64_t L[3]) {
        int k0 = 0, k1 = 0, k2 = 0, far = -1;
        for (int i = 0; i < n; ++i) {
            const int d = byte_dist(tb[i], tb[0], nch);
            if (d > far) { far = d; k0 = i; }
        }
        far = -1;
        for (int i = 0; i < n; ++i) {
            const int d = byte_dist(tb[i], tb[k0], nch);
            if (d > far) { far = d; k1 = i; }
        }
        far = -1;
        for (int i = 0; i < n; ++i) {
            const int d0 = byte_dist(tb[i], tb[k0], nch), d1 = byte_dist(tb[i], tb[k1], nch);
            const int d = d0 < d1 ? d0 : d1;
            if (d > far) { far = d; k2 = i; }
        }
        L[0] = L[1] = L[2] = 0;
        for (int i = 0; i < n; ++i) {
            const int a = byte_dist(tb[i], tb[k0], nch), b = byte_dist(tb[i], tb[k1], nch);
            const int c = byte_dist(tb[i], tb[k2], nch);
            L[(a <= b && a <= c) ? 0 : (b <= c ? 1 : 2)] |= 1ull << i;
        }
        return L[0] && L[1] && L[2];
    }

    // Texels of a pattern class that disagree with the labels under the best
    // matching of labels to partitions.
    static int three_mismatch(const uint64_t L[3], const ThreeClass& k, uint64_t full, int n) {
        const uint64_t pm[3] = {full & ~(k.m1 | k.m2), k.m1, k.m2};
        int M[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) M[a][b] = popcount64(L[a] & pm[b]);
        static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
        int most = 0;
        for (const auto& q : perm) {
            const int m = M[0][q[0]] + M[1][q[1]] + M[2][q[2]];
            if (m > most) most = m;
        }
        return n - most;
    }

    // Three-partition candidates (RGB only: a block carries at most 18 colour
    // endpoint integers, three RGBA partitions would need 24): the four
    // pattern classes that best match the labels (fewest mismatches, then
    // smallest index), each partition fitted on its own (fit_partition),
    // every weight range whose endpoint range (18 values after the 29-bit
    // header) is legal scored with each texel decoded on its partition.
    // Returns the best error (UINT32_MAX if none) and its block; *chosen =
    // 300 + 16 * rank + wq.
    static uint32_t three_partitions(const T (*tex)[4], const int (*tb)[4], int dim, bool alpha, bool srgb,
                                     uint8_t out[16], int* chosen) {
        const Tables& tbl = tables();
        const int n = dim * dim, nch = alpha ? 4 : 3, nv = alpha ? 8 : 6;
        const uint64_t full = n == 64 ? ~0ull : ((1ull << n) - 1);
        if (alpha) return UINT32_MAX;
        uint64_t L[3];
        if (!three_labels(tb, n, nch, L)) return UINT32_MAX;
        uint32_t key[4] = {UINT32_MAX, UINT32_MAX, UINT32_MAX, UINT32_MAX};
        const std::vector<ThreeClass>& cls = three_partition_classes(dim);
        for (int c = 0; c < (int)cls.size(); ++c) {
            uint32_t k = (uint32_t)three_mismatch(L, cls[c], full, n) << 16 | (uint32_t)c;
            for (int r = 0; r < 4; ++r)
                if (k < key[r]) std::swap(k, key[r]);
        }
        uint32_t best = UINT32_MAX;
        for (int rank = 0; rank < 4; ++rank) {
            if (key[rank] == UINT32_MAX) break;
            const ThreeClass& pc = cls[key[rank] & 0xFFFF];
            const uint64_t pm[3] = {full & ~(pc.m1 | pc.m2), pc.m1, pc.m2};
            T pe0[3][4], pe1[3][4];
            for (int p = 0; p < 3; ++p) fit_partition(tex, n, pm[p], alpha, pe0[p], pe1[p]);
            for (int wq = QUANT_3; wq <= QUANT_32; ++wq) {
                const int cq = endpoint_quant(wq, 3 * nv, 29);
                if (cq < 0) continue;
                int sym0[3][4], sym1[3][4], Q0[3][4], Q1[3][4];
                for (int p = 0; p < 3; ++p) {
                    for (int c = 0; c < 4; ++c) { sym0[p][c] = sym1[p][c] = 0; Q0[p][c] = Q1[p][c] = 255; }
                    for (int c = 0; c < nch; ++c) {
                        sym0[p][c] = nearest_color(cq, (int)P::rint(pe0[p][c]), &Q0[p][c]);
                        sym1[p][c] = nearest_color(cq, (int)P::rint(pe1[p][c]), &Q1[p][c]);
                    }
                    if (Q1[p][0] + Q1[p][1] + Q1[p][2] < Q0[p][0] + Q0[p][1] + Q0[p][2])
                        for (int c = 0; c < 4; ++c) {
                            std::swap(sym0[p][c], sym1[p][c]);
                            std::swap(Q0[p][c], Q1[p][c]);
                        }
                }
                T pd[3][4], r[3];
                bool flat[3];
                for (int p = 0; p < 3; ++p) {
                    for (int c = 0; c < 4; ++c) pd[p][c] = (T)(Q1[p][c] - Q0[p][c]);
                    const T pdd = dot4(pd[p], pd[p]);
                    flat[p] = pdd == 0;
                    r[p] = flat[p] ? (T)0 : P::div(P::lit(1.0f, 1.0), pdd);
                }
                int part[36];
                for (int i = 0; i < n; ++i) part[i] = ((pc.m1 >> i) & 1) ? 1 : ((pc.m2 >> i) & 1) ? 2 : 0;
                T wt[36];
                for (int i = 0; i < n; ++i) {
                    const int p = part[i];
                    if (flat[p]) { wt[i] = 0; continue; }
                    T diff[4];
                    for (int c = 0; c < 4; ++c) diff[c] = P::sub(tex[i][c], (T)Q0[p][c]);
                    const T w = P::mul(dot4(diff, pd[p]), r[p]);
                    wt[i] = P::min(P::max(w, (T)0), P::lit(1.0f, 1.0));
                }
                const uint32_t R = (uint32_t)kQuantLevels[wq] - 1;
                uint32_t q[16];
                for (int g = 0; g < 16; ++g) {
                    T w = wt[g];
                    if (dim == 6) {
                        int idx[4]; T cw[4];
                        grid_taps(g, idx, cw);
                        w = P::mul(wt[idx[0]], cw[0]);
                        w = P::mad(wt[idx[1]], cw[1], w);
                        w = P::mad(wt[idx[2]], cw[2], w);
                        w = P::mad(wt[idx[3]], cw[3], w);
                    }
                    const uint32_t v = (uint32_t)P::rint(P::mul(w, (T)R));
                    q[g] = v > R ? R : v;
                }
                int wv[16];
                trial_weights(wq, q, wv);
                uint32_t err = 0;
                for (int i = 0; i < n; ++i) {
                    const int p = part[i];
                    const int w = dim == 4 ? wv[i] : infill_6x6(wv, i % 6, i / 6);
                    for (int c = 0; c < nch; ++c) {
                        const int e = decode_channel(Q0[p][c], Q1[p][c], w, srgb) - tb[i][c];
                        err += (uint32_t)(e * e);
                    }
                }
                if (err < best) {
                    best = err;
                    *chosen = 300 + 16 * rank + wq;
                    uint32_t ev[24], sw[16];
                    for (int p = 0; p < 3; ++p)
                        for (int c = 0; c < nv / 2; ++c) {
                            ev[p * nv + 2 * c] = (uint32_t)sym0[p][c];
                            ev[p * nv + 2 * c + 1] = (uint32_t)sym1[p][c];
                        }
                    for (int g = 0; g < 16; ++g) sw[g] = (uint32_t)tbl.scramble[wq][q[g]];
                    assemble_partitions(3, (uint32_t)wq, (uint32_t)cq, alpha ? 12u : 8u, (uint32_t)pc.seed, ev,
                                        3 * nv, sw, out);
                }
            }
        }
        return best;
    }

    // ---- dual plane (qualities 2 and 3) ------------------------------------
    // Plane 2 carries one channel pc.  For each channel that varies over the
    // block, the shader's power iteration runs on the block's covariance with
    // that channel's row and column zeroed (the PCA of the block with the
    // channel held constant); pc is the channel whose zeroed covariance keeps
    // the least off-axis variance (its trace minus the Rayleigh quotient
    // k.Ck / k.k; the first channel on ties) -- or, when fewer than three
    // channels vary (a normal map's x and y), the first varying channel.  The other channels are fitted
    // on pc's axis by the shader's find_min_max, pc's endpoints are its min
    // and max.  Every weight range QUANT_2.. whose 32 weights (24..96 bits)
    // leave a
    // legal endpoint range after the plane selector is scored.  Plane-1
    // weights project the grid colours on the decoded endpoints without pc,
    // plane-2 weights are (c_pc - E0_pc) / (E1_pc - E0_pc), both clamped to
    // [0, 1] and rounded to the range.  Returns the best error (UINT32_MAX if
    // none) and its block in out; *chosen = 200 + 16 * pc + wq.
    static uint32_t dual_plane(const T (*tex)[4], const int (*tb)[4], int dim, bool alpha, bool srgb,
                               uint8_t out[16], int* chosen) {
        const Tables& tbl = tables();
        const int n = dim * dim, nch = alpha ? 4 : 3, nv = alpha ? 8 : 6;
        uint32_t best = UINT32_MAX;
        T mean[4], cov[4][4];
        covariance(tex, n, mean, cov);
        // each channel's range; constant channels have nothing to split off
        T clo[4], chi[4];
        int nvary = 0, first = -1;
        for (int c = 0; c < nch; ++c) {
            clo[c] = P::lit(1e31f, 1e31);
            chi[c] = P::lit(-1e31f, -1e31);
            for (int i = 0; i < n; ++i) {
                clo[c] = P::min(clo[c], tex[i][c]);
                chi[c] = P::max(chi[c], tex[i][c]);
            }
            if (clo[c] != chi[c]) {
                ++nvary;
                if (first < 0) first = c;
            }
        }
        // the other channels' axis for channel c: the power iteration on the
        // covariance without c's row and column (c's component of the axis is
        // then exactly 0, so c takes no part in the projections)
        auto axis_without = [&](int c, T kc[4], T cp[4][4]) {
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) cp[i][j] = (i == c || j == c) ? (T)0 : cov[i][j];
            eigen_vector(cp, kc);
        };
        int pc = -1;
        T k[4] = {0, 0, 0, 0};
        if (nvary > 0 && nvary < 3) {
            // two varying channels (or one): each plane carries one, so plane 2
            // takes the first
            T cp[4][4];
            pc = first;
            axis_without(pc, k, cp);
        } else if (nvary >= 3) {
            T least = 0;
            for (int c = 0; c < nch; ++c) {
                if (clo[c] == chi[c]) continue;
                T kc[4], cp[4][4];
                axis_without(c, kc, cp);
                T ck[4];
                for (int r = 0; r < 4; ++r) ck[r] = dot4(cp[r], kc);
                const T kk = dot4(kc, kc);
                const T lam = kk > 0 ? P::div(dot4(kc, ck), kk) : (T)0;
                T tr = 0;
                for (int r = 0; r < 4; ++r) tr = P::add(tr, cp[r][r]);
                const T resid = P::sub(tr, lam);
                if (pc < 0 || resid < least) {
                    pc = c; least = resid;
                    for (int r = 0; r < 4; ++r) k[r] = kc[r];
                }
            }
        }
        const T lo = pc >= 0 ? clo[pc] : (T)0, hi = pc >= 0 ? chi[pc] : (T)0;
        if (pc >= 0) {
            T e0[4], e1[4];
            find_min_max(tex, n, mean, k, alpha, e0, e1);
            e0[pc] = lo;
            e1[pc] = hi;
            T s[16][4];
            for (int g = 0; g < 16; ++g) grid_sample(tex, dim, g, s[g]);
            for (int wq = QUANT_2; wq <= QUANT_32; ++wq) {
                const int cq = endpoint_quant(wq, nv, 19, 32);
                if (cq < 0) continue;
                int sym0[4], sym1[4], Q0[4], Q1[4];
                for (int c = 0; c < 4; ++c) { sym0[c] = sym1[c] = 0; Q0[c] = Q1[c] = 255; }
                for (int c = 0; c < nch; ++c) {
                    sym0[c] = nearest_color(cq, (int)P::rint(e0[c]), &Q0[c]);
                    sym1[c] = nearest_color(cq, (int)P::rint(e1[c]), &Q1[c]);
                }
                if (Q1[0] + Q1[1] + Q1[2] < Q0[0] + Q0[1] + Q0[2])
                    for (int c = 0; c < 4; ++c) {
                        std::swap(sym0[c], sym1[c]);
                        std::swap(Q0[c], Q1[c]);
                    }
                T d[4];
                for (int c = 0; c < 4; ++c) d[c] = c == pc ? (T)0 : (T)(Q1[c] - Q0[c]);
                const T dd = dot4(d, d);
                const T r = dd == 0 ? (T)0 : P::div(P::lit(1.0f, 1.0), dd);
                const T dp = (T)(Q1[pc] - Q0[pc]);
                const T rp = dp == 0 ? (T)0 : P::div(P::lit(1.0f, 1.0), dp);
                const uint32_t R = (uint32_t)kQuantLevels[wq] - 1;
                uint32_t q1[16], q2[16];
                for (int g = 0; g < 16; ++g) {
                    T diff[4];
                    for (int c = 0; c < 4; ++c) diff[c] = P::sub(s[g][c], (T)Q0[c]);
                    T w1 = P::mul(dot4(diff, d), r);
                    w1 = P::min(P::max(w1, (T)0), P::lit(1.0f, 1.0));
                    T w2 = P::mul(diff[pc], rp);
                    w2 = P::min(P::max(w2, (T)0), P::lit(1.0f, 1.0));
                    q1[g] = (uint32_t)P::rint(P::mul(w1, (T)R));
                    q2[g] = (uint32_t)P::rint(P::mul(w2, (T)R));
                }
                int wv1[16], wv2[16];
                trial_weights(wq, q1, wv1);
                trial_weights(wq, q2, wv2);
                uint32_t err = 0;
                for (int i = 0; i < n; ++i) {
                    const int w1 = dim == 4 ? wv1[i] : infill_6x6(wv1, i % 6, i / 6);
                    const int w2 = dim == 4 ? wv2[i] : infill_6x6(wv2, i % 6, i / 6);
                    for (int c = 0; c < nch; ++c) {
                        const int e = decode_channel(Q0[c], Q1[c], c == pc ? w2 : w1, srgb) - tb[i][c];
                        err += (uint32_t)(e * e);
                    }
                }
                if (err < best) {
                    best = err;
                    *chosen = 200 + 16 * pc + wq;
                    uint32_t ev[8], sw[32];
                    for (int c = 0; c < nv / 2; ++c) { ev[2 * c] = (uint32_t)sym0[c]; ev[2 * c + 1] = (uint32_t)sym1[c]; }
                    for (int g = 0; g < 16; ++g) {
                        sw[2 * g] = (uint32_t)tbl.scramble[wq][q1[g]];
                        sw[2 * g + 1] = (uint32_t)tbl.scramble[wq][q2[g]];
                    }
                    assemble_dual_plane((uint32_t)wq, (uint32_t)cq, alpha ? 12u : 8u, (uint32_t)pc, ev, nv, sw, out);
                }
            }
        }
        return best;
    }

    static void assemble_trial(const Trial& tr, bool alpha, uint8_t out[16]) {
        const Tables& tb = tables();
        const int nvals = alpha ? 8 : 6;
        const uint32_t ev[8] = {(uint32_t)tr.sym0[0], (uint32_t)tr.sym1[0], (uint32_t)tr.sym0[1],
                                (uint32_t)tr.sym1[1], (uint32_t)tr.sym0[2], (uint32_t)tr.sym1[2],
                                (uint32_t)tr.sym0[3], (uint32_t)tr.sym1[3]};
        uint32_t sw[16];
        for (int g = 0; g < 16; ++g) sw[g] = (uint32_t)tb.scramble[tr.wq][tr.q[g]];
        assemble_general((uint32_t)tr.wq, (uint32_t)tr.cq, alpha ? 12u : 8u, ev, nvals, sw, out);
    }

    // MainCS texel fetch (ASTC_Encode.hlsl:561-580)
    static void fetch(const uint8_t* rgba, int w, int h, int bx, int by,
                      const oracle_opts& o, T (*tex)[4]) {
        const int dim = o.block_dim;
        for (int kk = 0; kk < dim * dim; ++kk) {
            const int y = kk / dim, x = kk - y * dim;
            int px = bx * dim + x, py = by * dim + y;
            const bool inside = px < w && py < h;
            T c[4] = {0, 0, 0, 0};
            if (inside || o.border == 1) {
                if (px >= w) px = w - 1;
                if (py >= h) py = h - 1;
                const uint8_t* p = rgba + ((size_t)py * w + px) * 4;
                for (int ch = 0; ch < 4; ++ch) {
                    if (o.srgb && ch < 3) c[ch] = P::srgb(p[ch]);
                    else c[ch] = P::div((T)p[ch], P::lit(255.0f, 255.0));
                }
            }
            if (o.is_normal) { c[2] = P::lit(1.0f, 1.0); c[3] = P::lit(1.0f, 1.0); }
            for (int ch = 0; ch < 4; ++ch) tex[kk][ch] = P::mul(c[ch], P::lit(255.0f, 255.0));
        }
    }

    static int encode_image(const uint8_t* rgba, int w, int h, const oracle_opts* o,
                            uint8_t* out, int threads) {
        if (!rgba || !out || !o || w <= 0 || h <= 0) return -1;
        if (o->block_dim != 4 && o->block_dim != 6) return -2;
        if (o->border != 0 && o->border != 1) return -3;
        if (o->axis < 0 || o->axis > 2) return -4;
        if (o->quality < 0 || o->quality > 4) return -5;
        tables();
        const int dim = o->block_dim;
        const int nbx = (w + dim - 1) / dim, nby = (h + dim - 1) / dim;
        const long long nb = (long long)nbx * nby;
#ifdef _OPENMP
        const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
#else
        (void)threads;
#endif
        for (long long b = 0; b < nb; ++b) {
            const int by = (int)(b / nbx), bx = (int)(b - (long long)by * nbx);
            T tex[36][4];
            fetch(rgba, w, h, bx, by, *o, tex);
            if (o->quality || o->axis == 2) {
                // quality 0 with axis 2: the better of the two fixed-mode blocks
                int chosen;
                uint32_t err, err_fixed;
                search(tex, dim, o->has_alpha != 0, o->srgb != 0, o->quality >= 2 ? 2 : o->axis,
                       out + 16 * b, &chosen, &err, &err_fixed, o->quality >= 3 ? o->quality - 2 : 0,
                       o->quality >= 1, o->quality >= 2);
                continue;
            }
            uint32_t ep[8], qw[16];
            encode(tex, dim, o->has_alpha != 0, ep, qw, out + 16 * b, o->axis);
        }
        return 0;
    }
};

// ---------------------------------------------------------------------------
// Spec LDR decoder (integer only)
// ---------------------------------------------------------------------------
struct BlockMode {
    int gw, gh, dual, quant, ok;
};

BlockMode decode_block_mode(int m) {
    BlockMode r = {0, 0, 0, 0, 0};
    int R, H = bit(m, 9), D = bit(m, 10);
    if ((m & 3) != 0) {
        R = bit(m, 4) | (bit(m, 0) << 1) | (bit(m, 1) << 2);
        const int A = (m >> 5) & 3, B = (m >> 7) & 3;
        switch ((m >> 2) & 3) {
        case 0: r.gw = B + 4; r.gh = A + 2; break;
        case 1: r.gw = B + 8; r.gh = A + 2; break;
        case 2: r.gw = A + 2; r.gh = B + 8; break;
        default:
            if (bit(m, 8) == 0) { r.gw = A + 2; r.gh = bit(m, 7) + 6; }
            else { r.gw = bit(m, 7) + 2; r.gh = A + 2; }
        }
    } else {
        if (((m >> 2) & 3) == 0) return r;                 // reserved (incl. R<2)
        R = bit(m, 4) | (bit(m, 2) << 1) | (bit(m, 3) << 2);
        const int A = (m >> 5) & 3;
        switch ((m >> 7) & 3) {
        case 0: r.gw = 12; r.gh = A + 2; break;
        case 1: r.gw = A + 2; r.gh = 12; break;
        case 3:
            if (bit(m, 6)) return r;                       // reserved
            if (bit(m, 5) == 0) { r.gw = 6; r.gh = 10; } else { r.gw = 10; r.gh = 6; }
            break;
        default: {
            const int B = (m >> 9) & 3;
            r.gw = A + 6; r.gh = B + 6; H = 0; D = 0;
        }
        }
    }
    r.dual = D;
    r.quant = (R - 2) + 6 * H;
    r.ok = 1;
    return r;
}

inline int clamp255(int v) { return v < 0 ? 0 : v > 255 ? 255 : v; }

void bit_transfer_signed(int& a, int& b) {
    b >>= 1;
    b |= a & 0x80;
    a >>= 1;
    a &= 0x3F;
    if (a & 0x20) a -= 0x40;
}

void blue_contract(int c[4]) {
    c[0] = (c[0] + c[2]) >> 1;
    c[1] = (c[1] + c[2]) >> 1;
}

// Returns false for HDR / invalid CEMs.
bool unpack_endpoints(int cem, const int* v, int e0[4], int e1[4]) {
    switch (cem) {
    case 0:
        e0[0] = e0[1] = e0[2] = v[0]; e0[3] = 255;
        e1[0] = e1[1] = e1[2] = v[1]; e1[3] = 255;
        return true;
    case 1: {
        const int l0 = (v[0] >> 2) | (v[1] & 0xC0);
        int l1 = l0 + (v[1] & 0x3F);
        if (l1 > 255) l1 = 255;
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
        const int s0 = v[0] + v[2] + v[4], s1 = v[1] + v[3] + v[5];
        if (s1 >= s0) {
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
        return false;                                       // HDR modes
    }
}

// Spec partition hash (select_partition) for multi-partition blocks.
int select_partition(int seed, int x, int y, int z, int pcount, bool small) {
    if (small) { x <<= 1; y <<= 1; z <<= 1; }
    seed += (pcount - 1) * 1024;
    uint32_t p = (uint32_t)seed;
    p ^= p >> 15; p -= p << 17; p += p << 7; p += p << 4;
    p ^= p >> 5;  p += p << 16; p ^= p >> 7; p ^= p >> 3;
    p ^= p << 6;  p ^= p >> 17;
    const uint32_t rnum = p;
    // seed1..seed8 are the eight nibbles of rnum; seed9..seed12 start at
    // bits 18, 22, 26 and 30 (the last one wraps around to bit 0).
    int s[12];
    for (int i = 0; i < 8; ++i) s[i] = (rnum >> (4 * i)) & 0xF;
    s[8] = (rnum >> 18) & 0xF;
    s[9] = (rnum >> 22) & 0xF;
    s[10] = (rnum >> 26) & 0xF;
    s[11] = ((rnum >> 30) | (rnum << 2)) & 0xF;
    for (int i = 0; i < 12; ++i) s[i] *= s[i];
    int sh1, sh2;
    if (seed & 1) { sh1 = (seed & 2) ? 4 : 5; sh2 = (pcount == 3) ? 6 : 5; }
    else { sh1 = (pcount == 3) ? 6 : 5; sh2 = (seed & 2) ? 4 : 5; }
    const int sh3 = (seed & 0x10) ? sh1 : sh2;
    s[0] >>= sh1; s[1] >>= sh2; s[2] >>= sh1; s[3] >>= sh2;
    s[4] >>= sh1; s[5] >>= sh2; s[6] >>= sh1; s[7] >>= sh2;
    s[8] >>= sh3; s[9] >>= sh3; s[10] >>= sh3; s[11] >>= sh3;
    int a = s[0] * x + s[1] * y + s[10] * z + (int)(rnum >> 14);
    int b = s[2] * x + s[3] * y + s[11] * z + (int)(rnum >> 10);
    int c = s[4] * x + s[5] * y + s[8] * z + (int)(rnum >> 6);
    int d = s[6] * x + s[7] * y + s[9] * z + (int)(rnum >> 2);
    a &= 0x3F; b &= 0x3F; c &= 0x3F; d &= 0x3F;
    if (pcount < 4) d = 0;
    if (pcount < 3) c = 0;
    if (a >= b && a >= c && a >= d) return 0;
    if (b >= c && b >= d) return 1;
    if (c >= d) return 2;
    return 3;
}

const uint64_t* partition_masks(int dim) {
    struct Masks {
        uint64_t m[2][1024];
        Masks() {
            for (int d = 0; d < 2; ++d) {
                const int dim = d ? 6 : 4;
                for (int s = 0; s < 1024; ++s) {
                    uint64_t v = 0;
                    for (int y = 0; y < dim; ++y)
                        for (int x = 0; x < dim; ++x)
                            if (select_partition(s, x, y, 0, 2, dim * dim < 31) == 1) v |= 1ull << (y * dim + x);
                    m[d][s] = v;
                }
            }
        }
    };
    static const Masks masks;
    return masks.m[dim == 6 ? 1 : 0];
}

const std::vector<ThreeClass>& three_partition_classes(int dim) {
    struct Classes {
        std::vector<ThreeClass> c[2];
        Classes() {
            for (int d = 0; d < 2; ++d) {
                const int dim = d ? 6 : 4, n = dim * dim;
                std::vector<std::pair<uint64_t, uint64_t>> seen;
                for (int s = 0; s < 1024; ++s) {
                    int part[36], first[3] = {-1, -1, -1}, order = 0;
                    uint64_t m[3] = {0, 0, 0}, cm[3] = {0, 0, 0};
                    for (int i = 0; i < n; ++i) {
                        part[i] = select_partition(s, i % dim, i / dim, 0, 3, n < 31);
                        m[part[i]] |= 1ull << i;
                        if (first[part[i]] < 0) first[part[i]] = order++;
                        cm[first[part[i]]] |= 1ull << i;      // relabelled in order of first texel
                    }
                    if (!m[0] || !m[1] || !m[2]) continue;
                    bool dup = false;
                    for (const auto& q : seen) dup = dup || (q.first == cm[1] && q.second == cm[2]);
                    if (dup) continue;
                    seen.emplace_back(cm[1], cm[2]);
                    c[d].push_back(ThreeClass{s, m[1], m[2]});
                }
            }
        }
    };
    static const Classes cl;
    return cl.c[dim == 6 ? 1 : 0];
}

void error_block(int bw, int bh, uint8_t* out) {
    for (int i = 0; i < bw * bh; ++i) {
        out[i * 4 + 0] = 255; out[i * 4 + 1] = 0; out[i * 4 + 2] = 255; out[i * 4 + 3] = 255;
    }
}

// Decode one block to UNORM8 RGBA (bw*bh texels, row-major). Returns 0 on
// success, 1 for an error block.
int decode_block(const uint8_t* blk, int bw, int bh, bool srgb, uint8_t* out) {
    const Tables& tb = tables();
    const int mode = (int)read_bits(blk, 0, 11);
    if ((mode & 0x1FF) == 0x1FC) {                          // void extent
        if (bit(mode, 9)) { error_block(bw, bh, out); return 1; }   // HDR
        uint8_t c[4];
        for (int i = 0; i < 4; ++i) c[i] = (uint8_t)(read_bits(blk, 64 + 16 * i, 16) >> 8);
        for (int i = 0; i < bw * bh; ++i) std::memcpy(out + 4 * i, c, 4);
        return 0;
    }
    const BlockMode bm = decode_block_mode(mode);
    if (!bm.ok || bm.gw > bw || bm.gh > bh) { error_block(bw, bh, out); return 1; }
    const int pcount = (int)read_bits(blk, 11, 2) + 1;
    const int nweights = bm.gw * bm.gh * (bm.dual ? 2 : 1);
    const int wbits = ise_bits(bm.quant, nweights);
    if (nweights > 64 || wbits < 24 || wbits > 96 || (pcount == 4 && bm.dual)) {
        error_block(bw, bh, out);
        return 1;
    }
    int cems[4];
    int color_start, extra_cem_bits = 0;
    int below_weights = 128 - wbits;
    if (pcount == 1) {
        cems[0] = (int)read_bits(blk, 13, 4);
        color_start = 17;
    } else {
        color_start = 29;
        const int cem_field = (int)read_bits(blk, 23, 6);
        if ((cem_field & 3) == 0) {
            for (int p = 0; p < pcount; ++p) cems[p] = cem_field >> 2;
        } else {
            extra_cem_bits = 3 * pcount - 4;
            const int extra = (int)read_bits(blk, below_weights - extra_cem_bits, extra_cem_bits);
            const int combined = (cem_field >> 2) | (extra << 4);
            const int base = (cem_field & 3) - 1;
            for (int p = 0; p < pcount; ++p) {
                const int cls = (combined >> p) & 1;
                const int m = (combined >> (pcount + 2 * p)) & 3;
                cems[p] = ((base + cls) << 2) | m;
            }
        }
    }
    const int plane2_bits = bm.dual ? 2 : 0;
    const int color_end = below_weights - extra_cem_bits - plane2_bits;
    const int plane2_comp = bm.dual ? (int)read_bits(blk, color_end, 2) : -1;
    int nvals = 0;
    for (int p = 0; p < pcount; ++p) nvals += 2 * ((cems[p] >> 2) + 1);
    const int color_bits = color_end - color_start;
    if (nvals > 18 || color_bits < 0) { error_block(bw, bh, out); return 1; }
    int cq = -1;
    for (int q = QUANT_256; q >= QUANT_2; --q)
        if (ise_bits(q, nvals) <= color_bits) { cq = q; break; }
    if (cq < QUANT_6) { error_block(bw, bh, out); return 1; }
    uint32_t cv[18];
    ise_decode(cq, nvals, blk, color_start, cv);
    int ep[4][2][4];
    int off = 0;
    for (int p = 0; p < pcount; ++p) {
        int v[8];
        const int n = 2 * ((cems[p] >> 2) + 1);
        for (int i = 0; i < n; ++i) v[i] = tb.cunq[cq][cv[off + i]];
        off += n;
        if (!unpack_endpoints(cems[p], v, ep[p][0], ep[p][1])) { error_block(bw, bh, out); return 1; }
    }
    // weights: stored bit-reversed from bit 127 downward
    uint8_t rev[16];
    for (int i = 0; i < 16; ++i) rev[i] = (uint8_t)reverse_byte(blk[15 - i]);
    uint32_t wv[64];
    ise_decode(bm.quant, nweights, rev, 0, wv);
    int wq[64];
    for (int i = 0; i < nweights; ++i) wq[i] = tb.wunq[bm.quant][wv[i]];
    // infill (spec bilinear decimation), per plane
    const int planes = bm.dual ? 2 : 1;
    const int ds = (1024 + bw / 2) / (bw - 1), dt = (1024 + bh / 2) / (bh - 1);
    const bool small = bw * bh < 31;
    const int seed = pcount > 1 ? (int)read_bits(blk, 13, 10) : 0;
    for (int t = 0; t < bh; ++t)
        for (int s = 0; s < bw; ++s) {
            int w[2] = {0, 0};
            for (int pl = 0; pl < planes; ++pl) {
                const int gs = (ds * s * (bm.gw - 1) + 32) >> 6;
                const int gt = (dt * t * (bm.gh - 1) + 32) >> 6;
                const int js = gs >> 4, fs = gs & 0xF, jt = gt >> 4, ft = gt & 0xF;
                const int w11 = (fs * ft + 8) >> 4, w10 = ft - w11, w01 = fs - w11;
                const int w00 = 16 - fs - ft + w11;
                const int v0 = js + jt * bm.gw;
                auto P = [&](int idx) -> int {
                    return (idx < bm.gw * bm.gh) ? wq[idx * planes + pl] : 0;
                };
                int acc = P(v0) * w00;
                if (w01) acc += P(v0 + 1) * w01;
                if (w10) acc += P(v0 + bm.gw) * w10;
                if (w11) acc += P(v0 + bm.gw + 1) * w11;
                w[pl] = (acc + 8) >> 4;
            }
            const int part = pcount > 1 ? select_partition(seed, s, t, 0, pcount, small) : 0;
            uint8_t* o = out + 4 * (t * bw + s);
            for (int c = 0; c < 4; ++c) {
                const int wt = (c == plane2_comp) ? w[1] : w[0];
                const int c0 = srgb ? ((ep[part][0][c] << 8) | 0x80) : ep[part][0][c] * 257;
                const int c1 = srgb ? ((ep[part][1][c] << 8) | 0x80) : ep[part][1][c] * 257;
                const int v = (c0 * (64 - wt) + c1 * wt + 32) >> 6;
                o[c] = (uint8_t)(v >> 8);
            }
        }
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// C interface
// ---------------------------------------------------------------------------
extern "C" {

int oracle_encode_fp32(const uint8_t* rgba, int width, int height, const oracle_opts* opts,
                       uint8_t* out_blocks, int threads) {
    return Pipe<F32>::encode_image(rgba, width, height, opts, out_blocks, threads);
}

int oracle_encode_fp64(const uint8_t* rgba, int width, int height, const oracle_opts* opts,
                       uint8_t* out_blocks, int threads) {
    return Pipe<F64>::encode_image(rgba, width, height, opts, out_blocks, threads);
}

int oracle_encode_block_fp32(const float* texels, int block_dim, int has_alpha, uint32_t ep[8],
                             uint32_t qw[16], uint8_t out[16]) {
    if (!texels || (block_dim != 4 && block_dim != 6)) return -1;
    float tex[36][4];
    for (int i = 0; i < block_dim * block_dim; ++i)
        for (int c = 0; c < 4; ++c) tex[i][c] = texels[4 * i + c];
    Pipe<F32>::encode(tex, block_dim, has_alpha != 0, ep, qw, out);
    return 0;
}

int oracle_trace_block_fp32(const float* texels, int block_dim, int has_alpha, float start_w,
                            oracle_trace* tr) {
    if (!texels || !tr || (block_dim != 4 && block_dim != 6)) return -1;
    float tex[36][4];
    for (int i = 0; i < block_dim * block_dim; ++i)
        for (int c = 0; c < 4; ++c) tex[i][c] = texels[4 * i + c];
    std::memset(tr, 0, sizeof(*tr));
    tr->start_w = start_w;
    float e0[4], e1[4];
    Pipe<F32>::pca(tex, block_dim * block_dim, has_alpha != 0, e0, e1, tr);
    trace_put(tr->e0, e0, 4);
    trace_put(tr->e1, e1, 4);
    for (int c = 0; c < 4; ++c) {                           // encode_color 233-245
        tr->ep[2 * c] = (uint32_t)std::rint(e0[c]);
        tr->ep[2 * c + 1] = (uint32_t)std::rint(e1[c]);
    }
    Pipe<F32>::weights(tex, block_dim, e0, e1, has_alpha ? 5u : 11u, tr->qw, tr);
    assemble_symbolic(tr->ep, tr->qw, has_alpha != 0, tr->block);
    return 0;
}

int oracle_find_seed(const float* texels, int block_dim, int has_alpha, const uint8_t target[16],
                     const float* seeds, int n_seeds) {
    if (!texels || !target || !seeds || n_seeds < 0) return -2;
    oracle_trace tr;
    for (int i = 0; i < n_seeds; ++i) {
        if (oracle_trace_block_fp32(texels, block_dim, has_alpha, seeds[i], &tr) != 0) return -2;
        if (std::memcmp(tr.block, target, 16) == 0) return i;
    }
    return -1;
}

int oracle_assemble_symbolic(const uint32_t ep[8], const uint32_t qw[16], int has_alpha,
                             uint8_t out[16]) {
    const uint32_t range = has_alpha ? 5u : 11u;
    for (int i = 0; i < 8; ++i) if (ep[i] > 255) return -1;
    for (int i = 0; i < 16; ++i) if (qw[i] > range) return -1;
    assemble_symbolic(ep, qw, has_alpha != 0, out);
    return 0;
}

int oracle_ise_encode(int quant, int count, const uint32_t* values, uint8_t out[16]) {
    if (quant < 0 || quant >= QUANT_MAX || count < 0 || ise_bits(quant, count) > 128) return -1;
    for (int i = 0; i < count; ++i) if (values[i] >= (uint32_t)kQuantLevels[quant]) return -1;
    Bits128 o = {{0, 0, 0, 0}};
    ise_encode(quant, count, values, o);
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 4; ++k) out[4 * i + k] = (uint8_t)(o.w[i] >> (8 * k));
    return 0;
}

int oracle_ise_decode(int quant, int count, const uint8_t in[16], int bit_offset,
                      uint32_t* values) {
    if (quant < 0 || quant >= QUANT_MAX || count < 0) return -1;
    ise_decode(quant, count, in, bit_offset, values);
    return 0;
}

int oracle_ise_bits(int quant, int count) {
    if (quant < 0 || quant >= QUANT_MAX || count < 0) return -1;
    return ise_bits(quant, count);
}

void oracle_table_trits(int out[243]) { std::memcpy(out, tables().trits_enc, sizeof(int) * 243); }
void oracle_table_quints(int out[125]) { std::memcpy(out, tables().quints_enc, sizeof(int) * 125); }
void oracle_table_btq(int out[63]) { std::memcpy(out, tables().btq, sizeof(int) * 63); }
void oracle_table_scramble(int out[384]) { std::memcpy(out, tables().scramble, sizeof(int) * 384); }
void oracle_srgb_lut(float out[256]) {
    for (int c = 0; c < 256; ++c) out[c] = tables().srgb_lut[c] * 255.0f;
}

int oracle_decode_block(const uint8_t blk[16], int block_w, int block_h, int srgb,
                        uint8_t* out_rgba) {
    if (block_w < 2 || block_h < 2 || block_w > 12 || block_h > 12) return -1;
    return decode_block(blk, block_w, block_h, srgb != 0, out_rgba);
}

int oracle_decode(const uint8_t* blocks, int width, int height, int block_w, int block_h,
                  int srgb, uint8_t* out_rgba) {
    if (!blocks || !out_rgba || width <= 0 || height <= 0) return -1;
    if (block_w < 2 || block_h < 2 || block_w > 12 || block_h > 12) return -1;
    const int nbx = (width + block_w - 1) / block_w, nby = (height + block_h - 1) / block_h;
    int errors = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(+ : errors)
#endif
    for (int by = 0; by < nby; ++by)
        for (int bx = 0; bx < nbx; ++bx) {
            uint8_t tmp[144 * 4];
            errors += decode_block(blocks + 16 * ((size_t)by * nbx + bx), block_w, block_h,
                                   srgb != 0, tmp);
            for (int y = 0; y < block_h; ++y)
                for (int x = 0; x < block_w; ++x) {
                    const int px = bx * block_w + x, py = by * block_h + y;
                    if (px < width && py < height)
                        std::memcpy(out_rgba + 4 * ((size_t)py * width + px),
                                    tmp + 4 * (y * block_w + x), 4);
                }
        }
    return errors;
}

int oracle_unquant_weight(int quant, int value) {
    if (quant < 0 || quant >= 12 || value < 0 || value >= kQuantLevels[quant]) return -1;
    return spec_unquant_weight(quant, value);
}

int oracle_unquant_color(int quant, int value) {
    // colour endpoints are never coded below QUANT_6 (the decoder rejects it)
    if (quant < QUANT_6 || quant >= QUANT_MAX || value < 0 || value >= kQuantLevels[quant]) return -1;
    return spec_unquant_color(quant, value);
}

void oracle_grid_taps(int g, int idx[4], float wt[4]) {
    Pipe<F32>::grid_taps(g & 15, idx, wt);
}

int oracle_three_classes(int dim, int* seeds, uint64_t* m1, uint64_t* m2, int cap) {
    if (dim != 4 && dim != 6) return -1;
    const std::vector<ThreeClass>& cls = three_partition_classes(dim);
    const int n = (int)cls.size();
    for (int i = 0; i < n && i < cap; ++i) {
        seeds[i] = cls[i].seed;
        m1[i] = cls[i].m1;
        m2[i] = cls[i].m2;
    }
    return n;
}

int oracle_endpoint_quant(int wq, int nvals) {
    if (nvals != 6 && nvals != 8) return -1;
    return endpoint_quant(wq, nvals);
}

int oracle_search_block_fp32(const float* texels, int block_dim, int has_alpha, int srgb, int axis,
                             int partitions, uint8_t out[16], int* chosen_wq, uint32_t* err,
                             uint32_t* err_fixed) {
    if (!texels || !out || !chosen_wq || !err || !err_fixed) return -1;
    if ((block_dim != 4 && block_dim != 6) || axis < 0 || axis > 2) return -1;
    float tex[36][4];
    for (int i = 0; i < block_dim * block_dim; ++i)
        for (int c = 0; c < 4; ++c) tex[i][c] = texels[4 * i + c];
    if (partitions < 0 || partitions > 2) return -1;
    Pipe<F32>::search(tex, block_dim, has_alpha != 0, srgb != 0, axis, out, chosen_wq, err, err_fixed,
                      partitions, true, axis == 2);
    return 0;
}

double oracle_flops_per_block(int block_dim, int has_alpha, int is_normal) {
    if (block_dim != 4 && block_dim != 6) return -1.0;
    // A fixed non-degenerate block: every stage runs its full path.
    float tex[36][4];
    uint32_t s = 12345u;
    for (int i = 0; i < block_dim * block_dim; ++i)
        for (int c = 0; c < 4; ++c) {
            s = s * 1664525u + 1013904223u;
            tex[i][c] = (float)((s >> 24) & 0xFF);
            if (is_normal && c >= 2) tex[i][c] = 255.0f;
        }
    g_flops = 0.0;
    uint32_t ep[8], qw[16];
    uint8_t out[16];
    Pipe<F32Count>::encode(tex, block_dim, has_alpha != 0, ep, qw, out);
    return g_flops;
}

}  // extern "C"
