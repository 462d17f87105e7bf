// astc_tables.h -- ASTC integer tables built at compile time from the
// specification's definitions (host and device).
//
// The reference ships these as literal arrays:
//   bits_trits_quints_table  ASTC_IntegerSequenceEncoding.hlsl:5-28
//   integer_from_trits       ASTC_IntegerSequenceEncoding.hlsl:30-62
//   integer_from_quints      ASTC_IntegerSequenceEncoding.hlsl:64-71
//   scramble_table           ASTC_Table.hlsl:4-66
// Here every entry is derived: the trit/quint packings are the inverse of the
// spec's block decode (taking the largest code where several decode to the
// same digits, which is the choice the reference's arrays make), and the
// weight scramble orders each range's ISE symbols by their spec-unquantised
// weight value.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ASTC_HD __host__ __device__
#else
#define ASTC_HD
#endif

namespace astc {

enum QuantMethod : int {
    kQuant2 = 0, kQuant3, kQuant4, kQuant5, kQuant6, kQuant8, kQuant10, kQuant12,
    kQuant16, kQuant20, kQuant24, kQuant32, kQuant40, kQuant48, kQuant64, kQuant80,
    kQuant96, kQuant128, kQuant160, kQuant192, kQuant256, kQuantCount
};

// Number of levels of each quant method (QUANT_2 .. QUANT_256).
constexpr ASTC_HD int quant_levels(int q) {
    return q == 0 ? 2 : q == 1 ? 3 : q == 2 ? 4 : q == 3 ? 5 : q == 4 ? 6 : q == 5 ? 8
         : q == 6 ? 10 : q == 7 ? 12 : q == 8 ? 16 : q == 9 ? 20 : q == 10 ? 24 : q == 11 ? 32
         : q == 12 ? 40 : q == 13 ? 48 : q == 14 ? 64 : q == 15 ? 80 : q == 16 ? 96
         : q == 17 ? 128 : q == 18 ? 160 : q == 19 ? 192 : 256;
}

// Levels = 2^bits * {1, 3 (trit), 5 (quint)}.
struct RangeShape { int bits, trits, quints; };
constexpr ASTC_HD RangeShape range_shape(int quant) {
    int l = quant_levels(quant), b = 0;
    while ((l & 1) == 0) { l >>= 1; ++b; }
    return RangeShape{b, l == 3 ? 1 : 0, l == 5 ? 1 : 0};
}

constexpr ASTC_HD int ise_bit_count(int quant, int count) {
    const RangeShape s = range_shape(quant);
    return s.trits ? ((8 + 5 * s.bits) * count + 4) / 5
         : s.quints ? ((7 + 3 * s.bits) * count + 2) / 3
         : count * s.bits;
}

constexpr ASTC_HD int bit_of(int x, int i) { return (x >> i) & 1; }

// Spec: decode an 8-bit trit block T into five trits.
constexpr ASTC_HD void trit_block_decode(int T, int t[5]) {
    int C = 0;
    if (((T >> 2) & 7) == 7) {
        C = (((T >> 5) & 7) << 2) | (T & 3);
        t[4] = 2; t[3] = 2;
    } else {
        C = T & 31;
        if (((T >> 5) & 3) == 3) { t[4] = 2; t[3] = bit_of(T, 7); }
        else { t[4] = bit_of(T, 7); t[3] = (T >> 5) & 3; }
    }
    if ((C & 3) == 3) {
        t[2] = 2; t[1] = bit_of(C, 4);
        t[0] = (bit_of(C, 3) << 1) | (bit_of(C, 2) & (1 - bit_of(C, 3)));
    } else if (((C >> 2) & 3) == 3) {
        t[2] = 2; t[1] = 2; t[0] = C & 3;
    } else {
        t[2] = bit_of(C, 4); t[1] = (C >> 2) & 3;
        t[0] = (bit_of(C, 1) << 1) | (bit_of(C, 0) & (1 - bit_of(C, 1)));
    }
}

// Spec: decode a 7-bit quint block Q into three quints.
constexpr ASTC_HD void quint_block_decode(int Q, int q[3]) {
    if (((Q >> 1) & 3) == 3 && ((Q >> 5) & 3) == 0) {
        q[2] = (bit_of(Q, 0) << 2) | ((bit_of(Q, 4) & (1 - bit_of(Q, 0))) << 1) |
               (bit_of(Q, 3) & (1 - bit_of(Q, 0)));
        q[1] = 4; q[0] = 4;
        return;
    }
    int C = 0;
    if (((Q >> 1) & 3) == 3) {
        q[2] = 4;
        C = (((Q >> 3) & 3) << 3) | ((3 - ((Q >> 5) & 3)) << 1) | bit_of(Q, 0);
    } else {
        q[2] = (Q >> 5) & 3;
        C = Q & 31;
    }
    if ((C & 7) == 5) { q[1] = 4; q[0] = (C >> 3) & 3; }
    else { q[1] = (C >> 3) & 3; q[0] = C & 7; }
}

// Spec: unquantise a weight ISE symbol to 0..64.
constexpr ASTC_HD int unquant_weight(int quant, int v) {
    const RangeShape s = range_shape(quant);
    int r = 0;
    if (!s.trits && !s.quints) {
        int have = 0;
        while (have < 6) { r = (r << s.bits) | v; have += s.bits; }
        r >>= (have - 6);
    } else if (s.bits == 0) {
        if (s.trits) r = v == 0 ? 0 : v == 1 ? 32 : 63;
        else r = v == 0 ? 0 : v == 1 ? 16 : v == 2 ? 32 : v == 3 ? 47 : 63;
    } else {
        const int D = v >> s.bits, m = v & ((1 << s.bits) - 1);
        const int A = (m & 1) ? 0x7F : 0;
        const int b = bit_of(m, 1), c = bit_of(m, 2);
        int B = 0, C = 0;
        if (s.trits) {
            if (s.bits == 1) { C = 50; }
            else if (s.bits == 2) { C = 23; B = (b << 6) | (b << 2) | b; }
            else { C = 11; B = (c << 6) | (b << 5) | (c << 1) | b; }
        } else {
            if (s.bits == 1) { C = 28; }
            else { C = 13; B = (b << 6) | (b << 1) | b; }
        }
        int T = D * C + B;
        T ^= A;
        r = (A & 0x20) | (T >> 2);
    }
    return r > 32 ? r + 1 : r;
}

// Spec: unquantise a colour endpoint ISE symbol to 0..255.
constexpr ASTC_HD int unquant_color(int quant, int v) {
    const RangeShape s = range_shape(quant);
    if (!s.trits && !s.quints) {
        int r = 0, have = 0;
        while (have < 8) { r = (r << s.bits) | v; have += s.bits; }
        return r >> (have - 8);
    }
    const int D = v >> s.bits, m = v & ((1 << s.bits) - 1);
    const int A = (m & 1) ? 0x1FF : 0;
    const int b = bit_of(m, 1), c = bit_of(m, 2), d = bit_of(m, 3), e = bit_of(m, 4),
              f = bit_of(m, 5);
    int B = 0, C = 0;
    if (s.trits) {
        switch (s.bits) {
        case 1: C = 204; break;
        case 2: C = 93; B = (b << 8) | (b << 4) | (b << 2) | (b << 1); break;
        case 3: C = 44; B = (c << 8) | (b << 7) | (c << 3) | (b << 2) | (c << 1) | b; break;
        case 4: C = 22; B = (d << 8) | (c << 7) | (b << 6) | (d << 2) | (c << 1) | b; break;
        case 5: C = 11; B = (e << 8) | (d << 7) | (c << 6) | (b << 5) | (e << 1) | d; break;
        default: C = 5; B = (f << 8) | (e << 7) | (d << 6) | (c << 5) | (b << 4) | f; break;
        }
    } else {
        switch (s.bits) {
        case 1: C = 113; break;
        case 2: C = 54; B = (b << 8) | (b << 3) | (b << 2); break;
        case 3: C = 26; B = (c << 8) | (b << 7) | (c << 2) | (b << 1) | c; break;
        case 4: C = 13; B = (d << 8) | (c << 7) | (b << 6) | (d << 1) | c; break;
        default: C = 6; B = (e << 8) | (d << 7) | (c << 6) | (b << 5) | e; break;
        }
    }
    int T = D * C + B;
    T ^= A;
    return (A & 0x80) | (T >> 2);
}

struct IseTables {
    uint8_t trit_pack[243];      // t4*81+t3*27+t2*9+t1*3+t0 -> T
    uint8_t trit_unpack[256][5];
    uint8_t quint_pack[125];     // q2*25+q1*5+q0 -> Q
    uint8_t quint_unpack[128][3];
    uint8_t scramble[12][32];    // linear weight index -> ISE symbol
    uint8_t unscramble[12][32];  // ISE symbol -> linear weight index
    uint8_t weight_unq[12][32];  // ISE symbol -> 0..64
    uint8_t color_unq[kQuantCount][256];
};

constexpr IseTables make_ise_tables() {
    IseTables t{};
    for (int T = 0; T < 256; ++T) {
        int d[5] = {0, 0, 0, 0, 0};
        trit_block_decode(T, d);
        for (int i = 0; i < 5; ++i) t.trit_unpack[T][i] = (uint8_t)d[i];
        t.trit_pack[d[4] * 81 + d[3] * 27 + d[2] * 9 + d[1] * 3 + d[0]] = (uint8_t)T;
    }
    for (int Q = 0; Q < 128; ++Q) {
        int d[3] = {0, 0, 0};
        quint_block_decode(Q, d);
        for (int i = 0; i < 3; ++i) t.quint_unpack[Q][i] = (uint8_t)d[i];
        t.quint_pack[d[2] * 25 + d[1] * 5 + d[0]] = (uint8_t)Q;
    }
    for (int q = 0; q < 12; ++q) {
        const int n = quant_levels(q);
        int order[32] = {};
        for (int v = 0; v < n; ++v) {
            order[v] = v;
            t.weight_unq[q][v] = (uint8_t)unquant_weight(q, v);
        }
        for (int i = 1; i < n; ++i)
            for (int j = i; j > 0 && unquant_weight(q, order[j - 1]) > unquant_weight(q, order[j]); --j) {
                const int x = order[j];
                order[j] = order[j - 1];
                order[j - 1] = x;
            }
        for (int i = 0; i < n; ++i) {
            t.scramble[q][i] = (uint8_t)order[i];
            t.unscramble[q][order[i]] = (uint8_t)i;
        }
    }
    for (int q = 0; q < kQuantCount; ++q)
        for (int v = 0; v < quant_levels(q); ++v) t.color_unq[q][v] = (uint8_t)unquant_color(q, v);
    return t;
}

// Nibble-packed scramble of a trit weight range (index i -> bits [4i, 4i+4)).
constexpr uint64_t scramble_nibbles(int quant) {
    const IseTables t = make_ise_tables();
    uint64_t v = 0;
    for (int i = 0; i < quant_levels(quant); ++i) v |= (uint64_t)t.scramble[quant][i] << (4 * i);
    return v;
}

// Block mode word for a 4x4 weight grid, single plane (ASTC_Encode.hlsl:446-473).
constexpr ASTC_HD uint32_t blockmode_4x4_grid(int weight_quant) {
    const uint32_t a = (4 - 2) & 3, b = (4 - 4) & 3, d = 0;
    const uint32_t h = weight_quant < 6 ? 0u : 1u;
    const uint32_t r = (uint32_t)(weight_quant % 6) + 2u;
    return ((r >> 1) & 3u) | ((r & 1u) << 4) | (a << 5) | (b << 7) | (h << 9) | (d << 10);
}

// ---------------------------------------------------------------------------
// search mode: the single-partition modes with a 4x4 weight grid
// ---------------------------------------------------------------------------
// Endpoint quant method of weight quant method wq with nvals endpoint values:
// the decoder takes the largest range whose ISE fits between the header (17
// bits for one partition, 29 for two or three sharing one CEM, 19 for one
// dual-plane partition: its 2-bit plane selector sits below the weights) and
// the nweights weights (32 for dual plane); the mode is illegal outside 24..96
// weight bits, below QUANT_6, or above 18 endpoint values.
constexpr ASTC_HD int endpoint_quant_for(int wq, int nvals, int header_bits = 17, int nweights = 16) {
    if (wq < kQuant2 || wq > kQuant32 || nvals > 18) return -1;
    const int wbits = ise_bit_count(wq, nweights);
    if (wbits < 24 || wbits > 96) return -1;
    const int avail = 128 - header_bits - wbits;
    for (int q = kQuant256; q >= kQuant6; --q)
        if (ise_bit_count(q, nvals) <= avail) return q;
    return -1;
}

struct SearchTables {
    // (unquantised << 8) | symbol of the colour value nearest each byte
    // (ties: the smaller value), per endpoint range used below QUANT_256;
    // kind 0 = one partition (6 / 8 values), 1 = two partitions (12 / 16
    // values), 2 = one dual-plane partition (6 / 8 values, 32 weights), 3 =
    // three partitions (18 values; none with alpha: 24 exceed the format's 18)
    uint16_t color[4][2][8][256];  // [kind][alpha][slot][byte]
    int8_t slot[4][2][12];         // [kind][alpha][wq] -> slot, -1 = QUANT_256
    int8_t cq[4][2][12];           // [kind][alpha][wq] -> endpoint quant method
    uint8_t wval[12][32];          // [wq][value-order index] -> weight 0..64
    uint8_t scramble[12][32];      // [wq][value-order index] -> ISE symbol
    uint8_t trit_pack[256];
    uint8_t quint_pack[128];
    int nslots[4][2];              // [kind][alpha] rows of color in use
};

constexpr SearchTables make_search_tables() {
    SearchTables s{};
    const IseTables t = make_ise_tables();
    for (int pt = 0; pt < 4; ++pt)
    for (int a = 0; a < 2; ++a) {
        int nslots = 0;
        for (int wq = 0; wq < 12; ++wq) {
            const int parts = pt == 3 ? 3 : pt == 1 ? 2 : 1;
            const int cq = pt == 2 ? endpoint_quant_for(wq, a ? 8 : 6, 19, 32)
                                   : endpoint_quant_for(wq, (a ? 8 : 6) * parts, parts > 1 ? 29 : 17);
            s.cq[pt][a][wq] = (int8_t)cq;
            s.slot[pt][a][wq] = -1;
            if (cq < 0 || cq == kQuant256) continue;
            int slot = -1;
            for (int w2 = 0; w2 < wq; ++w2)
                if (s.cq[pt][a][w2] == cq) slot = s.slot[pt][a][w2];
            if (slot < 0) {
                slot = nslots++;
                // symbols by value, then each byte's nearest on either side
                int sym_at[256] = {};
                for (int v = 0; v < 256; ++v) sym_at[v] = -1;
                for (int v = 0; v < quant_levels(cq); ++v) sym_at[unquant_color(cq, v)] = v;
                int below[256] = {}, above[256] = {};
                int last = 0;
                for (int v = 0; v < 256; ++v) { if (sym_at[v] >= 0) last = v; below[v] = last; }
                last = 255;
                for (int v = 255; v >= 0; --v) { if (sym_at[v] >= 0) last = v; above[v] = last; }
                for (int v = 0; v < 256; ++v) {
                    const int u = (v - below[v] <= above[v] - v) ? below[v] : above[v];
                    s.color[pt][a][slot][v] = (uint16_t)((u << 8) | sym_at[u]);
                }
            }
            s.slot[pt][a][wq] = (int8_t)slot;
        }
        s.nslots[pt][a] = nslots;
    }
    for (int wq = 0; wq < 12; ++wq)
        for (int i = 0; i < quant_levels(wq); ++i) {
            s.scramble[wq][i] = t.scramble[wq][i];
            s.wval[wq][i] = t.weight_unq[wq][t.scramble[wq][i]];
        }
    for (int i = 0; i < 243; ++i) s.trit_pack[i] = t.trit_pack[i];
    for (int i = 0; i < 125; ++i) s.quint_pack[i] = t.quint_pack[i];
    return s;
}

// Spec bilinear infill of a 4x4 weight grid at texel k of a 6x6 block: the
// grid index of the top-left tap and the four tap weights (sum 16).
struct Infill { int v0, w00, w01, w10, w11; };
constexpr ASTC_HD Infill infill_6x6(int k) {
    const int s = k % 6, t = k / 6, ds = (1024 + 3) / 5;
    const int gs = (ds * s * 3 + 32) >> 6, gt = (ds * t * 3 + 32) >> 6;
    const int fs = gs & 15, ft = gt & 15, w11 = (fs * ft + 8) >> 4;
    return Infill{(gs >> 4) + 4 * (gt >> 4), 16 - fs - ft + w11, fs - w11, ft - w11, w11};
}

}  // namespace astc
