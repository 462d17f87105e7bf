// astc_ise.h -- integer sequence encoding (ISE) for the search-mode block
// assemblers, host and device.  The assemblers run it once per block, where
// long straight-line code pays an instruction-cache miss on nearly every
// instruction: a runtime range goes through one rolled loop over the values
// (ise_encode_packed), and the few legal weight ranges of each call site get
// short compile-time forms (ise_encode_fixed).
//
// The sequence follows the reference's ASTC_IntegerSequenceEncoding.hlsl
// (encode_trits 142-176, encode_quints 181-205, bise_* 207-276): values of a
// range with a trit (quint) factor go in groups of five (three), each value's
// low `bits` bits followed by a field of the group's packed digit T:
//   trits:  m0 T[1:0] m1 T[3:2] m2 T[4] m3 T[6:5] m4 T[7]
//   quints: m0 Q[2:0] m1 Q[4:3] m2 Q[6:5]
// a last partial group is padded with zero values, and the sequence is cut to
// ise_bit_count(quant, count) bits.  Plain ranges are bit fields.
#pragma once
#include "astc_tables.h"

namespace astc {

struct Bits128 { uint64_t lo, hi; };

// OR x into b from bit pos (0 <= pos < 128); bits past 127 are dropped.
ASTC_HD inline void put_bits64(Bits128& b, int pos, uint64_t x) {
    if (pos < 64) {
        b.lo |= x << pos;
        if (pos > 0) b.hi |= x >> (64 - pos);
    } else {
        b.hi |= x << (pos - 64);
    }
}

ASTC_HD inline void keep_low_bits(Bits128& b, int n) {
    if (n < 64) { b.lo &= (n ? (~0ull >> (64 - n)) : 0ull); b.hi = 0; }
    else if (n < 128) { b.hi &= (n > 64 ? (~0ull >> (128 - n)) : 0ull); }
}

// Pack N byte values four to a word, value i in byte i % 4 of word i / 4.
template <int N>
ASTC_HD inline void pack_bytes(const uint32_t (&v)[N], uint32_t (&w)[(N + 3) / 4]) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int k = 0; k < (N + 3) / 4; ++k) {
        uint32_t x = 0;
        for (int j = 0; j < 4; ++j)
            if (4 * k + j < N) x |= (v[4 * k + j < N ? 4 * k + j : 0] & 0xFFu) << (8 * j);
        w[k] = x;
    }
}

// `count` values of range `quant`, packed by pack_bytes into w (consumed).
// trits/quints: the digit packing tables (T of t4*81+...+t0, Q of q2*25+q1*5+q0).
// Within a group, value j sits at j*bits + c_j and the digit field after it
// at (j+1)*bits + c_j, c_{j+1} - c_j bits wide, holding bits c_j.. of T, with
// c = 0 2 4 5 7 8 (trits) or 0 3 5 7 (quints); the group is c_gs + gs*bits
// bits long.
template <int WORDS>
ASTC_HD inline Bits128 ise_encode_packed(int quant, int count, uint32_t (&w)[WORDS], const uint8_t* trits,
                                         const uint8_t* quints) {
    const RangeShape sh = range_shape(quant);
    const int b = sh.bits;
    const uint32_t mask = (1u << b) - 1u;
    const int gs = sh.trits ? 5 : sh.quints ? 3 : 1;
    const uint32_t base = sh.trits ? 3u : 5u;
    const uint32_t cpack = sh.trits ? 0x875420u : sh.quints ? 0x7530u : 0u;   // c_j in nibble j
    const int gbits = gs * b + (int)((cpack >> (4 * gs)) & 0xFu);
    Bits128 o{0ull, 0ull};
    uint64_t group = 0;
    uint32_t digits = 0, mul = 1;
    int j = 0, pos = 0;
#ifdef __CUDA_ARCH__
#pragma unroll 1
#endif
    for (int i = 0; i < count; ++i) {
        const uint32_t x = w[0] & 0xFFu;
        w[0] >>= 8;
        if ((i & 3) == 3) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
            for (int k = 0; k + 1 < WORDS; ++k) w[k] = w[k + 1];
            w[WORDS - 1] = 0;
        }
        group |= (uint64_t)(x & mask) << (j * b + (int)((cpack >> (4 * j)) & 0xFu));
        digits += (x >> b) * mul;
        mul *= base;
        if (++j == gs || i == count - 1) {
            if (gs > 1) {
                const uint32_t T = sh.trits ? trits[digits] : quints[digits];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
                for (int k = 0; k < 5; ++k) {
                    if (k < gs) {
                        const int ck = (int)((cpack >> (4 * k)) & 0xFu), ck1 = (int)((cpack >> (4 * k + 4)) & 0xFu);
                        group |= (uint64_t)((T >> ck) & ((1u << (ck1 - ck)) - 1u)) << ((k + 1) * b + ck);
                    }
                }
            }
            put_bits64(o, pos, group);
            pos += gbits;
            group = 0;
            digits = 0;
            mul = 1;
            j = 0;
        }
    }
    keep_low_bits(o, ise_bit_count(quant, count));
    return o;
}

// The same sequence for a range known at compile time: every value's and
// digit field's position is a constant, so the code is a few independent
// shifts per value instead of a loop whose group ends diverge across threads
// holding different ranges.  On GB300 the rolled loop spent 125 us of an
// 842 us 4x4 normal-map THOROUGH launch on the dual-plane blocks' 32 weights,
// this form 23 us; with it at every weight site (rolled loop for endpoints)
// against the rolled loop everywhere: SEARCH 274 -> 253 us, THOROUGH 768 ->
// 715 us, PARTITIONS 1595 -> 1469 us (4x4 normal map), SEARCH 97.5 -> 93.7 us
// (6x6 RGBA sRGB).
template <int Q, int COUNT>
ASTC_HD inline Bits128 ise_encode_fixed(const uint32_t (&v)[COUNT], const uint8_t* trits, const uint8_t* quints) {
    constexpr RangeShape sh = range_shape(Q);
    constexpr int b = sh.bits;
    constexpr uint32_t mask = (1u << b) - 1u;
    constexpr int gs = sh.trits ? 5 : sh.quints ? 3 : 1;
    constexpr uint32_t cpack = sh.trits ? 0x875420u : sh.quints ? 0x7530u : 0u;
    constexpr int gbits = gs * b + (int)((cpack >> (4 * gs)) & 0xFu);
    Bits128 o{0ull, 0ull};
    auto put = [&](int pos, uint32_t x) {           // pos < 128, x below 2^9
        if (pos < 64) {
            o.lo |= (uint64_t)x << pos;
            if (pos > 55) o.hi |= (uint64_t)x >> (64 - pos);
        } else {
            o.hi |= (uint64_t)x << (pos - 64);
        }
    };
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int g = 0; g < (COUNT + gs - 1) / gs; ++g) {
        uint32_t digits = 0, mul = 1;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
        for (int j = 0; j < gs; ++j) {
            const int i = g * gs + j;
            const uint32_t x = i < COUNT ? v[i < COUNT ? i : 0] : 0u;
            if (b) put(g * gbits + j * b + (int)((cpack >> (4 * j)) & 0xFu), x & mask);
            digits += (x >> b) * mul;
            mul *= sh.trits ? 3u : 5u;
        }
        if (gs > 1) {
            const uint32_t T = sh.trits ? trits[digits] : quints[digits];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
            for (int k = 0; k < gs; ++k) {
                const int ck = (int)((cpack >> (4 * k)) & 0xFu), ck1 = (int)((cpack >> (4 * k + 4)) & 0xFu);
                put(g * gbits + (k + 1) * b + ck, (T >> ck) & ((1u << (ck1 - ck)) - 1u));
            }
        }
    }
    keep_low_bits(o, ise_bit_count(Q, COUNT));
    return o;
}

template <int COUNT, int Q, int QMAX>
ASTC_HD inline Bits128 ise_encode_chain(int quant, const uint32_t (&v)[COUNT], const uint8_t* trits,
                                        const uint8_t* quints) {
    if constexpr (Q < QMAX) {
        if (quant != Q) return ise_encode_chain<COUNT, Q + 1, QMAX>(quant, v, trits, quints);
    }
    return ise_encode_fixed<Q, COUNT>(v, trits, quints);
}

// Weights: a call site's legal weight ranges QMIN..QMAX each get their
// compile-time form (any other range takes the rolled loop).
template <int COUNT, int QMIN, int QMAX>
ASTC_HD inline Bits128 ise_encode_weights(int quant, const uint32_t (&v)[COUNT], const uint8_t* trits,
                                          const uint8_t* quints) {
    if (quant >= QMIN && quant <= QMAX) return ise_encode_chain<COUNT, QMIN, QMAX>(quant, v, trits, quints);
    uint32_t w[(COUNT + 3) / 4];
    pack_bytes<COUNT>(v, w);
    return ise_encode_packed<(COUNT + 3) / 4>(quant, COUNT, w, trits, quints);
}

// Endpoints: the rolled loop.  (A compile-time QUANT_256 path measured
// slower on GB300: 4x4 normal-map THOROUGH 715 -> 852 us, PARTITIONS 1469 ->
// 1673 us, as warps mixing QUANT_256 with other endpoint ranges ran both.)
template <int COUNT>
ASTC_HD inline Bits128 ise_encode_endpoints(int quant, const uint32_t (&v)[COUNT], const uint8_t* trits,
                                            const uint8_t* quints) {
    uint32_t w[(COUNT + 3) / 4];
    pack_bytes<COUNT>(v, w);
    return ise_encode_packed<(COUNT + 3) / 4>(quant, COUNT, w, trits, quints);
}

}  // namespace astc
