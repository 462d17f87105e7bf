// astc_ise.h -- integer sequence encoding (ISE) for the search-mode block
// assemblers, host and device: one rolled loop over the values instead of
// straight-line code per value.  The assemblers run it once per block, and
// code that runs once per block must stay short: long straight-line code run
// once per warp pays an instruction-cache miss on nearly every instruction.
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

}  // namespace astc
