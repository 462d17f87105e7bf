// astc_pipeline_partition.cuh -- two-partition candidates of the FP32
// encoder's ASTC_QUALITY_PARTITIONS mode (the reference shader has only a
// commented-out bit-layout stub for partitions, ASTC_Encode.hlsl:422-431).
//
// From the kept single-partition fit's rounded endpoints E0/E1, the texels
// beyond their midpoint (2 dot(t - E0, E1 - E0) > |E1 - E0|^2) form the ideal
// split.  The partition index whose specification pattern, or its complement,
// differs from it in the fewest texels is taken (smallest index on ties; the
// scan runs over one index per {pattern, complement} class, which picks the
// same index as a scan of all 1024).  Each partition is fitted on its own
// (mean and covariance over its texels with correctly rounded divisions by
// the texel count, the shader's power iteration and find_min_max), then every
// weight range whose endpoint range (12 or 16 values after the 29-bit
// header: mode, partition count, index, one shared CEM) is legal is scored
// like the single-partition search, with each texel decoded on its own
// partition.  The oracle's two_partitions follows the same steps.
#pragma once
#include "astc_partition_table.h"
#include "astc_pipeline_search.cuh"

namespace astc {

// Unroll factor of the candidates' per-texel loops: rolled loops keep the
// candidate loop short (instruction fetch), unrolled ones keep the texels in
// registers (a rolled loop indexes them, so they live in local memory).  On
// GB300 with the rolled ISE encoder, PARTITIONS launches: 4x4 normal map
// 4096^2 1.63 ms rolled, 1.66 at 4, 1.75 unrolled (4x4 RGB 512^2: 90, 86,
// 84 us); 6x6 RGBA sRGB 2048^2 615 us at 2, 560 unrolled.
template <int DIM>
constexpr int kPartTexelUnroll = DIM == 4 ? 1 : 36;

// Per-CTA copies of the two-partition tables (shared memory).
struct PartSmem {
    uint16_t color[8][256];                  // endpoint ranges of two-partition modes
    union {
        uint64_t c6[kPartition2Classes6x6Count];   // (index << 54) | 36-bit pattern
        uint32_t c4[kPartition2Classes4x4Count];   // (index << 16) | 16-bit pattern
    } classes;
    int8_t cq[12];                           // weight range -> endpoint range (-1: illegal)
    int8_t slot[12];
    int nclasses;
};

// One partition's fit over the texels in `sel` (q0/q1: rounded endpoints,
// darker first; alpha 255 without ALPHA).
template <int N, bool ALPHA, class S>
__device__ __forceinline__ void fit_partition(const S& st, uint64_t sel, uint32_t q0[4], uint32_t q1[4]) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (!((sel >> k) & 1)) continue;
        const float4 t = st.get(k);
        s0 = __fadd_rn(s0, t.x); s1 = __fadd_rn(s1, t.y); s2 = __fadd_rn(s2, t.z); s3 = __fadd_rn(s3, t.w);
    }
    const int cnt = __popcll(sel);
    const float fc = (float)cnt;
    const float4 m = make_float4(__fdiv_rn(s0, fc), __fdiv_rn(s1, fc), __fdiv_rn(s2, fc), __fdiv_rn(s3, fc));
    float c00 = 0.f, c01 = 0.f, c02 = 0.f, c03 = 0.f, c11 = 0.f, c12 = 0.f, c13 = 0.f,
          c22 = 0.f, c23 = 0.f, c33 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (!((sel >> k) & 1)) continue;
        const float4 t = st.get(k);
        const float d0 = __fsub_rn(t.x, m.x), d1 = __fsub_rn(t.y, m.y);
        const float d2 = __fsub_rn(t.z, m.z), d3 = __fsub_rn(t.w, m.w);
        c00 = __fmaf_rn(d0, d0, c00); c01 = __fmaf_rn(d0, d1, c01);
        c02 = __fmaf_rn(d0, d2, c02); c03 = __fmaf_rn(d0, d3, c03);
        c11 = __fmaf_rn(d1, d1, c11); c12 = __fmaf_rn(d1, d2, c12);
        c13 = __fmaf_rn(d1, d3, c13); c22 = __fmaf_rn(d2, d2, c22);
        c23 = __fmaf_rn(d2, d3, c23); c33 = __fmaf_rn(d3, d3, c33);
    }
    const float den = (float)(cnt > 1 ? cnt - 1 : 1);
    c00 = __fdiv_rn(c00, den); c01 = __fdiv_rn(c01, den); c02 = __fdiv_rn(c02, den);
    c03 = __fdiv_rn(c03, den); c11 = __fdiv_rn(c11, den); c12 = __fdiv_rn(c12, den);
    c13 = __fdiv_rn(c13, den); c22 = __fdiv_rn(c22, den); c23 = __fdiv_rn(c23, den);
    c33 = __fdiv_rn(c33, den);
    const float4 v = power_iteration(c00, c01, c02, c03, c11, c12, c13, c22, c23, c33);
    float e0[4], e1[4];
    find_min_max<N, ALPHA>(st, m, v, e0, e1, q0, q1, sel);
}

// The squared error of a two-partition decode: as BlockError::eval with the
// endpoints of each texel's partition (bit k of sel1 set: partition 1).
template <int DIM, bool ALPHA, bool SRGB>
__device__ __forceinline__ uint32_t eval_two_partitions(const uint32_t (&tw)[DIM * DIM], uint32_t t2, uint64_t sel1,
                                                        const int E0[2][4], const int E1[2][4], const int (&W)[16]) {
    constexpr int NCH = ALPHA ? 4 : 3;
    int base[2][NCH], delta[2][NCH];
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const int c0 = SRGB ? ((E0[p][c] << 8) | 0x80) : E0[p][c] * 257;
            const int c1 = SRGB ? ((E1[p][c] << 8) | 0x80) : E1[p][c] * 257;
            base[p][c] = 4 * (64 * c0 + 32);
            delta[p][c] = 4 * (c1 - c0);
        }
    uint32_t dd = 0, dt = 0;
#pragma unroll kPartTexelUnroll<DIM>
    for (int k = 0; k < DIM * DIM; ++k) {
        int w;
        if constexpr (DIM == 6) {
            const Infill f = infill_6x6(k);
            int acc = W[f.v0] * f.w00;
            if (f.w01) acc += W[f.v0 + 1] * f.w01;
            if (f.w10) acc += W[f.v0 + 4] * f.w10;
            if (f.w11) acc += W[f.v0 + 5] * f.w11;
            w = (acc + 8) >> 4;
        } else {
            w = W[k];
        }
        const bool p1 = (sel1 >> k) & 1;
        uint32_t v[NCH];
#pragma unroll
        for (int c = 0; c < NCH; ++c)
            v[c] = (uint32_t)((p1 ? base[1][c] : base[0][c]) + (p1 ? delta[1][c] : delta[0][c]) * w);
        uint32_t dec = __byte_perm(v[0], v[1], 0x3362u);
        dec = __byte_perm(dec, v[2], 0x3610u);
        if constexpr (ALPHA) dec = __byte_perm(dec, v[3], 0x6210u);
        dd = __dp4a(dec, dec, dd);
        dt = __dp4a(dec, tw[k], dt);
    }
    return dd - 2u * dt + t2;
}

// Snapped endpoints of both partitions for the endpoint range whose
// nearest-colour table is row `slot` (symbols and decoded values, darker
// first in each partition).
template <bool ALPHA>
__device__ __forceinline__ void snap_two(int slot, const uint32_t a0[4], const uint32_t a1[4],
                                         const uint32_t b0[4], const uint32_t b1[4], const PartSmem& pm,
                                         int sym0[2][4], int sym1[2][4], int E0[2][4], int E1[2][4]) {
    constexpr int NCH = ALPHA ? 4 : 3;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const uint32_t* lo = p ? b0 : a0;
        const uint32_t* hi = p ? b1 : a1;
#pragma unroll
        for (int c = 0; c < 4; ++c) { sym0[p][c] = 0; sym1[p][c] = 0; E0[p][c] = 255; E1[p][c] = 255; }
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const uint32_t x = pm.color[slot][lo[c]], y = pm.color[slot][hi[c]];
            sym0[p][c] = (int)(x & 0xFFu); E0[p][c] = (int)(x >> 8);
            sym1[p][c] = (int)(y & 0xFFu); E1[p][c] = (int)(y >> 8);
        }
        if (E1[p][0] + E1[p][1] + E1[p][2] < E0[p][0] + E0[p][1] + E0[p][2]) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                int t = sym0[p][c]; sym0[p][c] = sym1[p][c]; sym1[p][c] = t;
                t = E0[p][c]; E0[p][c] = E1[p][c]; E1[p][c] = t;
            }
        }
    }
}

// Integer projections (UNORM input, where every fit-space texel value is an
// integer): for a texel's packed bytes t (the target word: blue and alpha
// 255 for normal maps, alpha 0 for RGB blocks, whose endpoint alpha
// difference is 0), dot(t - E0, E1 - E0) = t.dpos - t.dneg - E0.d with the
// difference split into its positive and negative parts, exactly; the FP32
// dot product of the same integers is exact too (below 2^24), so the two are
// equal.
struct IntLine {
    uint32_t dpos, dneg;   // max(d, 0), max(-d, 0) per channel, packed bytes
    int e0d;               // E0 . d
    float r;               // 1 / |d|^2 (0 for equal endpoints)
    bool flat;
};

__device__ __forceinline__ IntLine int_line(const int E0[4], const int E1[4]) {
    IntLine l;
    l.dpos = 0; l.dneg = 0; l.e0d = 0;
    int dd = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int d = E1[c] - E0[c];
        l.dpos |= (uint32_t)(d > 0 ? d : 0) << (8 * c);
        l.dneg |= (uint32_t)(d < 0 ? -d : 0) << (8 * c);
        l.e0d += E0[c] * d;
        dd += d * d;
    }
    l.flat = dd == 0;
    l.r = l.flat ? 0.0f : __frcp_rn((float)dd);
    return l;
}

__device__ __forceinline__ float int_weight(uint32_t t, uint32_t dpos, uint32_t dneg, int e0d, float r) {
    const int x = (int)__dp4a(t, dpos, 0u) - (int)__dp4a(t, dneg, 0u) - e0d;
    return fminf(fmaxf(__fmul_rn((float)x, r), 0.0f), 1.0f);
}

// Grid weights (value-order indices q) of a two-partition candidate: texel
// weights on the texel's own partition (integer projections for UNORM input,
// equal to the FP32 ones there; on GB300 this trims the normal-map
// candidates by a few per cent); 4x4 rounds them directly, 6x6 keeps them in
// `tws` ([texel][thread] floats) and samples the shader's 2x2 taps.
// Each partition's values are held in named registers and chosen with the
// texel's partition bit (an array indexed by it would live in local memory).
struct PartLine {
    float f0, f1, f2, f3;   // decoded low endpoint
    float d0, d1, d2, d3;   // high - low
    float r;                // 1 / |d|^2 (0 for a flat partition)
    bool flat;
};

__device__ __forceinline__ PartLine part_line(const int E0[4], const int E1[4]) {
    PartLine l;
    l.f0 = (float)E0[0]; l.f1 = (float)E0[1]; l.f2 = (float)E0[2]; l.f3 = (float)E0[3];
    l.d0 = (float)(E1[0] - E0[0]); l.d1 = (float)(E1[1] - E0[1]);
    l.d2 = (float)(E1[2] - E0[2]); l.d3 = (float)(E1[3] - E0[3]);
    const float dd = dot4(l.d0, l.d1, l.d2, l.d3, l.d0, l.d1, l.d2, l.d3);
    l.flat = dd == 0.0f;
    l.r = l.flat ? 0.0f : __frcp_rn(dd);
    return l;
}

__device__ __forceinline__ float part_weight_sel(const float4 t, bool p1, const PartLine& a, const PartLine& b) {
    const bool flat = p1 ? b.flat : a.flat;
    const float x = dot4(__fsub_rn(t.x, p1 ? b.f0 : a.f0), __fsub_rn(t.y, p1 ? b.f1 : a.f1),
                         __fsub_rn(t.z, p1 ? b.f2 : a.f2), __fsub_rn(t.w, p1 ? b.f3 : a.f3),
                         p1 ? b.d0 : a.d0, p1 ? b.d1 : a.d1, p1 ? b.d2 : a.d2, p1 ? b.d3 : a.d3);
    const float w = fminf(fmaxf(__fmul_rn(x, p1 ? b.r : a.r), 0.0f), 1.0f);
    return flat ? 0.0f : w;
}

template <int DIM, bool SRGB, class S, class TW>
__device__ __forceinline__ void two_partition_weights(const S& st, const uint32_t (&tw)[DIM * DIM], uint64_t sel1,
                                                      const int E0[2][4], const int E1[2][4], float R, TW& tws,
                                                      uint32_t (&q)[16]) {
    // texel weight k: integer projections for UNORM input, FP32 for sRGB
    auto weight = [&](int k, bool p1, const auto& la, const auto& lb) -> float {
        if constexpr (SRGB) {
            return part_weight_sel(st.get(k), p1, la, lb);
        } else {
            const float w = int_weight(tw[k], p1 ? lb.dpos : la.dpos, p1 ? lb.dneg : la.dneg, p1 ? lb.e0d : la.e0d,
                                       p1 ? lb.r : la.r);
            return (p1 ? lb.flat : la.flat) ? 0.0f : w;
        }
    };
    using Line = typename std::conditional<SRGB, PartLine, IntLine>::type;
    Line la, lb;
    if constexpr (SRGB) {
        la = part_line(E0[0], E1[0]);
        lb = part_line(E0[1], E1[1]);
    } else {
        la = int_line(E0[0], E1[0]);
        lb = int_line(E0[1], E1[1]);
    }
    if constexpr (DIM == 4) {
#pragma unroll kPartTexelUnroll<DIM>
        for (int k = 0; k < 16; ++k) {
            const float w = weight(k, (sel1 >> k) & 1, la, lb);
            const uint32_t v = rint_u32(__fmul_rn(w, R));
            q[k] = v < (uint32_t)R ? v : (uint32_t)R;
        }
    } else {
#pragma unroll kPartTexelUnroll<DIM>
        for (int k = 0; k < 36; ++k) tws.put(k, weight(k, (sel1 >> k) & 1, la, lb));
#pragma unroll
        for (int g = 0; g < 16; ++g) {
            const int i0 = grid_tap0(g);
            float w00, w01, w10, w11;
            grid_weights(g, w00, w01, w10, w11);
            const float w = __fmaf_rn(tws.get(i0 + 7), w11,
                                      __fmaf_rn(tws.get(i0 + 6), w10,
                                                __fmaf_rn(tws.get(i0 + 1), w01, __fmul_rn(tws.get(i0), w00))));
            const uint32_t v = rint_u32(__fmul_rn(w, R));
            q[g] = v < (uint32_t)R ? v : (uint32_t)R;
        }
    }
}

// Two partitions sharing CEM 8/12, 4x4 weight grid of range wq, endpoint
// range cq: mode [10:0], partition count - 1 = 1 at [12:11], index [22:13],
// CEM field [28:23] = CEM << 2, endpoint ISE from bit 29, weight ISE
// bit-reversed from bit 127.
template <bool ALPHA>
__device__ __forceinline__ uint4 assemble_two_partitions(int wq, int cq, int seed,
                                                         const uint32_t (&ev)[ALPHA ? 16 : 12],
                                                         const uint32_t (&sw)[16], const SearchSmem& sm) {
    const Bits128 ep = ise_encode_endpoints<ALPHA ? 16 : 12>(cq, ev, sm.trits, sm.quints);
    const Bits128 wt = ise_encode_weights<16, kQuant3, kQuant16>(wq, sw, sm.trits, sm.quints);
    const uint64_t head = (uint64_t)blockmode_4x4_grid(wq) | (1ull << 11) | ((uint64_t)(seed & 0x3FF) << 13) |
                          ((uint64_t)(ALPHA ? 12u : 8u) << 25);
    const uint64_t lo = head | (ep.lo << 29) | __brevll(wt.hi);
    const uint64_t hi = (ep.lo >> 35) | (ep.hi << 29) | __brevll(wt.lo);
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// Two-partition candidates of one block; returns `best` unless one decodes
// with less error than best_err (which it then lowers).
template <int DIM, bool ALPHA, bool SRGB, class S, class TW>
__device__ __forceinline__ uint4 two_partition_block(const S& st, const uint32_t (&tw)[DIM * DIM], uint32_t t2,
                                                     const uint32_t qa[4], const uint32_t qb[4], uint32_t& best_err,
                                                     uint4 best, const SearchSmem& sm, const PartSmem& pm,
                                                     TW& tws) {
    constexpr int N = DIM * DIM;
    constexpr uint64_t kFull = (N == 64) ? ~0ull : ((1ull << N) - 1);
    constexpr uint64_t kPatternBits = (1ull << 54) - 1;
    // the ideal split along the kept fit
    const float d0 = (float)((int)qb[0] - (int)qa[0]), d1 = (float)((int)qb[1] - (int)qa[1]);
    const float d2 = (float)((int)qb[2] - (int)qa[2]), d3 = (float)((int)qb[3] - (int)qa[3]);
    const float dd = dot4(d0, d1, d2, d3, d0, d1, d2, d3);
    if (dd == 0.0f) return best;
    const float f0 = (float)qa[0], f1 = (float)qa[1], f2 = (float)qa[2], f3 = (float)qa[3];
    uint64_t ideal = 0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        const float x = dot4(__fsub_rn(t.x, f0), __fsub_rn(t.y, f1), __fsub_rn(t.z, f2), __fsub_rn(t.w, f3),
                             d0, d1, d2, d3);
        if (__fadd_rn(x, x) > dd) ideal |= 1ull << k;
    }
    if (ideal == 0 || ideal == kFull) return best;
    // the best-matching partition pattern
    int best_m = N + 1;
    uint64_t sel1;
    int seed;
    if constexpr (DIM == 4) {
        const uint32_t ideal32 = (uint32_t)ideal;
        uint32_t pick = 0;
#pragma unroll 4
        for (int i = 0; i < pm.nclasses; ++i) {
            const uint32_t e = pm.classes.c4[i];
            int m = __popc((e & 0xFFFFu) ^ ideal32);
            m = (N - m < m) ? N - m : m;
            if (m < best_m) { best_m = m; pick = e; }
        }
        sel1 = pick & 0xFFFFu;
        seed = (int)(pick >> 16);
    } else {
        uint64_t pick = 0;
#pragma unroll 4
        for (int i = 0; i < pm.nclasses; ++i) {
            const uint64_t e = pm.classes.c6[i];
            int m = __popcll((e & kPatternBits) ^ ideal);
            m = (N - m < m) ? N - m : m;
            if (m < best_m) { best_m = m; pick = e; }
        }
        sel1 = pick & kPatternBits;
        seed = (int)(pick >> 54);
    }
    const uint64_t sel0 = kFull & ~sel1;
    // one fit per partition (one copy of the code: the loop is not unrolled)
    uint32_t a0[4], a1[4], b0[4], b1[4];
#pragma unroll 1
    for (int p = 0; p < 2; ++p) {
        uint32_t lo[4], hi[4];
        fit_partition<N, ALPHA>(st, p ? sel1 : sel0, lo, hi);
        if (p) {
#pragma unroll
            for (int c = 0; c < 4; ++c) { b0[c] = lo[c]; b1[c] = hi[c]; }
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) { a0[c] = lo[c]; a1[c] = hi[c]; }
        }
    }
    // every legal weight range, then one more pass over the best to assemble it
    int found = -1;
    uint4 out = best;
    int sym0[2][4], sym1[2][4], E0[2][4], E1[2][4], W[16];
    uint32_t q[16];
#pragma unroll 1
    for (int it = kQuant3; it <= kQuant32 + 1; ++it) {
        const bool final_pass = it > kQuant32;
        if (final_pass && found < 0) break;
        const int wq = final_pass ? found : it;
        const int cq = pm.cq[wq];
        if (cq < 0) continue;
        snap_two<ALPHA>(pm.slot[wq], a0, a1, b0, b1, pm, sym0, sym1, E0, E1);
        two_partition_weights<DIM, SRGB>(st, tw, sel1, E0, E1, sm.wmax[wq], tws, q);
        if (!final_pass) {
#pragma unroll
            for (int g = 0; g < 16; ++g) W[g] = sm.wval[wq][q[g]];
            const uint32_t err = eval_two_partitions<DIM, ALPHA, SRGB>(tw, t2, sel1, E0, E1, W);
            if (err < best_err) { best_err = err; found = wq; }
            continue;
        }
        constexpr int NV = ALPHA ? 8 : 6;
        uint32_t ev[2 * NV];
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int c = 0; c < NV / 2; ++c) {
                ev[p * NV + 2 * c] = (uint32_t)sym0[p][c];
                ev[p * NV + 2 * c + 1] = (uint32_t)sym1[p][c];
            }
        uint32_t sw[16];
#pragma unroll
        for (int g = 0; g < 16; ++g) sw[g] = sm.scramble[wq][q[g]];
        out = assemble_two_partitions<ALPHA>(wq, cq, seed, ev, sw, sm);
        break;
    }
    return out;
}

}  // namespace astc
