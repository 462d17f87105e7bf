// astc_pipeline_partition3.cuh -- three-partition candidates of the FP32
// encoder's ASTC_QUALITY_THREE_PARTITIONS mode (RGB blocks: a block carries at
// most 18 colour endpoint integers, three RGBA partitions would need 24).
// The reference has only a commented-out layout stub for multi-partition
// blocks (ASTC_Encode.hlsl:422-431).
//
// Per block, after the single-, dual-plane and two-partition candidates:
//  1. integer labels on the texels rounded to bytes: k0 = the texel farthest
//     from texel 0, k1 the one farthest from k0, k2 the one farthest from
//     both (first on ties); each texel takes the nearest (lowest on ties);
//  2. of the three-partition pattern classes (one per distinct split of the
//     block into three non-empty sets), the four with the fewest texels
//     disagreeing with the labels under the best label-to-partition
//     matching (then the smaller index);
//  3. for each, every partition fitted on its own (fit_partition) and every
//     legal weight range scored with each texel decoded on its partition.
// The oracle's three_partitions follows the same steps.
#pragma once
#include "astc_pipeline_partition.cuh"

namespace astc {

// Per-CTA copies of the three-partition endpoint tables (shared memory).
struct Part3Smem {
    uint16_t color[8][256];
    int8_t cq[12];      // weight range -> endpoint range (-1: illegal)
    int8_t slot[12];
};

// The class tables, in index order: 4x4 m1 | (m2 << 16) | (index << 32);
// 6x6 A = m1 | (index << 54), B = m2 (m1 / m2: partitions 1 / 2).
struct Partition3Classes {
    uint64_t c4[kPartition3Classes4x4Count];
    uint64_t c6a[kPartition3Classes6x6Count];
    uint64_t c6b[kPartition3Classes6x6Count];
};

// Squared distance of two packed RGB byte words (alpha bytes zero).
__device__ __forceinline__ uint32_t byte_dist(uint32_t a, uint32_t b) {
    const uint32_t d = __vabsdiffu4(a, b);
    return __dp4a(d, d, 0u);
}

// Step 1: label masks L0, L1, L2 of the block's target words (RGB bytes);
// false if a label is left empty.
template <int N>
__device__ __forceinline__ bool three_labels(const uint32_t (&tw)[N], uint64_t& L0, uint64_t& L1, uint64_t& L2) {
    uint32_t a0 = tw[0], a1 = tw[0], a2 = tw[0];
    int far = -1;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const int d = (int)byte_dist(tw[k], tw[0]);
        if (d > far) { far = d; a0 = tw[k]; }
    }
    far = -1;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const int d = (int)byte_dist(tw[k], a0);
        if (d > far) { far = d; a1 = tw[k]; }
    }
    far = -1;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const int d = (int)min(byte_dist(tw[k], a0), byte_dist(tw[k], a1));
        if (d > far) { far = d; a2 = tw[k]; }
    }
    L0 = L1 = L2 = 0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const uint32_t da = byte_dist(tw[k], a0), db = byte_dist(tw[k], a1), dc = byte_dist(tw[k], a2);
        const uint64_t bit = 1ull << k;
        if (da <= db && da <= dc) L0 |= bit;
        else if (db <= dc) L1 |= bit;
        else L2 |= bit;
    }
    return L0 && L1 && L2;
}

// Step 2's count: texels of class (m1, m2) that disagree with the labels
// under the best of the six label-to-partition matchings.  c0/c1/c2: popc of
// L0/L1/L2.
__device__ __forceinline__ int three_mismatch(uint64_t L0, uint64_t L1, int c0, int c1, int c2, uint64_t m1,
                                              uint64_t m2, int n) {
    const int a1 = __popcll(L0 & m1), a2 = __popcll(L0 & m2), a0 = c0 - a1 - a2;
    const int b1 = __popcll(L1 & m1), b2 = __popcll(L1 & m2), b0 = c1 - b1 - b2;
    const int p1 = __popcll(m1), p2 = __popcll(m2);
    const int g1 = p1 - a1 - b1, g2 = p2 - a2 - b2, g0 = c2 - g1 - g2;
    int most = a0 + b1 + g2;
    most = max(most, a0 + b2 + g1);
    most = max(most, a1 + b0 + g2);
    most = max(most, a1 + b2 + g0);
    most = max(most, a2 + b0 + g1);
    most = max(most, a2 + b1 + g0);
    return n - most;
}

template <int DIM>
__device__ __forceinline__ void three_class(const Partition3Classes& t, int i, uint64_t& m1, uint64_t& m2, int& seed) {
    if constexpr (DIM == 4) {
        const uint64_t v = t.c4[i];
        m1 = v & 0xFFFFu;
        m2 = (v >> 16) & 0xFFFFu;
        seed = (int)(v >> 32);
    } else {
        const uint64_t a = t.c6a[i];
        m1 = a & ((1ull << 36) - 1);
        m2 = t.c6b[i];
        seed = (int)(a >> 54);
    }
}

// The squared error of a three-partition RGB decode (texel k in partition 1
// when bit k of m1 is set, 2 when bit k of m2 is, else 0).
template <int DIM, bool SRGB>
__device__ __forceinline__ uint32_t eval_three_partitions(const uint32_t (&tw)[DIM * DIM], uint32_t t2, uint64_t m1,
                                                          uint64_t m2, const int E0[3][4], const int E1[3][4],
                                                          const int (&W)[16]) {
    int base[3][3], delta[3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
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
        const bool q1 = (m1 >> k) & 1, q2 = (m2 >> k) & 1;
        uint32_t v[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int b = q1 ? base[1][c] : (q2 ? base[2][c] : base[0][c]);
            const int d = q1 ? delta[1][c] : (q2 ? delta[2][c] : delta[0][c]);
            v[c] = (uint32_t)(b + d * w);
        }
        uint32_t dec = __byte_perm(v[0], v[1], 0x3362u);
        dec = __byte_perm(dec, v[2], 0x3610u);
        dd = __dp4a(dec, dec, dd);
        dt = __dp4a(dec, tw[k], dt);
    }
    return dd - 2u * dt + t2;
}

// Texel weight on its own partition's line (FP32, as the oracle), 0 on a
// flat partition.
__device__ __forceinline__ float part3_weight(const float4 t, bool q1, bool q2, const PartLine& a, const PartLine& b,
                                              const PartLine& c) {
    const PartLine& l0 = q2 ? c : a;
    const bool flat = q1 ? b.flat : l0.flat;
    const float x = dot4(__fsub_rn(t.x, q1 ? b.f0 : l0.f0), __fsub_rn(t.y, q1 ? b.f1 : l0.f1),
                         __fsub_rn(t.z, q1 ? b.f2 : l0.f2), __fsub_rn(t.w, q1 ? b.f3 : l0.f3),
                         q1 ? b.d0 : l0.d0, q1 ? b.d1 : l0.d1, q1 ? b.d2 : l0.d2, q1 ? b.d3 : l0.d3);
    const float w = fminf(fmaxf(__fmul_rn(x, q1 ? b.r : l0.r), 0.0f), 1.0f);
    return flat ? 0.0f : w;
}

// Grid weights (value-order indices q) of a three-partition candidate: 4x4
// rounds the texel weights, 6x6 keeps them in `tws` ([texel][thread] floats)
// and samples the shader's 2x2 taps.
template <int DIM, class S, class TW>
__device__ __forceinline__ void three_partition_weights(const S& st, uint64_t m1, uint64_t m2, const int E0[3][4],
                                                        const int E1[3][4], float R, TW& tws, uint32_t (&q)[16]) {
    const PartLine la = part_line(E0[0], E1[0]), lb = part_line(E0[1], E1[1]), lc = part_line(E0[2], E1[2]);
    if constexpr (DIM == 4) {
#pragma unroll kPartTexelUnroll<DIM>
        for (int k = 0; k < 16; ++k) {
            const float w = part3_weight(st.get(k), (m1 >> k) & 1, (m2 >> k) & 1, la, lb, lc);
            const uint32_t v = rint_u32(__fmul_rn(w, R));
            q[k] = v < (uint32_t)R ? v : (uint32_t)R;
        }
    } else {
#pragma unroll kPartTexelUnroll<DIM>
        for (int k = 0; k < 36; ++k) tws.put(k, part3_weight(st.get(k), (m1 >> k) & 1, (m2 >> k) & 1, la, lb, lc));
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

// Three partitions sharing CEM 8, 4x4 weight grid of range wq, endpoint range
// cq: mode [10:0], partition count - 1 = 2 at [12:11], index [22:13], CEM
// field [28:23] = 8 << 2, endpoint ISE (18 values, partition 0's first) from
// bit 29, weight ISE bit-reversed from bit 127.
__device__ __forceinline__ uint4 assemble_three_partitions(int wq, int cq, int seed, const uint32_t (&ev)[18],
                                                           const uint32_t (&sw)[16], const SearchSmem& sm) {
    const Bits128 ep = ise_encode_endpoints<18>(cq, ev, sm.trits, sm.quints);
    const Bits128 wt = ise_encode_weights<16, kQuant3, kQuant8>(wq, sw, sm.trits, sm.quints);
    const uint64_t head = (uint64_t)blockmode_4x4_grid(wq) | (2ull << 11) | ((uint64_t)(seed & 0x3FF) << 13) |
                          (8ull << 25);
    const uint64_t lo = head | (ep.lo << 29) | __brevll(wt.hi);
    const uint64_t hi = (ep.lo >> 35) | (ep.hi << 29) | __brevll(wt.lo);
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// Three-partition candidates of one RGB block; returns `best` unless one
// decodes with less error than best_err (which it then lowers).
template <int DIM, bool SRGB, class S, class TW>
__device__ __forceinline__ uint4 three_partition_block(const S& st, const uint32_t (&tw)[DIM * DIM], uint32_t t2,
                                                       uint32_t& best_err, uint4 best, const SearchSmem& sm,
                                                       const Part3Smem& p3, const Partition3Classes& cls, TW& tws) {
    constexpr int N = DIM * DIM;
    constexpr int NCLS = DIM == 4 ? kPartition3Classes4x4Count : kPartition3Classes6x6Count;
    constexpr uint64_t kFull = (1ull << N) - 1;
    uint64_t L0, L1, L2;
    if (!three_labels<N>(tw, L0, L1, L2)) return best;
    const int c0 = __popcll(L0), c1 = __popcll(L1), c2 = __popcll(L2);
    // the four best-matching classes: keys (mismatch << 16) | class, ascending
    uint32_t k0 = 0xFFFFFFFFu, k1 = 0xFFFFFFFFu, k2 = 0xFFFFFFFFu, k3 = 0xFFFFFFFFu;
#pragma unroll 4
    for (int i = 0; i < NCLS; ++i) {
        uint64_t m1, m2;
        int seed;
        three_class<DIM>(cls, i, m1, m2, seed);
        uint32_t k = ((uint32_t)three_mismatch(L0, L1, c0, c1, c2, m1, m2, N) << 16) | (uint32_t)i;
        if (k < k3) {
            k3 = k;
            if (k3 < k2) { const uint32_t t = k2; k2 = k3; k3 = t; }
            if (k2 < k1) { const uint32_t t = k1; k1 = k2; k2 = t; }
            if (k1 < k0) { const uint32_t t = k0; k0 = k1; k1 = t; }
        }
    }
    // each class's fits and every legal weight range; then one more pass over
    // the best (class, range) to assemble it
    int found_r = -1, found_wq = -1;
    uint4 out = best;
#pragma unroll 1
    for (int it = 0; it <= 4; ++it) {
        const bool final_pass = it == 4;
        if (final_pass && found_r < 0) break;
        const int r = final_pass ? found_r : it;
        const uint32_t key = r == 0 ? k0 : r == 1 ? k1 : r == 2 ? k2 : k3;
        if (key == 0xFFFFFFFFu) break;
        uint64_t m1, m2;
        int seed;
        three_class<DIM>(cls, (int)(key & 0xFFFFu), m1, m2, seed);
        const uint64_t m0 = kFull & ~(m1 | m2);
        uint32_t lo[3][4], hi[3][4];
#pragma unroll 1
        for (int p = 0; p < 3; ++p) {
            uint32_t a[4], b[4];
            fit_partition<N, false>(st, p == 0 ? m0 : p == 1 ? m1 : m2, a, b);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                lo[0][c] = p == 0 ? a[c] : lo[0][c]; hi[0][c] = p == 0 ? b[c] : hi[0][c];
                lo[1][c] = p == 1 ? a[c] : lo[1][c]; hi[1][c] = p == 1 ? b[c] : hi[1][c];
                lo[2][c] = p == 2 ? a[c] : lo[2][c]; hi[2][c] = p == 2 ? b[c] : hi[2][c];
            }
        }
#pragma unroll 1
        for (int wq = kQuant3; wq <= kQuant32; ++wq) {
            if (final_pass && wq != found_wq) continue;
            const int cq = p3.cq[wq];
            if (cq < 0) continue;
            const int slot = p3.slot[wq];
            int sym0[3][4], sym1[3][4], E0[3][4], E1[3][4];
#pragma unroll
            for (int p = 0; p < 3; ++p) {
#pragma unroll
                for (int c = 0; c < 4; ++c) { sym0[p][c] = 0; sym1[p][c] = 0; E0[p][c] = 255; E1[p][c] = 255; }
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const uint32_t x = p3.color[slot][lo[p][c]], y = p3.color[slot][hi[p][c]];
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
            uint32_t q[16];
            three_partition_weights<DIM>(st, m1, m2, E0, E1, sm.wmax[wq], tws, q);
            if (!final_pass) {
                int W[16];
#pragma unroll
                for (int g = 0; g < 16; ++g) W[g] = sm.wval[wq][q[g]];
                const uint32_t err = eval_three_partitions<DIM, SRGB>(tw, t2, m1, m2, E0, E1, W);
                if (err < best_err) { best_err = err; found_r = r; found_wq = wq; }
                continue;
            }
            uint32_t ev[18];
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    ev[6 * p + 2 * c] = (uint32_t)sym0[p][c];
                    ev[6 * p + 2 * c + 1] = (uint32_t)sym1[p][c];
                }
            uint32_t sw[16];
#pragma unroll
            for (int g = 0; g < 16; ++g) sw[g] = sm.scramble[wq][q[g]];
            out = assemble_three_partitions(wq, cq, seed, ev, sw, sm);
            break;
        }
    }
    return out;
}

}  // namespace astc
