// astc_pipeline_search.cuh -- search mode of the FP32 encoder: the
// choose_best_quantmethod that the reference shader sketches but leaves out
// (niepp/astc_encoder ASTC_Encode.hlsl:524-526).
//
// After the endpoint fit (PCA, or the shader's unused
// max_accumulation_pixel_direction), a block is encoded in the shader's fixed
// mode and, besides, in every single-partition mode with a 4x4 weight grid:
// weight ranges QUANT_3..QUANT_32, each with the endpoint range the decoder
// derives from the bits left over (QUANT_256 down to QUANT_12).  A candidate
// snaps the rounded endpoints to the nearest representable values (darker
// one first, so the decoder neither swaps nor blue-contracts), projects the
// grid colours onto the decoded endpoints and rounds the weights to the
// range.  Every candidate is scored by the exact squared error of its spec
// decode against the texels rounded to bytes in the fit space (UNORM codes
// as they are, sRGB codes linearised x255 and rounded), in 32-bit integers,
// and the first candidate with the least error is kept.  Weight ranges that
// share an endpoint range share the endpoints and so the projections, which
// are computed once per endpoint range.  The oracle's search mode follows
// the same steps, so blocks are bit-identical to it.
#pragma once
#include <type_traits>

#include "astc_pipeline_fp32.cuh"
#include "astc_ise.h"

namespace astc {

// Decode steps the compiler may neither hoist nor merge across passes (a
// merged decode would keep the block's 4 floats per texel live next to the
// packed words): the byte_to_float permute and the sRGB table read.
__device__ __forceinline__ float byte_to_float_fresh(uint32_t px, int c) {
    uint32_t bits;
    asm volatile("prmt.b32 %0, %1, %2, %3;" : "=r"(bits) : "r"(px), "r"(0x4B000000u), "r"(0x7440u + (uint32_t)c));
    return __fsub_rn(__uint_as_float(bits), 8388608.0f);
}

__device__ __forceinline__ float lds_f32_volatile(const float* p) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}

// Texels re-decoded from their packed RGBA8 words on every read: 1 register
// per texel instead of 4, for the passes over the block.  Same values as
// decode_texel.
template <int N, bool SRGB, bool NORMAL>
struct PackedTexels {
    const uint32_t (&px)[N];
    const float* lut;
    __device__ __forceinline__ float4 get(int k) const {
        const uint32_t p = px[k];
        float4 t;
        if (SRGB) {
            t.x = lds_f32_volatile(lut + (p & 0xFFu));
            t.y = lds_f32_volatile(lut + ((p >> 8) & 0xFFu));
            t.z = NORMAL ? 255.0f : lds_f32_volatile(lut + ((p >> 16) & 0xFFu));
        } else {
            t.x = byte_to_float_fresh(p, 0);
            t.y = byte_to_float_fresh(p, 1);
            t.z = NORMAL ? 255.0f : byte_to_float_fresh(p, 2);
        }
        t.w = NORMAL ? 255.0f : byte_to_float_fresh(p, 3);
        return t;
    }
};

// Per-thread floats in a [k][thread] shared array.
template <int N>
struct SharedFloats {
    float* base;
    int stride;
    __device__ __forceinline__ void put(int k, float v) { base[k * stride] = v; }
    __device__ __forceinline__ float get(int k) const { return base[k * stride]; }
};

// Per-CTA copies of the search tables (shared memory).
struct SearchSmem {
    uint16_t color[8][256];      // this format's endpoint ranges below QUANT_256
    uint8_t wval[12][32];
    uint8_t scramble[12][32];
    uint8_t trits[256];
    uint8_t quints[128];
    int8_t cq[12];               // weight range -> endpoint range (-1: illegal)
    int8_t slot[12];             // weight range -> row of color (-1: QUANT_256)
    float wmax[12];              // weight range -> levels - 1
    float lut[256];              // sRGB code -> linear x255 (fit texels)
    uint8_t tbyte[256];          // sRGB code -> rint(linear x255) (scoring)
};

// ---------------------------------------------------------------------------
// general bounded integer sequence encoding (ISE) into a 128-bit field
// ---------------------------------------------------------------------------
// Single-partition block, 4x4 weight grid of range wq, endpoint range cq:
// mode [10:0], CEM [16:13], endpoint ISE from bit 17 up, weight ISE
// bit-reversed from bit 127 down.
template <bool ALPHA>
__device__ __forceinline__ uint4 assemble_search_block(int wq, int cq, const uint32_t (&ev)[ALPHA ? 8 : 6],
                                                       const uint32_t (&sw)[16], const SearchSmem& sm) {
    const Bits128 ep = ise_encode_endpoints<ALPHA ? 8 : 6>(cq, ev, sm.trits, sm.quints);
    const Bits128 wt = ise_encode_weights<16, kQuant3, kQuant32>(wq, sw, sm.trits, sm.quints);
    const uint64_t head = (uint64_t)blockmode_4x4_grid(wq) | ((uint64_t)(ALPHA ? 12u : 8u) << 13);
    const uint64_t lo = head | (ep.lo << 17) | __brevll(wt.hi);
    const uint64_t hi = (ep.lo >> 47) | (ep.hi << 17) | __brevll(wt.lo);
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// ---------------------------------------------------------------------------
// scoring
// ---------------------------------------------------------------------------
// The block's texels rounded to bytes in the fit space, packed r g b a:
// normal maps read blue and alpha as 255, sRGB codes go through tbyte, RGB
// blocks drop alpha (not scored).
template <bool ALPHA, bool NORMAL, bool SRGB>
__device__ __forceinline__ uint32_t target_word(uint32_t px, const uint8_t* tbyte) {
    uint32_t t = px;
    if (SRGB) {
        t = (uint32_t)tbyte[px & 0xFFu] | ((uint32_t)tbyte[(px >> 8) & 0xFFu] << 8) |
            ((uint32_t)tbyte[(px >> 16) & 0xFFu] << 16) | (px & 0xFF000000u);
    }
    if (NORMAL) t |= 0xFFFF0000u;
    return ALPHA ? t : (t & 0x00FFFFFFu);
}

// Squared error of the spec decode of endpoints E0/E1 (0..255) with grid
// weights W (0..64) against the target words tw.  A decoded UNORM8 channel
// is ((c0 * (64 - w) + c1 * w + 32) >> 6) >> 8 with c = e * 257 (linear) or
// (e << 8) | 0x80 (sRGB), i.e. byte 2 of 4 * (64 * c0 + 32) + 4 * (c1 - c0) * w.
// sum (dec - t)^2 = sum dec.dec - 2 sum dec.t + sum t.t over packed bytes
// (__dp4a), exact in 32-bit integers (at most 36 * 4 * 255^2); the last sum
// is per block (t2).
template <int DIM, bool ALPHA, bool SRGB>
struct BlockError {
    static __device__ __forceinline__ uint32_t target_sq(const uint32_t (&tw)[DIM * DIM]) {
        uint32_t t2 = 0;
#pragma unroll
        for (int k = 0; k < DIM * DIM; ++k) t2 = __dp4a(tw[k], tw[k], t2);
        return t2;
    }

    static __device__ __forceinline__ uint32_t eval(const uint32_t (&tw)[DIM * DIM], uint32_t t2,
                                                    const int E0[4], const int E1[4], const int (&W)[16]) {
        constexpr int NCH = ALPHA ? 4 : 3;
        int base[NCH], delta[NCH];
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const int c0 = SRGB ? ((E0[c] << 8) | 0x80) : E0[c] * 257;
            const int c1 = SRGB ? ((E1[c] << 8) | 0x80) : E1[c] * 257;
            base[c] = 4 * (64 * c0 + 32);
            delta[c] = 4 * (c1 - c0);
        }
        uint32_t dd = 0, dt = 0;
#pragma unroll
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
            uint32_t v[NCH];
#pragma unroll
            for (int c = 0; c < NCH; ++c) v[c] = (uint32_t)(base[c] + delta[c] * w);   // decoded in byte 2
            uint32_t dec = __byte_perm(v[0], v[1], 0x3362u);             // r, g, 0, 0
            dec = __byte_perm(dec, v[2], 0x3610u);                       // r, g, b, 0
            if constexpr (ALPHA) dec = __byte_perm(dec, v[3], 0x6210u);  // r, g, b, a
            dd = __dp4a(dec, dec, dd);
            dt = __dp4a(dec, tw[k], dt);
        }
        return dd - 2u * dt + t2;
    }
};

// Candidate endpoints for endpoint range cq: each rounded endpoint snapped to
// the nearest representable value (symbols sym, decoded values E), the
// darker (RGB sum) first.
template <bool ALPHA>
__device__ __forceinline__ void snap_endpoints(int cq, int slot, const uint32_t q0[4], const uint32_t q1[4],
                                               const SearchSmem& sm, int sym0[4], int sym1[4], int E0[4],
                                               int E1[4]) {
    constexpr int NCH = ALPHA ? 4 : 3;
#pragma unroll
    for (int c = 0; c < 4; ++c) { sym0[c] = 0; sym1[c] = 0; E0[c] = 255; E1[c] = 255; }
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
        if (cq == kQuant256) {
            sym0[c] = E0[c] = (int)q0[c];
            sym1[c] = E1[c] = (int)q1[c];
        } else {
            const uint32_t a = sm.color[slot][q0[c]], b = sm.color[slot][q1[c]];
            sym0[c] = (int)(a & 0xFFu); E0[c] = (int)(a >> 8);
            sym1[c] = (int)(b & 0xFFu); E1[c] = (int)(b >> 8);
        }
    }
    if (E1[0] + E1[1] + E1[2] < E0[0] + E0[1] + E0[2]) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int t = sym0[c]; sym0[c] = sym1[c]; sym1[c] = t;
            t = E0[c]; E0[c] = E1[c]; E1[c] = t;
        }
    }
}

// Projections of the grid colours on the decoded endpoints, clamped to [0, 1]
// (all 0 for equal endpoints).
template <class G>
__device__ __forceinline__ void project_weights(const G& s, const int E0[4], const int E1[4], float (&wf)[16]) {
    const float d0 = (float)(E1[0] - E0[0]), d1 = (float)(E1[1] - E0[1]);
    const float d2 = (float)(E1[2] - E0[2]), d3 = (float)(E1[3] - E0[3]);
    const float dd = dot4(d0, d1, d2, d3, d0, d1, d2, d3);
    if (dd == 0.0f) {
#pragma unroll
        for (int g = 0; g < 16; ++g) wf[g] = 0.0f;
        return;
    }
    const float r = __frcp_rn(dd);
    const float f0 = (float)E0[0], f1 = (float)E0[1], f2 = (float)E0[2], f3 = (float)E0[3];
#pragma unroll
    for (int g = 0; g < 16; ++g) {
        const float4 sg = s.get(g);
        const float x = dot4(__fsub_rn(sg.x, f0), __fsub_rn(sg.y, f1), __fsub_rn(sg.z, f2),
                             __fsub_rn(sg.w, f3), d0, d1, d2, d3);
        wf[g] = fminf(fmaxf(__fmul_rn(x, r), 0.0f), 1.0f);
    }
}

// The search over one block.  `fixed` is the fixed-mode block with rounded
// endpoints q0/q1 and weights qw; `grid` holds the 16 grid-point colours
// (grid_sample of the texels), in registers or shared memory; tw are the
// target words.
template <int DIM, bool ALPHA, bool SRGB, class G>
__device__ __forceinline__ uint4 search_block(const G& grid, const uint32_t (&tw)[DIM * DIM], const uint32_t q0[4],
                                              const uint32_t q1[4], const uint32_t qw[16], const uint4 fixed,
                                              const SearchSmem& sm, uint32_t* err_out = nullptr) {
    typedef BlockError<DIM, ALPHA, SRGB> Err;
    constexpr int WQ0 = ALPHA ? kQuant6 : kQuant12;
    int E0[4], E1[4], sym0[4], sym1[4], W[16];
#pragma unroll
    for (int c = 0; c < 4; ++c) { E0[c] = (int)q0[c]; E1[c] = (int)q1[c]; }
#pragma unroll
    for (int g = 0; g < 16; ++g) W[g] = sm.wval[WQ0][qw[g]];
    const uint32_t t2 = Err::target_sq(tw);
    uint32_t best = Err::eval(tw, t2, E0, E1, W);
    int best_wq = -1, prev_cq = -1;
    float wf[16];
#pragma unroll 1
    for (int wq = kQuant3; wq <= kQuant32; ++wq) {
        const int cq = sm.cq[wq];
        if (cq < 0) continue;
        if (cq != prev_cq) {                      // new endpoints: project again
            snap_endpoints<ALPHA>(cq, sm.slot[wq], q0, q1, sm, sym0, sym1, E0, E1);
            project_weights(grid, E0, E1, wf);
            prev_cq = cq;
        }
        const float R = sm.wmax[wq];
#pragma unroll
        for (int g = 0; g < 16; ++g) W[g] = sm.wval[wq][rint_u32(__fmul_rn(wf[g], R))];
        const uint32_t err = Err::eval(tw, t2, E0, E1, W);
        if (err < best) { best = err; best_wq = wq; }
    }
    if (err_out) *err_out = best;
    if (best_wq < 0) return fixed;
    const int cq = sm.cq[best_wq];
    snap_endpoints<ALPHA>(cq, sm.slot[best_wq], q0, q1, sm, sym0, sym1, E0, E1);
    project_weights(grid, E0, E1, wf);
    const float R = sm.wmax[best_wq];
    uint32_t ev[ALPHA ? 8 : 6];
#pragma unroll
    for (int c = 0; c < (ALPHA ? 4 : 3); ++c) { ev[2 * c] = (uint32_t)sym0[c]; ev[2 * c + 1] = (uint32_t)sym1[c]; }
    uint32_t sw[16];
#pragma unroll
    for (int g = 0; g < 16; ++g) sw[g] = sm.scramble[best_wq][rint_u32(__fmul_rn(wf[g], R))];
    return assemble_search_block<ALPHA>(best_wq, cq, ev, sw, sm);
}

}  // namespace astc
