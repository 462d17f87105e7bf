// astc_block_common.cuh -- device helpers shared by the encode kernels:
// exact FP32 primitives of the pinned arithmetic model, texel fetch, texel
// stores (registers or shared memory), and the integer back end (weight
// scramble, trit ISE, endpoint packing, 128-bit block assembly).
//
// Reference: niepp/astc_encoder ASTC_Encode.hlsl (MainCS 553-582, encode_block
// 510-550, assemble_block 400-444, assemble_blockmode 446-473) and
// ASTC_IntegerSequenceEncoding.hlsl (encode_trits 142-176, bise_* 207-276).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "astc_srgb_table.h"
#include "astc_tables.h"

namespace astc {

// ---------------------------------------------------------------------------
// Launch parameters of one texture (or one texture range of a batch)
// ---------------------------------------------------------------------------
struct TextureView {
    const uint8_t* in;    // RGBA8
    size_t pitch;         // bytes per row
    int width, height, nbx;
    int vec_ok;           // 128-bit (4x4) / 64-bit (6x6) row loads allowed
    int clamp;            // ASTC_BORDER_CLAMP
    uint32_t row_mul;     // block row of block b: (b * row_mul) >> row_shift
    uint32_t row_shift;
};

// (row_mul, row_shift) for divisor d = nbx: with L = ceil(log2 d), m =
// ceil(2^(31+L) / d) < 2^32 and floor(b * m / 2^(31+L)) = floor(b / d) for
// every 0 <= b < 2^31 (Granlund and Montgomery, "Division by invariant
// integers using multiplication", 1994: m = (2^(31+L) + e) / d with 0 <= e <
// d adds less than b / 2^(31+L) < 1/d to b/d).  Textures hold at most 2^31
// blocks, so every block index qualifies.
inline void block_row_divisor(int d, uint32_t* mul, uint32_t* shift) {
    int L = 0;
    while ((1ull << L) < (unsigned long long)d) ++L;
    const unsigned long long p = 1ull << (31 + L);
    *mul = (uint32_t)((p + (unsigned long long)d - 1) / (unsigned long long)d);
    *shift = (uint32_t)(31 + L);
}

// block (bx, by) of block index b < 2^31
__device__ __forceinline__ void block_coords(const TextureView& t, long long b, int& bx, int& by) {
    const uint32_t ub = (uint32_t)b;
    by = (int)(((uint64_t)ub * t.row_mul) >> t.row_shift);
    bx = (int)(ub - (uint32_t)by * (uint32_t)t.nbx);
}

// ---------------------------------------------------------------------------
// exact FP32 primitives (the oracle's model)
// ---------------------------------------------------------------------------
// float of byte c of a packed RGBA8 texel: bits 0x4B0000cc = 2^23 + c, minus 2^23
__device__ __forceinline__ float byte_to_float(uint32_t px, int c) {
    const uint32_t bits = __byte_perm(px, 0x4B000000u, 0x7440u + (uint32_t)c);
    return __fsub_rn(__uint_as_float(bits), 8388608.0f);
}

// round-half-even of x in [0, 2^22] as an integer: adding 2^23 rounds to the
// nearest integer, ties to even, at unit spacing
__device__ __forceinline__ uint32_t rint_u32(float x) {
    return __float_as_uint(__fadd_rn(x, 8388608.0f)) - 0x4B000000u;
}

// dot(a, b) = a.x*b.x, then fused multiply-adds over y, z, w
__device__ __forceinline__ float dot4(float ax, float ay, float az, float aw, float bx, float by,
                                      float bz, float bw) {
    float d = __fmul_rn(ax, bx);
    d = __fmaf_rn(ay, by, d);
    d = __fmaf_rn(az, bz, d);
    d = __fmaf_rn(aw, bw, d);
    return d;
}

// sqrt_rn(d) < 1e-5f  <=>  d < kLenThreshold, for every float d (sqrt_rn is
// monotone and correctly rounded; 0x2EDBE6FD is the smallest float whose
// correctly rounded square root is >= 1e-5f).  The length tests of
// eigen_vector (ASTC_Encode.hlsl:100) and calculate_normal_weights (323)
// therefore need no square root.
#define ASTC_LEN_THRESHOLD_BITS 0x2EDBE6FDu

__device__ __forceinline__ bool shorter_than_small_value(float dot_self) {
    return dot_self < __uint_as_float(ASTC_LEN_THRESHOLD_BITS);
}

// v * (1 / sqrt(dot(v, v))) with correctly rounded sqrt and reciprocal
__device__ __forceinline__ float rnorm_from_dot(float d) {
    return __frcp_rn(__fsqrt_rn(d));
}

// ---------------------------------------------------------------------------
// texel decode: UNORM8 value x255 is the code itself; sRGB goes through the
// 256-entry table (float(linear) * 255); normal maps force b = a = 255
// ---------------------------------------------------------------------------
template <bool SRGB, bool NORMAL>
__device__ __forceinline__ float4 decode_texel(uint32_t px, const float* lut) {
    float4 t;
    if (SRGB) {
        t.x = lut[px & 0xFFu];
        t.y = lut[(px >> 8) & 0xFFu];
        t.z = NORMAL ? 255.0f : lut[(px >> 16) & 0xFFu];
    } else {
        t.x = byte_to_float(px, 0);
        t.y = byte_to_float(px, 1);
        t.z = NORMAL ? 255.0f : byte_to_float(px, 2);
    }
    t.w = NORMAL ? 255.0f : byte_to_float(px, 3);
    return t;
}

// ---------------------------------------------------------------------------
// texel fetch of one block (MainCS 561-580): zero or clamp outside the image
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void load_block_packed(const TextureView& p, int bx, int by,
                                                  uint32_t (&px)[DIM * DIM]) {
    const int x0 = bx * DIM, y0 = by * DIM;
    if (x0 + DIM <= p.width && y0 + DIM <= p.height) {
        const uint8_t* row = p.in + (size_t)y0 * p.pitch + (size_t)x0 * 4;
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
            bool done = false;
            if constexpr (DIM == 4) {
                if (p.vec_ok) {
                    const uint4 v = __ldg(reinterpret_cast<const uint4*>(row));
                    px[r * 4 + 0] = v.x; px[r * 4 + 1] = v.y; px[r * 4 + 2] = v.z; px[r * 4 + 3] = v.w;
                    done = true;
                }
            } else {
                if (p.vec_ok) {
                    const uint2* q = reinterpret_cast<const uint2*>(row);
                    const uint2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
                    px[r * 6 + 0] = a.x; px[r * 6 + 1] = a.y; px[r * 6 + 2] = b.x;
                    px[r * 6 + 3] = b.y; px[r * 6 + 4] = c.x; px[r * 6 + 5] = c.y;
                    done = true;
                }
            }
            if (!done) {
                const uint32_t* q = reinterpret_cast<const uint32_t*>(row);
#pragma unroll
                for (int x = 0; x < DIM; ++x) px[r * DIM + x] = __ldg(q + x);
            }
            row += p.pitch;
        }
    } else {
#pragma unroll
        for (int k = 0; k < DIM * DIM; ++k) {
            int x = x0 + k % DIM, y = y0 + k / DIM;
            const bool inside = x < p.width && y < p.height;
            uint32_t v = 0;                                   // D3D11 OOB Load -> 0
            if (inside || p.clamp) {
                x = x < p.width ? x : p.width - 1;
                y = y < p.height ? y : p.height - 1;
                v = __ldg(reinterpret_cast<const uint32_t*>(p.in + (size_t)y * p.pitch) + x);
            }
            px[k] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// texel stores: where the decoded FP32 texels of one block live
// ---------------------------------------------------------------------------
// registers / shared memory / registers with the count capped near 168 (three
// 128-thread CTAs per SM) so the compiler trades a little spilling for warps;
// kStoreCoop is the cooperative mapping (four lanes per block, texels in a
// shared-memory tile; astc_encode_coop.cu)
enum TexelStore : int { kStoreRegisters = 0, kStoreShared = 1, kStoreRegistersCapped = 2, kStoreCoop = 3 };

template <int N>
struct RegTexels {
    float4 t[N];
    __device__ __forceinline__ void put(int k, float4 v) { t[k] = v; }
    __device__ __forceinline__ float4 get(int k) const { return t[k]; }
};

// [k][thread] layout: consecutive threads touch consecutive 16-byte words
template <int N>
struct SharedTexels {
    float4* base;
    int stride;
    __device__ __forceinline__ void put(int k, float4 v) { base[k * stride] = v; }
    __device__ __forceinline__ float4 get(int k) const { return base[k * stride]; }
};

// ---------------------------------------------------------------------------
// integer back end: weight scramble, trit ISE, endpoints, block assembly
// ---------------------------------------------------------------------------
struct TritPack { uint8_t v[256]; };
constexpr TritPack make_trit_pack() {
    TritPack p{};
    const IseTables t = make_ise_tables();
    for (int i = 0; i < 243; ++i) p.v[i] = t.trit_pack[i];
    return p;
}

struct SrgbBits { uint32_t v[256]; };
constexpr SrgbBits make_srgb_bits() {
    SrgbBits s{};
    for (int i = 0; i < 256; ++i) s.v[i] = kSrgbX255Bits[i];
    return s;
}

// Programmatic dependent launch (launch_pdl): wait until the previous kernel
// on the stream has completed with its writes visible (called after the
// constant-table set-up, before the first global load or store), then allow
// the next kernel to be launched.  Allowing it only after the wait keeps at
// most one launched-but-waiting kernel behind a running one: allowed before
// the wait, grids smaller than the GPU chained many waiting kernels whose CTAs
// held SM slots and crowded the next kernel onto fewer SMs (4x4 512x512
// two-partition launches 11% slower).
__device__ __forceinline__ void pdl_allow_next() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait_prior() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Per-CTA copies of the constant tables (trit packing, sRGB texel values).
template <bool SRGB>
__device__ __forceinline__ void load_cta_tables(const TritPack& tp, const SrgbBits& sb, uint8_t* s_trits,
                                                float* s_lut) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        s_trits[i] = tp.v[i];
        if (SRGB) s_lut[i] = __uint_as_float(sb.v[i]);
    }
}

// q0/q1: rounded endpoints (RGBA), qw: 16 quantised weights (0..R).
template <bool ALPHA>
__device__ __forceinline__ uint4 assemble_block(const uint32_t q0[4], const uint32_t q1[4],
                                                const uint32_t qw[16], const uint8_t* trits) {
    // scramble (ASTC_Encode.hlsl:498-502) + trits ISE of 16 weights (ISE 142-176, 243-256):
    // each group of five symbols packs into 5 B + 8 bits -- m0, T[1:0], m1, T[3:2], m2,
    // T[4], m3, T[6:5], m4, T[7] -- assembled in 32 bits (the widest group is 18 bits),
    // T's fields masked in place and shifted once each
    constexpr int WQ = ALPHA ? kQuant6 : kQuant12;
    constexpr int B = ALPHA ? 1 : 2;
    constexpr int GW = 5 * B + 8;
    constexpr uint32_t M = (1u << B) - 1u;
    constexpr uint32_t R = ALPHA ? 5u : 11u;
    constexpr uint64_t kScr = scramble_nibbles(WQ);
    uint32_t sym[20];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const uint32_t q = qw[i];
        sym[i] = (R < 8 ? ((uint32_t)kScr >> (4 * q)) : (uint32_t)(kScr >> (4 * q))) & 0xFu;
    }
#pragma unroll
    for (int i = 16; i < 20; ++i) sym[i] = 0u;
    uint64_t ws = 0;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        const uint32_t* v = sym + 5 * g;
        const uint32_t T = trits[(v[0] >> B) + 3u * (v[1] >> B) + 9u * (v[2] >> B) + 27u * (v[3] >> B) +
                                 81u * (v[4] >> B)];
        const uint32_t grp = (v[0] & M) | ((T & 0x3u) << B) | ((v[1] & M) << (B + 2)) | ((T & 0xCu) << (2 * B)) |
                             ((v[2] & M) << (2 * B + 4)) | ((T & 0x10u) << (3 * B)) | ((v[3] & M) << (3 * B + 5)) |
                             ((T & 0x60u) << (4 * B)) | ((v[4] & M) << (4 * B + 7)) | ((T & 0x80u) << (5 * B));
        ws |= (uint64_t)grp << (g * GW);
    }
    // endpoints in QUANT_256: r0 r1 g0 g1 b0 b1 [a0 a1], 8 bits each (bise_endpoints)
    uint64_t ep = (uint64_t)q0[0] | ((uint64_t)q1[0] << 8) | ((uint64_t)q0[1] << 16) |
                  ((uint64_t)q1[1] << 24) | ((uint64_t)q0[2] << 32) | ((uint64_t)q1[2] << 40);
    if (ALPHA) ep |= ((uint64_t)q0[3] << 48) | ((uint64_t)q1[3] << 56);
    // mode [10:0], CEM [16:13], endpoints from bit 17, weights bit-reversed from bit 127
    constexpr uint64_t kHead = (uint64_t)blockmode_4x4_grid(WQ) | ((uint64_t)(ALPHA ? 12u : 8u) << 13);
    const uint64_t lo = kHead | (ep << 17);
    const uint64_t hi = (ep >> 47) | __brevll(ws);
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// 6x6 -> 4x4 weight grid: grid point g samples the 2x2 texels from index
// i0(g) with weights 4/9, 2/9, 1/9 written as 0.444, 0.222, 0.111
// (idx_grids / wt_grids, ASTC_Encode.hlsl:268-304).
__device__ __forceinline__ int grid_tap0(int g) {
    const int gx = g & 3, gy = g >> 2;
    return (gy < 2 ? gy : gy + 1) * 6 + (gx < 2 ? gx : gx + 1);
}
__device__ __forceinline__ void grid_weights(int g, float& w00, float& w01, float& w10, float& w11) {
    const bool xl = ((g & 3) & 1) == 0, yl = ((g >> 2) & 1) == 0;
    w00 = (xl && yl) ? 0.444f : (xl || yl) ? 0.222f : 0.111f;
    w01 = (!xl && yl) ? 0.444f : (!xl || yl) ? 0.222f : 0.111f;
    w10 = (xl && !yl) ? 0.444f : (xl || !yl) ? 0.222f : 0.111f;
    w11 = (!xl && !yl) ? 0.444f : (!xl || !yl) ? 0.222f : 0.111f;
}

}  // namespace astc
