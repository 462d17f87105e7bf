// astc_encode.cu -- sm_103a kernels for the ASTC LDR block encoder (FP32).
//
// One thread encodes one ASTC block, following the per-block pipeline of the
// reference compute shader (niepp/astc_encoder ASTC_Encode.hlsl):
//   texel fetch          MainCS 561-580     (128-bit / 64-bit row loads)
//   mean + covariance    139-162            (10 unique covariance terms)
//   power iteration      eigen_vector 93-106
//   endpoint fit         find_min_max 108-137, encode_color 233-245
//   weights              calculate_normal_weights 316-372, 6x6 taps 268-314,
//                        quantize_weight 256-260
//   scramble + ISE       weight_ise 491-508, bise_* (ISE.hlsl 207-276)
//   block assembly       assemble_block 400-444, assemble_blockmode 446-473
// but written for the GPU: texels stay packed RGBA8 in registers and are
// expanded to exact floats on use (byte_perm into a 2^23-biased float), the
// ISE of a fixed weight range is unrolled into 64-bit shifts, and the weight
// bit reversal is one __brevll.
//
// Floating point follows the FP32 oracle's model operation by operation:
// mad = fused (__fmaf_rn), dot(a,b) = a.x*b.x then fused over y, z, w,
// normalize(v) = v * (1/sqrt(dot(v,v))) with correctly rounded sqrt and
// reciprocal, x/N for constant N = x * fl(1/N), round = half-to-even.  The
// file is compiled with --fmad=false so nothing else is contracted; blocks
// are therefore bit-identical to the oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "astc_internal.h"
#include "astc_tables.h"

namespace astc {
namespace {

constexpr int kThreads = 128;

struct TritPack { uint8_t v[256]; };
constexpr TritPack make_trit_pack() {
    TritPack p{};
    const IseTables t = make_ise_tables();
    for (int i = 0; i < 243; ++i) p.v[i] = t.trit_pack[i];
    return p;
}

__constant__ TritPack c_trit_pack = make_trit_pack();
__constant__ float c_srgb_x255[256];

struct Launch {
    const uint8_t* in;
    size_t pitch;
    int width, height, nbx;
    long long nblocks;
    uint4* out;
    int vec_ok;     // row vector loads allowed (alignment of base and pitch)
    int clamp;      // ASTC_BORDER_CLAMP
};

// exact float of byte c of a packed RGBA8 texel: bits 0x4B0000cc = 2^23 + c
__device__ __forceinline__ float byte_to_float(uint32_t px, int c) {
    const uint32_t bits = __byte_perm(px, 0x4B000000u, 0x7440u + (uint32_t)c);
    return __fsub_rn(__uint_as_float(bits), 8388608.0f);
}

// round-half-even of x in [0, 2^22] as an integer: the add rounds to nearest
// even at unit spacing.
__device__ __forceinline__ uint32_t rint_u32(float x) {
    return __float_as_uint(__fadd_rn(x, 8388608.0f)) - 0x4B000000u;
}

__device__ __forceinline__ float dot4(const float a[4], const float b[4]) {
    float d = __fmul_rn(a[0], b[0]);
    d = __fmaf_rn(a[1], b[1], d);
    d = __fmaf_rn(a[2], b[2], d);
    d = __fmaf_rn(a[3], b[3], d);
    return d;
}

__device__ __forceinline__ void normalize4(float v[4]) {
    const float r = __frcp_rn(__fsqrt_rn(dot4(v, v)));
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __fmul_rn(v[i], r);
}

template <bool SRGB, bool NORMAL>
__device__ __forceinline__ float texel(uint32_t px, int c, const float* lut) {
    if (NORMAL && c >= 2) return 255.0f;                 // b = a = 1.0 (x255)
    if (SRGB && c < 3) return lut[(px >> (8 * c)) & 0xFFu];
    return byte_to_float(px, c);                          // c/255*255 == c
}

// ---------------------------------------------------------------------------
// texel fetch (MainCS 561-580); zero or clamp outside the image
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void load_block(const Launch& p, int bx, int by,
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
// per-block pipeline (encode_block 510-550)
// ---------------------------------------------------------------------------
template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
__device__ __forceinline__ uint4 encode_block(const uint32_t (&px)[DIM * DIM], const float* lut,
                                              const uint8_t* trits) {
    constexpr int N = DIM * DIM;
    // mean (143-147), then x fl(1/N)
    float mean[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) mean[c] = __fadd_rn(mean[c], texel<SRGB, NORMAL>(px[k], c, lut));
    constexpr float kInvN = 1.0f / (float)N;
#pragma unroll
    for (int c = 0; c < 4; ++c) mean[c] = __fmul_rn(mean[c], kInvN);

    // covariance (149-162): symmetric, 10 unique terms, x fl(1/(N-1))
    float cv[10] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float d[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) d[c] = __fsub_rn(texel<SRGB, NORMAL>(px[k], c, lut), mean[c]);
        int e = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = i; j < 4; ++j, ++e) cv[e] = __fmaf_rn(d[i], d[j], cv[e]);
    }
    constexpr float kInvN1 = 1.0f / (float)(N - 1);
#pragma unroll
    for (int e = 0; e < 10; ++e) cv[e] = __fmul_rn(cv[e], kInvN1);
    const float m[4][4] = {{cv[0], cv[1], cv[2], cv[3]},
                           {cv[1], cv[4], cv[5], cv[6]},
                           {cv[2], cv[5], cv[7], cv[8]},
                           {cv[3], cv[6], cv[8], cv[9]}};

    // power iteration (93-106)
    float v[4] = {0.26726f, 0.80178f, 0.53452f, 0.0f};
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float t[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) t[r] = dot4(m[r], v);
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] = t[r];
        if (__fsqrt_rn(dot4(v, v)) < 1e-5f) break;
#pragma unroll
        for (int r = 0; r < 4; ++r) t[r] = dot4(m[r], v);
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] = t[r];
        normalize4(v);
    }

    // find_min_max (108-137)
    float a = 1e31f, b = -1e31f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float d[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) d[c] = __fsub_rn(texel<SRGB, NORMAL>(px[k], c, lut), mean[c]);
        const float t = dot4(d, v);
        a = fminf(a, t);
        b = fmaxf(b, t);
    }
    float e0[4], e1[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        e0[c] = fminf(fmaxf(__fmaf_rn(v[c], a, mean[c]), 0.0f), 255.0f);
        e1[c] = fminf(fmaxf(__fmaf_rn(v[c], b, mean[c]), 0.0f), 255.0f);
    }
    uint32_t q0[4], q1[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) { q0[c] = rint_u32(e0[c]); q1[c] = rint_u32(e1[c]); }
    if (q0[0] + q0[1] + q0[2] > q1[0] + q1[1] + q1[2]) {      // dark endpoint first
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float tf = e0[c]; e0[c] = e1[c]; e1[c] = tf;
            const uint32_t tq = q0[c]; q0[c] = q1[c]; q1[c] = tq;
        }
    }
    if (!ALPHA) { e0[3] = 255.0f; e1[3] = 255.0f; q0[3] = 255u; q1[3] = 255u; }

    // weights on the 4x4 grid (316-372), quantised (256-260, 374-393)
    constexpr uint32_t R = ALPHA ? 5u : 11u;
    uint32_t qw[16];
    {
        float k[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) k[c] = __fsub_rn(e1[c], e0[c]);
        if (__fsqrt_rn(dot4(k, k)) < 1e-5f) {
#pragma unroll
            for (int i = 0; i < 16; ++i) qw[i] = 0u;
        } else {
            normalize4(k);
            float w[16];
            float minw = 1e31f, maxw = -1e31f;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                float s[4];
                if constexpr (DIM == 6) {
                    // 2x2 taps of grid point i: columns/rows {0,1,3,4}+{0,1};
                    // 4/9, 2/9, 1/9 written as 0.444, 0.222, 0.111
                    const int gx = i & 3, gy = i >> 2;
                    const int i0 = (gy < 2 ? gy : gy + 1) * 6 + (gx < 2 ? gx : gx + 1);
                    const bool xl = (gx & 1) == 0, yl = (gy & 1) == 0;
                    const float w00 = (xl && yl) ? 0.444f : (xl || yl) ? 0.222f : 0.111f;
                    const float w01 = (!xl && yl) ? 0.444f : (!xl || yl) ? 0.222f : 0.111f;
                    const float w10 = (xl && !yl) ? 0.444f : (xl || !yl) ? 0.222f : 0.111f;
                    const float w11 = (!xl && !yl) ? 0.444f : (!xl || !yl) ? 0.222f : 0.111f;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        float acc = __fmul_rn(texel<SRGB, NORMAL>(px[i0], c, lut), w00);
                        acc = __fmaf_rn(texel<SRGB, NORMAL>(px[i0 + 1], c, lut), w01, acc);
                        acc = __fmaf_rn(texel<SRGB, NORMAL>(px[i0 + 6], c, lut), w10, acc);
                        acc = __fmaf_rn(texel<SRGB, NORMAL>(px[i0 + 7], c, lut), w11, acc);
                        s[c] = acc;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 4; ++c) s[c] = texel<SRGB, NORMAL>(px[i], c, lut);
                }
                float d[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) d[c] = __fsub_rn(s[c], e0[c]);
                const float x = dot4(k, d);
                minw = fminf(x, minw);
                maxw = fmaxf(x, maxw);
                w[i] = x;
            }
            float inv = fmaxf(1e-5f, __fsub_rn(maxw, minw));
            inv = __frcp_rn(inv);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const float wn = __fmul_rn(__fsub_rn(w[i], minw), inv);
                const uint32_t q = rint_u32(__fmul_rn(wn, (float)R));
                qw[i] = q < R ? q : R;
            }
        }
    }

    // scramble (491-502) + ISE of 16 weights in trits (ISE.hlsl 142-176, 243-256)
    constexpr int WQ = ALPHA ? kQuant6 : kQuant12;
    constexpr int B = ALPHA ? 1 : 2;
    constexpr uint64_t kScr = scramble_nibbles(WQ);
    constexpr uint32_t kScrLo = (uint32_t)kScr, kScrHi = (uint32_t)(kScr >> 32);
    uint64_t ws = 0;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        uint32_t mm[5], tt[5];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const int idx = g * 5 + j;
            uint32_t s = 0;
            if (idx < 16) {
                const uint32_t q = qw[idx < 16 ? idx : 0];
                s = (q < 8 ? (kScrLo >> (4 * q)) : (kScrHi >> (4 * (q - 8)))) & 0xFu;
            }
            mm[j] = s & ((1u << B) - 1u);
            tt[j] = s >> B;
        }
        const uint32_t T = trits[tt[4] * 81 + tt[3] * 27 + tt[2] * 9 + tt[1] * 3 + tt[0]];
        const uint64_t grp = (uint64_t)mm[0] | ((uint64_t)(T & 3u) << B) |
                             ((uint64_t)mm[1] << (B + 2)) | ((uint64_t)((T >> 2) & 3u) << (2 * B + 2)) |
                             ((uint64_t)mm[2] << (2 * B + 4)) | ((uint64_t)((T >> 4) & 1u) << (3 * B + 4)) |
                             ((uint64_t)mm[3] << (3 * B + 5)) | ((uint64_t)((T >> 5) & 3u) << (4 * B + 5)) |
                             ((uint64_t)mm[4] << (4 * B + 7)) | ((uint64_t)((T >> 7) & 1u) << (5 * B + 7));
        ws |= grp << (g * (5 * B + 8));
    }

    // endpoints in QUANT_256: r0 r1 g0 g1 b0 b1 [a0 a1], 8 bits each (bise_endpoints)
    uint64_t ep = (uint64_t)q0[0] | ((uint64_t)q1[0] << 8) | ((uint64_t)q0[1] << 16) |
                  ((uint64_t)q1[1] << 24) | ((uint64_t)q0[2] << 32) | ((uint64_t)q1[2] << 40);
    if (ALPHA) ep |= ((uint64_t)q0[3] << 48) | ((uint64_t)q1[3] << 56);

    // assemble_block (400-444): mode [10:0], CEM [16:13], endpoints from bit 17,
    // weight stream bit-reversed from bit 127 down.
    constexpr uint64_t kHead = (uint64_t)blockmode_4x4_grid(WQ) | ((uint64_t)(ALPHA ? 12u : 8u) << 13);
    const uint64_t lo = kHead | (ep << 17);
    const uint64_t hi = (ep >> 47) | __brevll(ws);
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
__global__ void __launch_bounds__(kThreads) astc_encode_blocks_fp32(const Launch p) {
    __shared__ uint8_t s_trits[256];
    __shared__ float s_lut[SRGB ? 256 : 1];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        s_trits[i] = c_trit_pack.v[i];
        if (SRGB) s_lut[i] = c_srgb_x255[i];
    }
    __syncthreads();
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblocks) return;
    const int by = (int)(b / p.nbx);
    const int bx = (int)(b - (long long)by * p.nbx);
    uint32_t px[DIM * DIM];
    load_block<DIM>(p, bx, by, px);
    p.out[b] = encode_block<DIM, ALPHA, NORMAL, SRGB>(px, s_lut, s_trits);
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
cudaError_t launch_t(const Launch& p, cudaStream_t s) {
    const long long grid = (p.nblocks + kThreads - 1) / kThreads;
    astc_encode_blocks_fp32<DIM, ALPHA, NORMAL, SRGB><<<(unsigned)grid, kThreads, 0, s>>>(p);
    return cudaGetLastError();
}

template <int DIM, bool ALPHA, bool NORMAL>
cudaError_t launch_srgb(const Launch& p, bool srgb, cudaStream_t s) {
    return srgb ? launch_t<DIM, ALPHA, NORMAL, true>(p, s) : launch_t<DIM, ALPHA, NORMAL, false>(p, s);
}
template <int DIM, bool ALPHA>
cudaError_t launch_norm(const Launch& p, bool normal, bool srgb, cudaStream_t s) {
    return normal ? launch_srgb<DIM, ALPHA, true>(p, srgb, s) : launch_srgb<DIM, ALPHA, false>(p, srgb, s);
}
template <int DIM>
cudaError_t launch_alpha(const Launch& p, bool alpha, bool normal, bool srgb, cudaStream_t s) {
    return alpha ? launch_norm<DIM, true>(p, normal, srgb, s) : launch_norm<DIM, false>(p, normal, srgb, s);
}

}  // namespace

float srgb_texel_value(int code) {
    const double x = code / 255.0;
    const double lin = x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4);
    return (float)lin * 255.0f;
}

// Uploads the sRGB table to the current device (once per pool set-up).
cudaError_t ensure_encode_constants(int device) {
    if (device < 0) return cudaErrorInvalidDevice;
    float lut[256];
    for (int c = 0; c < 256; ++c) lut[c] = srgb_texel_value(c);
    return cudaMemcpyToSymbol(c_srgb_x255, lut, sizeof(lut));
}

cudaError_t launch_encode(const EncodeJob& j, cudaStream_t stream) {
    Launch p;
    p.in = j.in;
    p.pitch = j.pitch;
    p.width = j.width;
    p.height = j.height;
    p.nbx = blocks_x(j.width, j.block_dim);
    p.nblocks = (long long)p.nbx * blocks_y(j.height, j.block_dim);
    p.out = reinterpret_cast<uint4*>(j.out);
    const uintptr_t base = reinterpret_cast<uintptr_t>(j.in);
    const size_t va = j.block_dim == 4 ? 16 : 8;
    p.vec_ok = (base % va == 0) && (j.pitch % va == 0);
    p.clamp = j.border == ASTC_BORDER_CLAMP;
    const bool alpha = j.has_alpha != 0, normal = j.is_normal != 0, srgb = j.srgb != 0;
    cudaError_t e = j.block_dim == 4 ? launch_alpha<4>(p, alpha, normal, srgb, stream)
                                     : launch_alpha<6>(p, alpha, normal, srgb, stream);
    if (e == cudaSuccess) count_launches(1);
    return e;
}

}  // namespace astc
