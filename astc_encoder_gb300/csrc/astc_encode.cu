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
// but written for the GPU: each texel is decoded once (UNORM8 by a byte_perm
// into a 2^23-biased float, sRGB through a shared-memory table) into a texel
// store -- registers, or for 6x6 a [texel][thread] shared-memory array that
// keeps the register count (and so the occupancy) of the 36-texel block in
// check; the length tests compare against an exact threshold instead of
// taking a square root; the ISE of the fixed weight range is unrolled into
// 64-bit shifts and the weight bit reversal is one __brevll.
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
#include <mutex>

#include "astc_block_common.cuh"
#include "astc_internal.h"

namespace astc {
namespace {

constexpr int kMaxThreads = 256;

__constant__ TritPack c_trit_pack = make_trit_pack();
__constant__ float c_srgb_x255[256];

struct Launch {
    TextureView tex;
    long long nblocks;
    uint4* out;
};

// ---------------------------------------------------------------------------
// per-block pipeline (encode_block 510-550) over a texel store S
// ---------------------------------------------------------------------------
template <int DIM, bool ALPHA, class S>
__device__ __forceinline__ uint4 encode_block_fp32(const S& st, const uint8_t* trits) {
    constexpr int N = DIM * DIM;
    // mean (143-147), then x fl(1/N)
    float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        m0 = __fadd_rn(m0, t.x); m1 = __fadd_rn(m1, t.y);
        m2 = __fadd_rn(m2, t.z); m3 = __fadd_rn(m3, t.w);
    }
    constexpr float kInvN = 1.0f / (float)N;
    m0 = __fmul_rn(m0, kInvN); m1 = __fmul_rn(m1, kInvN);
    m2 = __fmul_rn(m2, kInvN); m3 = __fmul_rn(m3, kInvN);

    // covariance (149-162): symmetric, 10 unique terms, x fl(1/(N-1))
    float c00 = 0.f, c01 = 0.f, c02 = 0.f, c03 = 0.f, c11 = 0.f, c12 = 0.f, c13 = 0.f,
          c22 = 0.f, c23 = 0.f, c33 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        const float d0 = __fsub_rn(t.x, m0), d1 = __fsub_rn(t.y, m1);
        const float d2 = __fsub_rn(t.z, m2), d3 = __fsub_rn(t.w, m3);
        c00 = __fmaf_rn(d0, d0, c00); c01 = __fmaf_rn(d0, d1, c01);
        c02 = __fmaf_rn(d0, d2, c02); c03 = __fmaf_rn(d0, d3, c03);
        c11 = __fmaf_rn(d1, d1, c11); c12 = __fmaf_rn(d1, d2, c12);
        c13 = __fmaf_rn(d1, d3, c13); c22 = __fmaf_rn(d2, d2, c22);
        c23 = __fmaf_rn(d2, d3, c23); c33 = __fmaf_rn(d3, d3, c33);
    }
    constexpr float kInvN1 = 1.0f / (float)(N - 1);
    c00 = __fmul_rn(c00, kInvN1); c01 = __fmul_rn(c01, kInvN1); c02 = __fmul_rn(c02, kInvN1);
    c03 = __fmul_rn(c03, kInvN1); c11 = __fmul_rn(c11, kInvN1); c12 = __fmul_rn(c12, kInvN1);
    c13 = __fmul_rn(c13, kInvN1); c22 = __fmul_rn(c22, kInvN1); c23 = __fmul_rn(c23, kInvN1);
    c33 = __fmul_rn(c33, kInvN1);

    // power iteration (93-106): v = M v; stop if |v| < 1e-5; v = normalize(M v)
    float v0 = 0.26726f, v1 = 0.80178f, v2 = 0.53452f, v3 = 0.0f;
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float t0 = dot4(c00, c01, c02, c03, v0, v1, v2, v3);
        float t1 = dot4(c01, c11, c12, c13, v0, v1, v2, v3);
        float t2 = dot4(c02, c12, c22, c23, v0, v1, v2, v3);
        float t3 = dot4(c03, c13, c23, c33, v0, v1, v2, v3);
        v0 = t0; v1 = t1; v2 = t2; v3 = t3;
        if (shorter_than_small_value(dot4(v0, v1, v2, v3, v0, v1, v2, v3))) break;
        t0 = dot4(c00, c01, c02, c03, v0, v1, v2, v3);
        t1 = dot4(c01, c11, c12, c13, v0, v1, v2, v3);
        t2 = dot4(c02, c12, c22, c23, v0, v1, v2, v3);
        t3 = dot4(c03, c13, c23, c33, v0, v1, v2, v3);
        const float r = rnorm_from_dot(dot4(t0, t1, t2, t3, t0, t1, t2, t3));
        v0 = __fmul_rn(t0, r); v1 = __fmul_rn(t1, r); v2 = __fmul_rn(t2, r); v3 = __fmul_rn(t3, r);
    }

    // find_min_max (108-137)
    float a = 1e31f, b = -1e31f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        const float p = dot4(__fsub_rn(t.x, m0), __fsub_rn(t.y, m1), __fsub_rn(t.z, m2),
                             __fsub_rn(t.w, m3), v0, v1, v2, v3);
        a = fminf(a, p);
        b = fmaxf(b, p);
    }
    float e0[4], e1[4];
    const float mv[4] = {m0, m1, m2, m3}, vv[4] = {v0, v1, v2, v3};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        e0[c] = fminf(fmaxf(__fmaf_rn(vv[c], a, mv[c]), 0.0f), 255.0f);
        e1[c] = fminf(fmaxf(__fmaf_rn(vv[c], b, mv[c]), 0.0f), 255.0f);
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
    float k0 = __fsub_rn(e1[0], e0[0]), k1 = __fsub_rn(e1[1], e0[1]);
    float k2 = __fsub_rn(e1[2], e0[2]), k3 = __fsub_rn(e1[3], e0[3]);
    const float kk = dot4(k0, k1, k2, k3, k0, k1, k2, k3);
    if (shorter_than_small_value(kk)) {
#pragma unroll
        for (int i = 0; i < 16; ++i) qw[i] = 0u;
    } else {
        const float r = rnorm_from_dot(kk);
        k0 = __fmul_rn(k0, r); k1 = __fmul_rn(k1, r); k2 = __fmul_rn(k2, r); k3 = __fmul_rn(k3, r);
        float w[16];
        float minw = 1e31f, maxw = -1e31f;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            float4 s;
            if constexpr (DIM == 6) {
                const int i0 = grid_tap0(i);
                float w00, w01, w10, w11;
                grid_weights(i, w00, w01, w10, w11);
                const float4 t00 = st.get(i0), t01 = st.get(i0 + 1), t10 = st.get(i0 + 6),
                             t11 = st.get(i0 + 7);
                s.x = __fmaf_rn(t11.x, w11, __fmaf_rn(t10.x, w10, __fmaf_rn(t01.x, w01, __fmul_rn(t00.x, w00))));
                s.y = __fmaf_rn(t11.y, w11, __fmaf_rn(t10.y, w10, __fmaf_rn(t01.y, w01, __fmul_rn(t00.y, w00))));
                s.z = __fmaf_rn(t11.z, w11, __fmaf_rn(t10.z, w10, __fmaf_rn(t01.z, w01, __fmul_rn(t00.z, w00))));
                s.w = __fmaf_rn(t11.w, w11, __fmaf_rn(t10.w, w10, __fmaf_rn(t01.w, w01, __fmul_rn(t00.w, w00))));
            } else {
                s = st.get(i);
            }
            const float x = dot4(k0, k1, k2, k3, __fsub_rn(s.x, e0[0]), __fsub_rn(s.y, e0[1]),
                                 __fsub_rn(s.z, e0[2]), __fsub_rn(s.w, e0[3]));
            minw = fminf(x, minw);
            maxw = fmaxf(x, maxw);
            w[i] = x;
        }
        const float inv = __frcp_rn(fmaxf(1e-5f, __fsub_rn(maxw, minw)));
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float wn = __fmul_rn(__fsub_rn(w[i], minw), inv);
            const uint32_t q = rint_u32(__fmul_rn(wn, (float)R));
            qw[i] = q < R ? q : R;
        }
    }
    return assemble_block<ALPHA>(q0, q1, qw, trits);
}

// The shared-memory store caps registers (two 256-thread CTAs per SM, <= 128
// registers) so the compiler re-reads texels from shared memory instead of
// holding all of them in registers across the passes.
template <int DIM, bool ALPHA, bool NORMAL, bool SRGB, int STORE>
__global__ void __launch_bounds__(kMaxThreads, STORE == kStoreShared ? 2 : 1)
astc_encode_blocks_fp32(const Launch p) {
    constexpr int N = DIM * DIM;
    extern __shared__ float4 s_texels[];                  // kStoreShared only
    __shared__ uint8_t s_trits[256];
    __shared__ float s_lut[SRGB ? 256 : 1];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        s_trits[i] = c_trit_pack.v[i];
        if (SRGB) s_lut[i] = c_srgb_x255[i];
    }
    __syncthreads();
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblocks) return;
    const int by = (int)(b / p.tex.nbx);
    const int bx = (int)(b - (long long)by * p.tex.nbx);
    uint32_t px[N];
    load_block_packed<DIM>(p.tex, bx, by, px);
    if constexpr (STORE == kStoreShared) {
        SharedTexels<N> st{s_texels + threadIdx.x, (int)blockDim.x};
#pragma unroll
        for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
        p.out[b] = encode_block_fp32<DIM, ALPHA>(st, s_trits);
    } else {
        RegTexels<N> st;
#pragma unroll
        for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
        p.out[b] = encode_block_fp32<DIM, ALPHA>(st, s_trits);
    }
}

// Kernel choice per format: texel store and CTA size.  Defaults come from
// measurements on GB300 (profiles/); the autotuner may replace them.
struct Choice { int store; int threads; };
Choice g_choice[2][2][2][2] = {};     // [dim6][alpha][normal][srgb]
bool g_choice_init = false;
std::mutex g_choice_mu;

// GB300 sweep over 2048x2048 textures (us per launch, registers / shared at
// 128 threads): 4x4 RGB 28.4 / 27.0, 4x4 RGBA sRGB 29.0 / 28.9, 4x4 normal
// 20.8 / 20.8, 6x6 RGBA sRGB 26.8 / 39.1, 6x6 RGB 24.8 / 40.9.  The capped
// shared-memory variant loses for 6x6 (its re-reads cost more than the
// occupancy it gains) and ties or wins slightly for 4x4.
Choice default_choice(int dim, bool /*alpha*/, bool /*normal*/, bool /*srgb*/) {
    return dim == 6 ? Choice{kStoreRegisters, 128} : Choice{kStoreShared, 128};
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB, int STORE>
cudaError_t launch_t(const Launch& p, int threads, cudaStream_t s) {
    constexpr int N = DIM * DIM;
    const size_t smem = STORE == kStoreShared ? (size_t)N * threads * sizeof(float4) : 0;
    auto kern = astc_encode_blocks_fp32<DIM, ALPHA, NORMAL, SRGB, STORE>;
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
        if (e != cudaSuccess) return e;
    }
    const long long grid = (p.nblocks + threads - 1) / threads;
    kern<<<(unsigned)grid, threads, smem, s>>>(p);
    return cudaGetLastError();
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
cudaError_t launch_store(const Launch& p, const Choice& c, cudaStream_t s) {
    if (c.store == kStoreShared)
        return launch_t<DIM, ALPHA, NORMAL, SRGB, kStoreShared>(p, c.threads, s);
    return launch_t<DIM, ALPHA, NORMAL, SRGB, kStoreRegisters>(p, c.threads, s);
}
template <int DIM, bool ALPHA, bool NORMAL>
cudaError_t launch_srgb(const Launch& p, bool srgb, const Choice& c, cudaStream_t s) {
    return srgb ? launch_store<DIM, ALPHA, NORMAL, true>(p, c, s)
                : launch_store<DIM, ALPHA, NORMAL, false>(p, c, s);
}
template <int DIM, bool ALPHA>
cudaError_t launch_norm(const Launch& p, bool normal, bool srgb, const Choice& c, cudaStream_t s) {
    return normal ? launch_srgb<DIM, ALPHA, true>(p, srgb, c, s)
                  : launch_srgb<DIM, ALPHA, false>(p, srgb, c, s);
}
template <int DIM>
cudaError_t launch_alpha(const Launch& p, bool alpha, bool normal, bool srgb, const Choice& c,
                         cudaStream_t s) {
    return alpha ? launch_norm<DIM, true>(p, normal, srgb, c, s)
                 : launch_norm<DIM, false>(p, normal, srgb, c, s);
}

Choice current_choice(int dim, bool alpha, bool normal, bool srgb) {
    std::lock_guard<std::mutex> lk(g_choice_mu);
    if (!g_choice_init) {
        for (int d = 0; d < 2; ++d)
            for (int a = 0; a < 2; ++a)
                for (int n = 0; n < 2; ++n)
                    for (int r = 0; r < 2; ++r)
                        g_choice[d][a][n][r] = default_choice(d ? 6 : 4, a, n, r);
        g_choice_init = true;
    }
    return g_choice[dim == 6][alpha][normal][srgb];
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

TextureView make_view(const EncodeJob& j) {
    TextureView t;
    t.in = j.in;
    t.pitch = j.pitch;
    t.width = j.width;
    t.height = j.height;
    t.nbx = blocks_x(j.width, j.block_dim);
    const uintptr_t base = reinterpret_cast<uintptr_t>(j.in);
    const size_t va = j.block_dim == 4 ? 16 : 8;
    t.vec_ok = (base % va == 0) && (j.pitch % va == 0);
    t.clamp = j.border == ASTC_BORDER_CLAMP;
    return t;
}

cudaError_t launch_encode_variant(const EncodeJob& j, int store, int threads, cudaStream_t stream) {
    if (threads != 32 && threads != 64 && threads != 128 && threads != 256) return cudaErrorInvalidValue;
    if (store != kStoreRegisters && store != kStoreShared) return cudaErrorInvalidValue;
    Launch p;
    p.tex = make_view(j);
    p.nblocks = (long long)p.tex.nbx * blocks_y(j.height, j.block_dim);
    p.out = reinterpret_cast<uint4*>(j.out);
    const bool alpha = j.has_alpha != 0, normal = j.is_normal != 0, srgb = j.srgb != 0;
    const Choice c{store, threads};
    cudaError_t e = j.block_dim == 4 ? launch_alpha<4>(p, alpha, normal, srgb, c, stream)
                                     : launch_alpha<6>(p, alpha, normal, srgb, c, stream);
    if (e == cudaSuccess) count_launches(1);
    return e;
}

cudaError_t launch_encode(const EncodeJob& j, cudaStream_t stream) {
    const Choice c = current_choice(j.block_dim, j.has_alpha != 0, j.is_normal != 0, j.srgb != 0);
    return launch_encode_variant(j, c.store, c.threads, stream);
}

void set_encode_choice(int dim, bool alpha, bool normal, bool srgb, int store, int threads) {
    current_choice(dim, alpha, normal, srgb);
    std::lock_guard<std::mutex> lk(g_choice_mu);
    g_choice[dim == 6][alpha][normal][srgb] = Choice{store, threads};
}

void get_encode_choice(int dim, bool alpha, bool normal, bool srgb, int* store, int* threads) {
    const Choice c = current_choice(dim, alpha, normal, srgb);
    *store = c.store;
    *threads = c.threads;
}

}  // namespace astc
