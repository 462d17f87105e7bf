// astc_pipeline_fp32.cuh -- the FP32 per-block pipeline of the reference
// shader (niepp/astc_encoder ASTC_Encode.hlsl encode_block 510-550 and the
// functions it calls), over any texel store, in stages the search mode
// reuses.  Floating point follows the FP32 oracle's model operation by
// operation, so every block is bit-identical to the oracle; compile
// including translation units with --fmad=false.
#pragma once
#include "astc_block_common.cuh"

namespace astc {

// ZW forms (normal maps): the blue and alpha of every texel are the constant
// 255 (ASTC_Encode.hlsl:575-578), so their deviations from the mean are +0
// and every product with them is a zero.  The ZW forms leave those terms out;
// a result then differs from the full form's at most in the sign of a zero,
// which no comparison, clamp or rounding downstream distinguishes (blocks stay
// bit-identical to the oracle, which computes every term).

// the mean of N texels whose channel is 255, computed as block_mean does
template <int N>
constexpr float mean_of_255() {
    float s = 0.0f;
    for (int k = 0; k < N; ++k) s = s + 255.0f;
    return s * (1.0f / (float)N);
}
static_assert(mean_of_255<16>() == 255.0f && mean_of_255<36>() == 255.0f, "constant channel mean");

// mean (ASTC_Encode.hlsl:143-147, 172-178): sum, then x fl(1/N)
template <int N, bool ZW = false, class S>
__device__ __forceinline__ float4 block_mean(const S& st) {
    if constexpr (ZW) {
        float m0 = 0.f, m1 = 0.f;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float4 t = st.get(k);
            m0 = __fadd_rn(m0, t.x); m1 = __fadd_rn(m1, t.y);
        }
        constexpr float kInvN = 1.0f / (float)N;
        return make_float4(__fmul_rn(m0, kInvN), __fmul_rn(m1, kInvN), 255.0f, 255.0f);
    }
    float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        m0 = __fadd_rn(m0, t.x); m1 = __fadd_rn(m1, t.y);
        m2 = __fadd_rn(m2, t.z); m3 = __fadd_rn(m3, t.w);
    }
    constexpr float kInvN = 1.0f / (float)N;
    return make_float4(__fmul_rn(m0, kInvN), __fmul_rn(m1, kInvN), __fmul_rn(m2, kInvN),
                       __fmul_rn(m3, kInvN));
}

// eigen_vector (93-106) of the symmetric 4x4 matrix c: v = M v; stop if
// |v| < 1e-5 (returning that v); v = normalize(M v); eight rounds
__device__ __forceinline__ float4 power_iteration(float c00, float c01, float c02, float c03, float c11,
                                                  float c12, float c13, float c22, float c23, float c33) {
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
    return make_float4(v0, v1, v2, v3);
}

// power_iteration for a matrix whose rows and columns 2 and 3 are zero (ZW)
__device__ __forceinline__ float4 power_iteration_zw(float c00, float c01, float c11) {
    float v0 = 0.26726f, v1 = 0.80178f;
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float t0 = __fmaf_rn(c01, v1, __fmul_rn(c00, v0));
        float t1 = __fmaf_rn(c11, v1, __fmul_rn(c01, v0));
        v0 = t0; v1 = t1;
        if (shorter_than_small_value(__fmaf_rn(v1, v1, __fmul_rn(v0, v0)))) break;
        t0 = __fmaf_rn(c01, v1, __fmul_rn(c00, v0));
        t1 = __fmaf_rn(c11, v1, __fmul_rn(c01, v0));
        const float r = rnorm_from_dot(__fmaf_rn(t1, t1, __fmul_rn(t0, t0)));
        v0 = __fmul_rn(t0, r); v1 = __fmul_rn(t1, r);
    }
    return make_float4(v0, v1, 0.0f, 0.0f);
}

// covariance (149-162): symmetric, 10 unique terms, x fl(1/(N-1))
struct Covariance {
    float c00, c01, c02, c03, c11, c12, c13, c22, c23, c33;
};

template <int N, bool ZW = false, class S>
__device__ __forceinline__ Covariance block_covariance(const S& st, const float4 m) {
    constexpr float kInvN1 = 1.0f / (float)(N - 1);
    if constexpr (ZW) {
        float c00 = 0.f, c01 = 0.f, c11 = 0.f;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float4 t = st.get(k);
            const float d0 = __fsub_rn(t.x, m.x), d1 = __fsub_rn(t.y, m.y);
            c00 = __fmaf_rn(d0, d0, c00); c01 = __fmaf_rn(d0, d1, c01); c11 = __fmaf_rn(d1, d1, c11);
        }
        return Covariance{__fmul_rn(c00, kInvN1), __fmul_rn(c01, kInvN1), 0.f, 0.f, __fmul_rn(c11, kInvN1),
                          0.f, 0.f, 0.f, 0.f, 0.f};
    }
    float c00 = 0.f, c01 = 0.f, c02 = 0.f, c03 = 0.f, c11 = 0.f, c12 = 0.f, c13 = 0.f,
          c22 = 0.f, c23 = 0.f, c33 = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        const float d0 = __fsub_rn(t.x, m.x), d1 = __fsub_rn(t.y, m.y);
        const float d2 = __fsub_rn(t.z, m.z), d3 = __fsub_rn(t.w, m.w);
        c00 = __fmaf_rn(d0, d0, c00); c01 = __fmaf_rn(d0, d1, c01);
        c02 = __fmaf_rn(d0, d2, c02); c03 = __fmaf_rn(d0, d3, c03);
        c11 = __fmaf_rn(d1, d1, c11); c12 = __fmaf_rn(d1, d2, c12);
        c13 = __fmaf_rn(d1, d3, c13); c22 = __fmaf_rn(d2, d2, c22);
        c23 = __fmaf_rn(d2, d3, c23); c33 = __fmaf_rn(d3, d3, c33);
    }
    return Covariance{__fmul_rn(c00, kInvN1), __fmul_rn(c01, kInvN1), __fmul_rn(c02, kInvN1),
                      __fmul_rn(c03, kInvN1), __fmul_rn(c11, kInvN1), __fmul_rn(c12, kInvN1),
                      __fmul_rn(c13, kInvN1), __fmul_rn(c22, kInvN1), __fmul_rn(c23, kInvN1),
                      __fmul_rn(c33, kInvN1)};
}

// principal axis: the covariance, then the power iteration (eigen_vector
// 93-106): v = M v; stop if |v| < 1e-5; v = normalize(M v)
template <int N, bool ZW = false, class S>
__device__ __forceinline__ float4 pca_axis(const S& st, const float4 m) {
    const Covariance c = block_covariance<N, ZW>(st, m);
    if constexpr (ZW) return power_iteration_zw(c.c00, c.c01, c.c11);
    return power_iteration(c.c00, c.c01, c.c02, c.c03, c.c11, c.c12, c.c13, c.c22, c.c23, c.c33);
}

// max_accumulation_pixel_direction (170-227), the shader's alternative axis:
// the largest of the sums of the deviations of the texels whose red, green,
// blue (with alpha: or alpha) lies above the mean; safe-normalised
template <int N, bool ALPHA, class S>
__device__ __forceinline__ float4 max_accumulation_axis(const S& st, const float4 m) {
    float s[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) s[a][c] = 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        const float d[4] = {__fsub_rn(t.x, m.x), __fsub_rn(t.y, m.y), __fsub_rn(t.z, m.z),
                            __fsub_rn(t.w, m.w)};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) s[a][c] = __fadd_rn(s[a][c], d[a] > 0.0f ? d[c] : 0.0f);
    }
    float k0 = s[0][0], k1 = s[0][1], k2 = s[0][2], k3 = s[0][3];
    float maxdot = dot4(k0, k1, k2, k3, k0, k1, k2, k3);
#pragma unroll
    for (int a = 1; a < (ALPHA ? 4 : 3); ++a) {
        const float d = dot4(s[a][0], s[a][1], s[a][2], s[a][3], s[a][0], s[a][1], s[a][2], s[a][3]);
        if (d > maxdot) {
            maxdot = d;
            k0 = s[a][0]; k1 = s[a][1]; k2 = s[a][2]; k3 = s[a][3];
        }
    }
    const float kk = dot4(k0, k1, k2, k3, k0, k1, k2, k3);
    if (!shorter_than_small_value(kk)) {
        const float r = rnorm_from_dot(kk);
        k0 = __fmul_rn(k0, r); k1 = __fmul_rn(k1, r); k2 = __fmul_rn(k2, r); k3 = __fmul_rn(k3, r);
    }
    return make_float4(k0, k1, k2, k3);
}

// The end of find_min_max (120-136): clamped endpoints m + v * a and
// m + v * b from the extreme projections a, b, the darker (rounded RGB sum)
// first; !ALPHA forces alpha 255.
template <bool ALPHA>
__device__ __forceinline__ void endpoints_from_range(const float4 m, const float4 v, float a, float b, float e0[4],
                                                     float e1[4], uint32_t q0[4], uint32_t q1[4]) {
    const float mv[4] = {m.x, m.y, m.z, m.w}, vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        e0[c] = fminf(fmaxf(__fmaf_rn(vv[c], a, mv[c]), 0.0f), 255.0f);
        e1[c] = fminf(fmaxf(__fmaf_rn(vv[c], b, mv[c]), 0.0f), 255.0f);
    }
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
}

// find_min_max (108-137): extreme projections on the axis, clamped
// endpoints, the darker (rounded RGB sum) first; !ALPHA forces alpha 255.
// e0/e1 are the float endpoints, q0/q1 their rounded (QUANT_256) values.
template <int N, bool ALPHA, bool ZW = false, class S>
__device__ __forceinline__ void find_min_max(const S& st, const float4 m, const float4 v, float e0[4],
                                             float e1[4], uint32_t q0[4], uint32_t q1[4], uint64_t sel = ~0ull) {
    float a = 1e31f, b = -1e31f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (!((sel >> k) & 1)) continue;                       // texels outside `sel` take no part
        const float4 t = st.get(k);
        const float p = ZW ? __fmaf_rn(__fsub_rn(t.y, m.y), v.y, __fmul_rn(__fsub_rn(t.x, m.x), v.x))
                           : dot4(__fsub_rn(t.x, m.x), __fsub_rn(t.y, m.y), __fsub_rn(t.z, m.z),
                                  __fsub_rn(t.w, m.w), v.x, v.y, v.z, v.w);
        a = fminf(a, p);
        b = fmaxf(b, p);
    }
    endpoints_from_range<ALPHA>(m, v, a, b, e0, e1, q0, q1);
}

// the colour at weight-grid point g: the texel (4x4) or sample_texel's 2x2
// bilinear tap sum (307-314, 6x6)
// NCH: the channels the caller uses (2: red and green, 3: no alpha, 4: all);
// the others are left as 0
template <int DIM, int NCH = 4, class S>
__device__ __forceinline__ float4 grid_sample(const S& st, int g) {
    if constexpr (DIM == 6) {
        const int i0 = grid_tap0(g);
        float w00, w01, w10, w11;
        grid_weights(g, w00, w01, w10, w11);
        const float4 t00 = st.get(i0), t01 = st.get(i0 + 1), t10 = st.get(i0 + 6), t11 = st.get(i0 + 7);
        float4 s;
        s.x = __fmaf_rn(t11.x, w11, __fmaf_rn(t10.x, w10, __fmaf_rn(t01.x, w01, __fmul_rn(t00.x, w00))));
        s.y = __fmaf_rn(t11.y, w11, __fmaf_rn(t10.y, w10, __fmaf_rn(t01.y, w01, __fmul_rn(t00.y, w00))));
        s.z = 0.0f;
        s.w = 0.0f;
        if constexpr (NCH >= 3)
            s.z = __fmaf_rn(t11.z, w11, __fmaf_rn(t10.z, w10, __fmaf_rn(t01.z, w01, __fmul_rn(t00.z, w00))));
        if constexpr (NCH >= 4)
            s.w = __fmaf_rn(t11.w, w11, __fmaf_rn(t10.w, w10, __fmaf_rn(t01.w, w01, __fmul_rn(t00.w, w00))));
        return s;
    } else {
        return st.get(g);
    }
}

// weights on the 4x4 grid (calculate_normal_weights 316-372): projections on
// normalize(e1 - e0) rescaled to [min, max], quantised (256-260, 374-393)
// to 0..R, R = 5 (QUANT_6, alpha) or 11 (QUANT_12)
template <int DIM, bool ALPHA, bool ZW = false, class S>
__device__ __forceinline__ void reference_weights(const S& st, const float e0[4], const float e1[4],
                                                  uint32_t qw[16]) {
    constexpr uint32_t R = ALPHA ? 5u : 11u;
    float k0 = __fsub_rn(e1[0], e0[0]), k1 = __fsub_rn(e1[1], e0[1]);
    float k2 = __fsub_rn(e1[2], e0[2]), k3 = __fsub_rn(e1[3], e0[3]);
    // the terms whose k component is exactly +0 are left out: ZW (normal
    // maps): both endpoints' blue and alpha are 255, k2 = k3 = +0; without
    // alpha both endpoints' alpha is forced to 255 (find_min_max), k3 = +0
    constexpr int NCH = ZW ? 2 : (ALPHA ? 4 : 3);
    const float kk2 = __fmaf_rn(k1, k1, __fmul_rn(k0, k0));
    const float kk = NCH == 2 ? kk2 : NCH == 3 ? __fmaf_rn(k2, k2, kk2) : dot4(k0, k1, k2, k3, k0, k1, k2, k3);
    if (shorter_than_small_value(kk)) {
#pragma unroll
        for (int i = 0; i < 16; ++i) qw[i] = 0u;
        return;
    }
    const float r = rnorm_from_dot(kk);
    k0 = __fmul_rn(k0, r); k1 = __fmul_rn(k1, r); k2 = __fmul_rn(k2, r); k3 = __fmul_rn(k3, r);
    float w[16];
    float minw = 1e31f, maxw = -1e31f;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float4 s = grid_sample<DIM, NCH>(st, i);
        const float x2 = __fmaf_rn(k1, __fsub_rn(s.y, e0[1]), __fmul_rn(k0, __fsub_rn(s.x, e0[0])));
        const float x = NCH == 2   ? x2
                        : NCH == 3 ? __fmaf_rn(k2, __fsub_rn(s.z, e0[2]), x2)
                                   : dot4(k0, k1, k2, k3, __fsub_rn(s.x, e0[0]), __fsub_rn(s.y, e0[1]),
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

// per-block pipeline (encode_block 510-550) over a texel store S
// (NORMAL: the ZW forms)
template <int DIM, bool ALPHA, bool NORMAL = false, class S>
__device__ __forceinline__ uint4 encode_block_fp32(const S& st, const uint8_t* trits) {
    constexpr int N = DIM * DIM;
    const float4 m = block_mean<N, NORMAL>(st);
    const float4 v = pca_axis<N, NORMAL>(st, m);
    float e0[4], e1[4];
    uint32_t q0[4], q1[4];
    find_min_max<N, ALPHA, NORMAL>(st, m, v, e0, e1, q0, q1);
    uint32_t qw[16];
    reference_weights<DIM, ALPHA, NORMAL>(st, e0, e1, qw);
    return assemble_block<ALPHA>(q0, q1, qw, trits);
}

}  // namespace astc
