// astc_pipeline_h2.cuh -- the packed-half2 per-block pipeline (precision
// ASTC_PRECISION_HALF2).
//
// Same algorithm as the reference shader (niepp/astc_encoder ASTC_Encode.hlsl
// encode_block 510-550: PCA axis by 8 power iterations, min/max projection
// endpoints, 4x4-grid weights, QUANT_6/12 weights, QUANT_256 endpoints), with
// the arithmetic split by what each stage needs:
//   * mean and covariance: for UNORM8 input, exact integer sums -- four texels
//     are byte-transposed (8 byte_perms) and every sum and cross product is a
//     __dp4a -- so the covariance is exact up to one final FP32 rounding; for
//     sRGB input, one FP32 pass over the linearised values;
//   * power iteration, endpoint fit and rounding: FP32, with the hardware
//     reciprocal square root for the normalisations;
//   * per-texel projection (find_min_max) and weights: packed half2, two
//     channels per instruction, on differences (texel - mean, texel - the
//     endpoints' midpoint) so the values stay small and a rounding of the
//     reference point only shifts every texel by the same amount, which the
//     min/max normalisation removes; 0..255 texels are exact in FP16;
//   * weight quantisation: one half2 FMA plus the 1024 magic add (FP16 has
//     unit spacing at 1024, so the add rounds half to even).
// Blocks are not bit-identical to the FP32 oracle; the gate is PSNR against
// the FP64 oracle.
#pragma once
#include <cuda_fp16.h>

#include "astc_block_common.cuh"

namespace astc {

// Byte-transpose four RGBA8 texels into R, G, B, A words of four bytes each.
__device__ __forceinline__ void transpose4(uint32_t p0, uint32_t p1, uint32_t p2, uint32_t p3,
                                           uint32_t& r, uint32_t& g, uint32_t& b, uint32_t& a) {
    const uint32_t lo01 = __byte_perm(p0, p1, 0x5140);   // r0 r1 g0 g1
    const uint32_t hi01 = __byte_perm(p0, p1, 0x7362);   // b0 b1 a0 a1
    const uint32_t lo23 = __byte_perm(p2, p3, 0x5140);
    const uint32_t hi23 = __byte_perm(p2, p3, 0x7362);
    r = __byte_perm(lo01, lo23, 0x5410);
    g = __byte_perm(lo01, lo23, 0x7632);
    b = __byte_perm(hi01, hi23, 0x5410);
    a = __byte_perm(hi01, hi23, 0x7632);
}

// UNORM8 bytes (r, g) / (b, a) of a texel as exact half2: 0x64cc is 1024 + c.
__device__ __forceinline__ __half2 bytes_to_half2(uint32_t px, uint32_t sel) {
    const uint32_t bits = __byte_perm(px, 0x6464u, sel);
    __half2 h = *reinterpret_cast<const __half2*>(&bits);
    return __hsub2(h, __floats2half2_rn(1024.0f, 1024.0f));
}

// (p_i, p_j) = per-lane sums of two partial dot products s_i, s_j.
__device__ __forceinline__ __half2 pair_dot(__half2 s_i, __half2 s_j) {
    return __hadd2(__lows2half2(s_i, s_j), __highs2half2(s_i, s_j));
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
__device__ __forceinline__ uint4 encode_block_h2(const uint32_t (&px)[DIM * DIM], const float* lut,
                                                 const uint8_t* trits) {
    constexpr int N = DIM * DIM;
    float m0, m1, m2, m3;
    float c00, c01, c02, c03, c11, c12, c13, c22, c23, c33;
    __half2 trg[N], tba[N];                                // texels as (r,g), (b,a)

    if constexpr (!SRGB) {
        // exact integer moments: S_c and S_cd over the block
        uint32_t sr = 0, sg = 0, sb = 0, sa = 0;
        uint32_t srr = 0, srg = 0, srb = 0, sra = 0, sgg = 0, sgb = 0, sga = 0, sbb = 0, sba = 0, saa = 0;
#pragma unroll
        for (int k = 0; k < N; k += 4) {
            uint32_t r, g, b, a;
            transpose4(px[k], px[k + 1], px[k + 2], px[k + 3], r, g, b, a);
            sr = __dp4a(r, 0x01010101u, sr);
            sg = __dp4a(g, 0x01010101u, sg);
            srr = __dp4a(r, r, srr);
            srg = __dp4a(r, g, srg);
            sgg = __dp4a(g, g, sgg);
            if (!NORMAL) {
                sb = __dp4a(b, 0x01010101u, sb);
                srb = __dp4a(r, b, srb);
                sgb = __dp4a(g, b, sgb);
                sbb = __dp4a(b, b, sbb);
                sa = __dp4a(a, 0x01010101u, sa);
                sra = __dp4a(r, a, sra);
                sga = __dp4a(g, a, sga);
                sba = __dp4a(b, a, sba);
                saa = __dp4a(a, a, saa);
            }
        }
        constexpr float kInvN = 1.0f / (float)N;
        constexpr float kInvNN1 = 1.0f / ((float)N * (float)(N - 1));
        // cov_ij = (N*S_ij - S_i*S_j) / (N*(N-1)); the numerator is an exact int32
        auto cov = [&](uint32_t sij, uint32_t si, uint32_t sj) {
            return (float)((int)(N * sij) - (int)(si * sj)) * kInvNN1;
        };
        m0 = (float)sr * kInvN;
        m1 = (float)sg * kInvN;
        c00 = cov(srr, sr, sr); c01 = cov(srg, sr, sg); c11 = cov(sgg, sg, sg);
        if (NORMAL) {
            m2 = 255.0f; m3 = 255.0f;
            c02 = c03 = c12 = c13 = c22 = c23 = c33 = 0.0f;
        } else {
            m2 = (float)sb * kInvN;
            m3 = (float)sa * kInvN;
            c02 = cov(srb, sr, sb); c03 = cov(sra, sr, sa); c12 = cov(sgb, sg, sb);
            c13 = cov(sga, sg, sa); c22 = cov(sbb, sb, sb); c23 = cov(sba, sb, sa);
            c33 = cov(saa, sa, sa);
        }
#pragma unroll
        for (int k = 0; k < N; ++k) {
            trg[k] = bytes_to_half2(px[k], 0x4140u);
            tba[k] = NORMAL ? __floats2half2_rn(255.0f, 255.0f) : bytes_to_half2(px[k], 0x4342u);
        }
    } else {
        // sRGB: one FP32 pass over the linearised texels
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        float q00 = 0.f, q01 = 0.f, q02 = 0.f, q03 = 0.f, q11 = 0.f, q12 = 0.f, q13 = 0.f,
              q22 = 0.f, q23 = 0.f, q33 = 0.f;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float4 t = decode_texel<true, NORMAL>(px[k], lut);
            s0 += t.x; s1 += t.y; s2 += t.z; s3 += t.w;
            q00 = fmaf(t.x, t.x, q00); q01 = fmaf(t.x, t.y, q01); q02 = fmaf(t.x, t.z, q02);
            q03 = fmaf(t.x, t.w, q03); q11 = fmaf(t.y, t.y, q11); q12 = fmaf(t.y, t.z, q12);
            q13 = fmaf(t.y, t.w, q13); q22 = fmaf(t.z, t.z, q22); q23 = fmaf(t.z, t.w, q23);
            q33 = fmaf(t.w, t.w, q33);
            trg[k] = __floats2half2_rn(t.x, t.y);
            tba[k] = __floats2half2_rn(t.z, t.w);
        }
        constexpr float kInvN = 1.0f / (float)N;
        constexpr float kInvN1 = 1.0f / (float)(N - 1);
        m0 = s0 * kInvN; m1 = s1 * kInvN; m2 = s2 * kInvN; m3 = s3 * kInvN;
        c00 = (q00 - s0 * m0) * kInvN1; c01 = (q01 - s0 * m1) * kInvN1; c02 = (q02 - s0 * m2) * kInvN1;
        c03 = (q03 - s0 * m3) * kInvN1; c11 = (q11 - s1 * m1) * kInvN1; c12 = (q12 - s1 * m2) * kInvN1;
        c13 = (q13 - s1 * m3) * kInvN1; c22 = (q22 - s2 * m2) * kInvN1; c23 = (q23 - s2 * m3) * kInvN1;
        c33 = (q33 - s3 * m3) * kInvN1;
        if (NORMAL) { c02 = c03 = c12 = c13 = c22 = c23 = c33 = 0.0f; m2 = m3 = 255.0f; }
    }

    // power iteration (ASTC_Encode.hlsl:93-106), FP32, hardware rsqrt
    float v0 = 0.26726f, v1 = 0.80178f, v2 = 0.53452f, v3 = 0.0f;
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float t0 = dot4(c00, c01, c02, c03, v0, v1, v2, v3);
        float t1 = dot4(c01, c11, c12, c13, v0, v1, v2, v3);
        float t2 = dot4(c02, c12, c22, c23, v0, v1, v2, v3);
        float t3 = dot4(c03, c13, c23, c33, v0, v1, v2, v3);
        if (shorter_than_small_value(dot4(t0, t1, t2, t3, t0, t1, t2, t3))) {
            v0 = t0; v1 = t1; v2 = t2; v3 = t3;
            break;
        }
        const float u0 = dot4(c00, c01, c02, c03, t0, t1, t2, t3);
        const float u1 = dot4(c01, c11, c12, c13, t0, t1, t2, t3);
        const float u2 = dot4(c02, c12, c22, c23, t0, t1, t2, t3);
        const float u3 = dot4(c03, c13, c23, c33, t0, t1, t2, t3);
        const float r = rsqrtf(dot4(u0, u1, u2, u3, u0, u1, u2, u3));
        v0 = u0 * r; v1 = u1 * r; v2 = u2 * r; v3 = u3 * r;
    }

    // find_min_max (108-137): projections of (texel - mean) in half2
    const __half2 mrg = __floats2half2_rn(m0, m1), mba = __floats2half2_rn(m2, m3);
    const __half2 krg = __floats2half2_rn(v0, v1), kba = __floats2half2_rn(v2, v3);
    __half2 pmin = __floats2half2_rn(65504.0f, 65504.0f), pmax = __floats2half2_rn(-65504.0f, -65504.0f);
#pragma unroll
    for (int k = 0; k < N; k += 2) {
        __half2 si = __hmul2(__hsub2(trg[k], mrg), krg);
        __half2 sj = __hmul2(__hsub2(trg[k + 1], mrg), krg);
        if (!NORMAL) {
            si = __hfma2(__hsub2(tba[k], mba), kba, si);
            sj = __hfma2(__hsub2(tba[k + 1], mba), kba, sj);
        }
        const __half2 p = pair_dot(si, sj);
        pmin = __hmin2(pmin, p);
        pmax = __hmax2(pmax, p);
    }
    const float a = fminf(__low2float(pmin), __high2float(pmin));
    const float b = fmaxf(__low2float(pmax), __high2float(pmax));
    float e0[4], e1[4];
    const float mv[4] = {m0, m1, m2, m3}, vv[4] = {v0, v1, v2, v3};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        e0[c] = fminf(fmaxf(fmaf(vv[c], a, mv[c]), 0.0f), 255.0f);
        e1[c] = fminf(fmaxf(fmaf(vv[c], b, mv[c]), 0.0f), 255.0f);
    }
    uint32_t q0[4], q1[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) { q0[c] = rint_u32(e0[c]); q1[c] = rint_u32(e1[c]); }
    if (q0[0] + q0[1] + q0[2] > q1[0] + q1[1] + q1[2]) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float tf = e0[c]; e0[c] = e1[c]; e1[c] = tf;
            const uint32_t tq = q0[c]; q0[c] = q1[c]; q1[c] = tq;
        }
    }
    if (!ALPHA) { e0[3] = 255.0f; e1[3] = 255.0f; q0[3] = 255u; q1[3] = 255u; }

    // weights (316-393): dot(k, sample - e0) in half2, quantised in half2
    constexpr uint32_t R = ALPHA ? 5u : 11u;
    uint32_t qw[16];
    float k0 = e1[0] - e0[0], k1 = e1[1] - e0[1], k2 = e1[2] - e0[2], k3 = e1[3] - e0[3];
    const float kk = dot4(k0, k1, k2, k3, k0, k1, k2, k3);
    if (shorter_than_small_value(kk)) {
#pragma unroll
        for (int i = 0; i < 16; ++i) qw[i] = 0u;
    } else {
        const float r = rsqrtf(kk);
        const __half2 wrg = __floats2half2_rn(k0 * r, k1 * r), wba = __floats2half2_rn(k2 * r, k3 * r);
        // project relative to the endpoint midpoint: |w| <= range/2 halves the
        // FP16 rounding of every product; the shift is the same for all
        // samples, so the min/max normalisation removes it
        const __half2 erg = __floats2half2_rn(0.5f * (e0[0] + e1[0]), 0.5f * (e0[1] + e1[1]));
        const __half2 eba = __floats2half2_rn(0.5f * (e0[2] + e1[2]), 0.5f * (e0[3] + e1[3]));
        const bool use_ba = !NORMAL;                     // normal maps: e0.ba == e1.ba, k.b = k.a = 0
        __half2 wv[8];
        __half2 wmin = __floats2half2_rn(65504.0f, 65504.0f), wmax = __floats2half2_rn(-65504.0f, -65504.0f);
#pragma unroll
        for (int i = 0; i < 16; i += 2) {
            __half2 s[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int g = i + h;
                __half2 drg, dba;
                if constexpr (DIM == 6) {
                    const int i0 = grid_tap0(g);
                    float f00, f01, f10, f11;
                    grid_weights(g, f00, f01, f10, f11);
                    const __half2 h00 = __float2half2_rn(f00), h01 = __float2half2_rn(f01),
                                  h10 = __float2half2_rn(f10), h11 = __float2half2_rn(f11);
                    drg = __hmul2(__hsub2(trg[i0], erg), h00);
                    drg = __hfma2(__hsub2(trg[i0 + 1], erg), h01, drg);
                    drg = __hfma2(__hsub2(trg[i0 + 6], erg), h10, drg);
                    drg = __hfma2(__hsub2(trg[i0 + 7], erg), h11, drg);
                    if (use_ba) {
                        dba = __hmul2(__hsub2(tba[i0], eba), h00);
                        dba = __hfma2(__hsub2(tba[i0 + 1], eba), h01, dba);
                        dba = __hfma2(__hsub2(tba[i0 + 6], eba), h10, dba);
                        dba = __hfma2(__hsub2(tba[i0 + 7], eba), h11, dba);
                    }
                } else {
                    drg = __hsub2(trg[g], erg);
                    if (use_ba) dba = __hsub2(tba[g], eba);
                }
                s[h] = __hmul2(drg, wrg);
                if (use_ba) s[h] = __hfma2(dba, wba, s[h]);
            }
            const __half2 p = pair_dot(s[0], s[1]);
            wv[i / 2] = p;
            wmin = __hmin2(wmin, p);
            wmax = __hmax2(wmax, p);
        }
        const __half lo_h = __hmin(__low2half(wmin), __high2half(wmin));   // exact: one of the w
        const float lo = __half2float(lo_h);
        const float hi = fmaxf(__low2float(wmax), __high2float(wmax));
        // R / max(1e-5, range), kept inside the FP16 range (tiny ranges only
        // give tiny differences, so the clamp keeps every product below R)
        const float scale = fminf(__fdividef((float)R, fmaxf(1e-5f, hi - lo)), 65504.0f);
        // q = rint((w - lo) * scale): the fused 1024 + x rounds to an integer
        // half to even, because FP16 has unit spacing on [1024, 2048)
        const __half2 hs = __float2half2_rn(scale), h1024 = __float2half2_rn(1024.0f);
        const __half2 lo2 = __half2half2(lo_h);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const __half2 q = __hfma2(__hsub2(wv[i], lo2), hs, h1024);
            const uint32_t bits = *reinterpret_cast<const uint32_t*>(&q);
            const int ql = (int)(bits & 0xFFFFu) - 0x6400, qh = (int)(bits >> 16) - 0x6400;
            qw[2 * i] = (uint32_t)min(max(ql, 0), (int)R);
            qw[2 * i + 1] = (uint32_t)min(max(qh, 0), (int)R);
        }
    }
    return assemble_block<ALPHA>(q0, q1, qw, trits);
}

}  // namespace astc
