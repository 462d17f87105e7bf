// astc_encode_best.cu -- sm_103a kernel for ASTC_AXIS_BEST with the fixed
// mode: per block, both of the reference shader's endpoint fits (its
// principal_component_analysis, ASTC_Encode.hlsl:139-168, and the
// max_accumulation_pixel_direction it leaves commented out, 170-227, 515),
// each taken through the fixed-mode pipeline (encode_block 510-550), and the
// block whose decode has the smaller squared error against the texels rounded
// to bytes in the fit space is kept (the PCA block on ties) -- the choice the
// oracle's search makes before its weight ranges.
//
// The texels stay in registers as in the fixed-mode kernel (capped at 168
// registers, three 128-thread CTAs per SM); the error of a fixed-mode block is
// the exact integer decode (endpoints e * 257, or (e << 8) | 0x80 for sRGB;
// weights through the spec's unquantisation and, for 6x6, its 4x4-grid
// infill) against rint of the fit-space texels, summed with __vabsdiffu4 and
// __dp4a.  Compiled with --fmad=false: blocks are bit-identical to the oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include "astc_internal.h"
#include "astc_pipeline_fp32.cuh"

namespace astc {
namespace {

__constant__ TritPack c_trit_pack_best = make_trit_pack();
__constant__ SrgbBits c_srgb_bits_best = make_srgb_bits();

// Unquantised weights (0..64) of the fixed mode's two ranges, by value index.
struct FixedWeights { uint8_t q12[12]; uint8_t q6[6]; };
constexpr FixedWeights make_fixed_weights() {
    FixedWeights f{};
    const IseTables t = make_ise_tables();
    for (int i = 0; i < 12; ++i) f.q12[i] = t.weight_unq[kQuant12][t.scramble[kQuant12][i]];
    for (int i = 0; i < 6; ++i) f.q6[i] = t.weight_unq[kQuant6][t.scramble[kQuant6][i]];
    return f;
}
__constant__ FixedWeights c_fixed_weights = make_fixed_weights();

struct BestLaunch {
    TextureView tex;
    long long nblocks;
    uint4* out;
};

// Squared error of a fixed-mode block (endpoints q0/q1, value-order weights
// qw) against the texels of st rounded to bytes.
template <int DIM, bool ALPHA, bool SRGB, class S>
__device__ __forceinline__ uint32_t fixed_error(const S& st, const uint32_t q0[4], const uint32_t q1[4],
                                                const uint32_t (&qw)[16]) {
    constexpr int NCH = ALPHA ? 4 : 3;
    int base[NCH], delta[NCH];
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
        const int c0 = SRGB ? (int)((q0[c] << 8) | 0x80u) : (int)q0[c] * 257;
        const int c1 = SRGB ? (int)((q1[c] << 8) | 0x80u) : (int)q1[c] * 257;
        base[c] = 4 * (64 * c0 + 32);
        delta[c] = 4 * (c1 - c0);
    }
    int W[16];
#pragma unroll
    for (int g = 0; g < 16; ++g) W[g] = ALPHA ? c_fixed_weights.q6[qw[g]] : c_fixed_weights.q12[qw[g]];
    uint32_t err = 0;
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
        for (int c = 0; c < NCH; ++c) v[c] = (uint32_t)(base[c] + delta[c] * w);
        // byte 2 of each channel's value is its decoded UNORM8 (bytes 3 are 0)
        uint32_t dec = __byte_perm(v[0], v[1], 0x3362u);
        dec = __byte_perm(dec, v[2], 0x3610u);
        if constexpr (ALPHA) dec = __byte_perm(dec, v[3], 0x6210u);
        const float4 t = st.get(k);
        uint32_t tb = rint_u32(t.x) | (rint_u32(t.y) << 8) | (rint_u32(t.z) << 16);
        if constexpr (ALPHA) tb |= rint_u32(t.w) << 24;
        const uint32_t d = __vabsdiffu4(dec, tb);
        err = __dp4a(d, d, err);
    }
    return err;
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
__global__ void __launch_bounds__(128, 3) astc_encode_blocks_best(const BestLaunch p) {
    constexpr int N = DIM * DIM;
    __shared__ uint8_t s_trits[256];
    __shared__ float s_lut[SRGB ? 256 : 1];
    load_cta_tables<SRGB>(c_trit_pack_best, c_srgb_bits_best, s_trits, s_lut);
    __syncthreads();
    pdl_wait_prior();
    pdl_allow_next();
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblocks) return;
    int bx, by;
    block_coords(p.tex, b, bx, by);
    uint32_t px[N];
    load_block_packed<DIM>(p.tex, bx, by, px);
    RegTexels<N> st;
#pragma unroll
    for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
    const float4 m = block_mean<N, NORMAL>(st);
    uint4 best = make_uint4(0u, 0u, 0u, 0u);
    uint32_t best_err = 0;
#pragma unroll 1
    for (int axis = 0; axis < 2; ++axis) {
        const float4 v = axis ? max_accumulation_axis<N, ALPHA>(st, m) : pca_axis<N, NORMAL>(st, m);
        float e0[4], e1[4];
        uint32_t q0[4], q1[4], qw[16];
        find_min_max<N, ALPHA, NORMAL>(st, m, v, e0, e1, q0, q1);
        reference_weights<DIM, ALPHA, NORMAL>(st, e0, e1, qw);
        const uint32_t err = fixed_error<DIM, ALPHA, SRGB>(st, q0, q1, qw);
        if (axis == 0 || err < best_err) {
            best_err = err;
            best = assemble_block<ALPHA>(q0, q1, qw, s_trits);
        }
    }
    p.out[b] = best;
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
cudaError_t launch_t(const BestLaunch& p, cudaStream_t s) {
    const long long grid = (p.nblocks + 127) / 128;
    return launch_pdl(astc_encode_blocks_best<DIM, ALPHA, NORMAL, SRGB>, (unsigned)grid, 128u, 0, s, p);
}

template <int DIM, bool ALPHA, bool NORMAL>
cudaError_t launch_srgb(const BestLaunch& p, bool srgb, cudaStream_t s) {
    return srgb ? launch_t<DIM, ALPHA, NORMAL, true>(p, s) : launch_t<DIM, ALPHA, NORMAL, false>(p, s);
}
template <int DIM, bool ALPHA>
cudaError_t launch_norm(const BestLaunch& p, bool normal, bool srgb, cudaStream_t s) {
    return normal ? launch_srgb<DIM, ALPHA, true>(p, srgb, s) : launch_srgb<DIM, ALPHA, false>(p, srgb, s);
}
template <int DIM>
cudaError_t launch_alpha(const BestLaunch& p, bool alpha, bool normal, bool srgb, cudaStream_t s) {
    return alpha ? launch_norm<DIM, true>(p, normal, srgb, s) : launch_norm<DIM, false>(p, normal, srgb, s);
}

}  // namespace

cudaError_t launch_encode_best(const EncodeJob& j, cudaStream_t stream) {
    BestLaunch p;
    p.tex = make_view(j);
    p.nblocks = (long long)p.tex.nbx * blocks_y(j.height, j.block_dim);
    p.out = reinterpret_cast<uint4*>(j.out);
    const bool alpha = j.has_alpha != 0, normal = j.is_normal != 0, srgb = j.srgb != 0;
    const cudaError_t e = j.block_dim == 4 ? launch_alpha<4>(p, alpha, normal, srgb, stream)
                                           : launch_alpha<6>(p, alpha, normal, srgb, stream);
    if (e == cudaSuccess) count_launches(1);
    return e;
}

}  // namespace astc
