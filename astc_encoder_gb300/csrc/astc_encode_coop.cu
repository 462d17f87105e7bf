// astc_encode_coop.cu -- the cooperative mapping of the FP32 fixed-mode
// encoder: four lanes of a warp share one ASTC block, so a warp encodes eight
// blocks (the reference runs one block per thread, MainCS,
// niepp/astc_encoder ASTC_Encode.hlsl:553-582).
//
// A block's path through the pipeline is about 2.4x shorter than with one
// thread per block, at about 1.7x the instructions per block (the power
// iteration and the endpoint tail run on all four lanes), so the mapping pays
// where a launch holds fewer blocks than the GPU has thread slots: small
// textures and mip levels, which one thread per block leaves latency-bound.
// The autotuner (astc_tune.cu) measures it against the one-thread mappings
// for textures under one wave and installs whichever is faster.
//
// Blocks stay bit-identical to the FP32 oracle: every FP32 sum keeps the
// oracle's operand order inside one lane, and only exact operations (min,
// max, copies) cross lanes.
//   texel fetch    each lane loads whole rows of its block (one 128-bit load
//                  per 4x4 row, three 64-bit loads per 6x6 row), decodes them
//                  and stages them in a [texel][block] shared-memory tile
//   mean           lane c sums channel c over the texels in order (143-147)
//   covariance     lane l keeps three of the ten terms, each summed over the
//                  texels in order: l0 c00 c01 c02, l1 c11 c12 c13, l2 c22,
//                  l3 c33 c03 c23 (149-162); the products d_i * d_j are the
//                  oracle's (multiplication commutes exactly)
//   power iter.    every lane, the one-thread code (93-106)
//   find_min_max   lane l projects texels l, l+4, ...; min and max combine
//                  across the four lanes (exact in any order) (108-137)
//   weights        lane l projects grid points l, l+4, l+8, l+12 on the
//                  shared normalized axis; min/max combine across lanes,
//                  each lane quantises its own four (316-393)
//   assembly       the 16 weights are gathered (4-bit fields, one shuffle
//                  per lane) and every lane assembles; lane 0 stores
#include <cuda_runtime.h>
#include <stdint.h>

#include "astc_internal.h"
#include "astc_pipeline_fp32.cuh"

namespace astc {
namespace {

constexpr int kLanes = 4;

__constant__ TritPack c_trit_pack_c = make_trit_pack();
__constant__ SrgbBits c_srgb_bits_c = make_srgb_bits();

struct LaunchCoop {
    TextureView tex;
    long long nblocks;
    uint4* out;
};

// One row of a block's texels, with the border rule of load_block_packed
// (D3D11 out-of-bounds Load = 0, or edge clamp).
template <int DIM>
__device__ __forceinline__ void load_row(const TextureView& p, int x0, int y, bool inside, uint32_t (&px)[DIM]) {
    if (inside) {
        const uint8_t* row = p.in + (size_t)y * p.pitch + (size_t)x0 * 4;
        if (p.vec_ok) {
            if constexpr (DIM == 4) {
                const uint4 v = __ldg(reinterpret_cast<const uint4*>(row));
                px[0] = v.x; px[1] = v.y; px[2] = v.z; px[3] = v.w;
            } else {
                const uint2* q = reinterpret_cast<const uint2*>(row);
                const uint2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
                px[0] = a.x; px[1] = a.y; px[2] = b.x; px[3] = b.y; px[4] = c.x; px[5] = c.y;
            }
            return;
        }
        const uint32_t* q = reinterpret_cast<const uint32_t*>(row);
#pragma unroll
        for (int x = 0; x < DIM; ++x) px[x] = __ldg(q + x);
        return;
    }
#pragma unroll
    for (int x = 0; x < DIM; ++x) {
        int xx = x0 + x, yy = y;
        const bool in = xx < p.width && yy < p.height;
        uint32_t v = 0;
        if (in || p.clamp) {
            xx = xx < p.width ? xx : p.width - 1;
            yy = yy < p.height ? yy : p.height - 1;
            v = __ldg(reinterpret_cast<const uint32_t*>(p.in + (size_t)yy * p.pitch) + xx);
        }
        px[x] = v;
    }
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
__global__ void __launch_bounds__(256) astc_encode_blocks_coop(const LaunchCoop p) {
    constexpr int N = DIM * DIM;
    constexpr uint32_t kFull = 0xFFFFFFFFu;
    extern __shared__ float4 s_tile[];                 // [N][slots + 1]
    __shared__ uint8_t s_trits[256];
    __shared__ float s_lut[SRGB ? 256 : 1];
    load_cta_tables<SRGB>(c_trit_pack_c, c_srgb_bits_c, s_trits, s_lut);
    __syncthreads();
    pdl_wait_prior();
    pdl_allow_next();

    const int slots = (int)blockDim.x / kLanes;
    // one float4 of padding per texel row of the tile: the four lanes of a
    // block read four different texels of the same slot, which then fall in
    // different banks
    const int tstride = slots + 1;
    const int slot = (int)threadIdx.x / kLanes;
    const int lane = (int)threadIdx.x & (kLanes - 1);
    const int gbase = (int)(threadIdx.x & 31) & ~(kLanes - 1);        // first lane of the group
    const long long b_req = (long long)blockIdx.x * slots + slot;
    // groups past the end encode the last block again and store nothing, so
    // every lane of the warp takes part in every shuffle
    const long long b = b_req < p.nblocks ? b_req : p.nblocks - 1;
    int bx, by;
    block_coords(p.tex, b, bx, by);

    // fetch: lane l decodes rows l (and l + 4) into the tile
    {
        const int x0 = bx * DIM, y0 = by * DIM;
        const bool inside = x0 + DIM <= p.tex.width && y0 + DIM <= p.tex.height;
        for (int r = lane; r < DIM; r += kLanes) {
            uint32_t px[DIM];
            load_row<DIM>(p.tex, x0, y0 + r, inside, px);
#pragma unroll
            for (int x = 0; x < DIM; ++x)
                s_tile[(r * DIM + x) * tstride + slot] = decode_texel<SRGB, NORMAL>(px[x], s_lut);
        }
    }
    __syncwarp();
    const float* tf = reinterpret_cast<const float*>(s_tile);
    auto texel_f = [&](int k, int c) -> float { return tf[((k * tstride + slot) << 2) + c]; };

    // mean: lane c sums channel c (a constant 255 channel sums to exactly 255)
    float4 m;
    {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < N; ++k) acc = __fadd_rn(acc, texel_f(k, lane));
        const float mc = __fmul_rn(acc, 1.0f / (float)N);
        m.x = __shfl_sync(kFull, mc, gbase + 0);
        m.y = __shfl_sync(kFull, mc, gbase + 1);
        m.z = __shfl_sync(kFull, mc, gbase + 2);
        m.w = __shfl_sync(kFull, mc, gbase + 3);
    }

    // covariance: lane l accumulates d_l*d_l, d_l*d_cb, d_l*d_cc
    float4 v;
    {
        const int cb = lane == 0 ? 1 : lane == 1 ? 2 : lane == 2 ? 3 : 0;
        const int cc = lane == 0 ? 2 : lane == 1 ? 3 : lane == 2 ? 3 : 2;
        const float mm[4] = {m.x, m.y, m.z, m.w};
        float ma = mm[0], mb = mm[0], mcc = mm[0];
#pragma unroll
        for (int c = 1; c < 4; ++c) {
            ma = lane == c ? mm[c] : ma;
            mb = cb == c ? mm[c] : mb;
            mcc = cc == c ? mm[c] : mcc;
        }
        float A = 0.0f, B = 0.0f, C = 0.0f;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float da = __fsub_rn(texel_f(k, lane), ma);
            const float db = __fsub_rn(texel_f(k, cb), mb);
            const float dc = __fsub_rn(texel_f(k, cc), mcc);
            A = __fmaf_rn(da, da, A);
            B = __fmaf_rn(da, db, B);
            C = __fmaf_rn(da, dc, C);
        }
        constexpr float kInvN1 = 1.0f / (float)(N - 1);
        A = __fmul_rn(A, kInvN1);
        B = __fmul_rn(B, kInvN1);
        C = __fmul_rn(C, kInvN1);
        const float c00 = __shfl_sync(kFull, A, gbase + 0), c01 = __shfl_sync(kFull, B, gbase + 0);
        const float c02 = __shfl_sync(kFull, C, gbase + 0), c11 = __shfl_sync(kFull, A, gbase + 1);
        const float c12 = __shfl_sync(kFull, B, gbase + 1), c13 = __shfl_sync(kFull, C, gbase + 1);
        const float c22 = __shfl_sync(kFull, A, gbase + 2), c33 = __shfl_sync(kFull, A, gbase + 3);
        const float c03 = __shfl_sync(kFull, B, gbase + 3), c23 = __shfl_sync(kFull, C, gbase + 3);
        v = NORMAL ? power_iteration_zw(c00, c01, c11)
                   : power_iteration(c00, c01, c02, c03, c11, c12, c13, c22, c23, c33);
    }

    // find_min_max: lane l projects texels l, l+4, ...
    const SharedTexels<N> st{s_tile + slot, tstride};
    float e0[4], e1[4];
    uint32_t q0[4], q1[4];
    {
        float a = 1e31f, bb = -1e31f;
#pragma unroll
        for (int j = 0; j < (N + kLanes - 1) / kLanes; ++j) {
            const int k = j * kLanes + lane;
            if (k < N) {
                const float4 t = st.get(k);
                const float pr = NORMAL ? __fmaf_rn(__fsub_rn(t.y, m.y), v.y, __fmul_rn(__fsub_rn(t.x, m.x), v.x))
                                        : dot4(__fsub_rn(t.x, m.x), __fsub_rn(t.y, m.y), __fsub_rn(t.z, m.z),
                                               __fsub_rn(t.w, m.w), v.x, v.y, v.z, v.w);
                a = fminf(a, pr);
                bb = fmaxf(bb, pr);
            }
        }
        a = fminf(a, __shfl_xor_sync(kFull, a, 1));
        a = fminf(a, __shfl_xor_sync(kFull, a, 2));
        bb = fmaxf(bb, __shfl_xor_sync(kFull, bb, 1));
        bb = fmaxf(bb, __shfl_xor_sync(kFull, bb, 2));
        endpoints_from_range<ALPHA>(m, v, a, bb, e0, e1, q0, q1);
    }

    // weights: lane l projects grid points l, l+4, l+8, l+12
    constexpr uint32_t R = ALPHA ? 5u : 11u;
    uint32_t qw[16];
    {
        float k0 = __fsub_rn(e1[0], e0[0]), k1 = __fsub_rn(e1[1], e0[1]);
        float k2 = __fsub_rn(e1[2], e0[2]), k3 = __fsub_rn(e1[3], e0[3]);
        constexpr int NCH = NORMAL ? 2 : (ALPHA ? 4 : 3);
        const float kk2 = __fmaf_rn(k1, k1, __fmul_rn(k0, k0));
        const float kk = NCH == 2 ? kk2 : NCH == 3 ? __fmaf_rn(k2, k2, kk2) : dot4(k0, k1, k2, k3, k0, k1, k2, k3);
        // kk is a function of the shared endpoints, so the four lanes of a
        // group agree on `flat`; other groups of the warp may not, so every
        // shuffle runs outside the branches (xor 1 and 2 stay in the group)
        const bool flat = shorter_than_small_value(kk);
        float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float minw = 1e31f, maxw = -1e31f;
        if (!flat) {
            const float r = rnorm_from_dot(kk);
            k0 = __fmul_rn(k0, r); k1 = __fmul_rn(k1, r); k2 = __fmul_rn(k2, r); k3 = __fmul_rn(k3, r);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int g = j * kLanes + lane;
                const float4 s = grid_sample<DIM, NCH>(st, g);
                const float x2 = __fmaf_rn(k1, __fsub_rn(s.y, e0[1]), __fmul_rn(k0, __fsub_rn(s.x, e0[0])));
                const float x = NCH == 2   ? x2
                                : NCH == 3 ? __fmaf_rn(k2, __fsub_rn(s.z, e0[2]), x2)
                                           : dot4(k0, k1, k2, k3, __fsub_rn(s.x, e0[0]), __fsub_rn(s.y, e0[1]),
                                                  __fsub_rn(s.z, e0[2]), __fsub_rn(s.w, e0[3]));
                minw = fminf(x, minw);
                maxw = fmaxf(x, maxw);
                w[j] = x;
            }
        }
        minw = fminf(minw, __shfl_xor_sync(kFull, minw, 1));
        minw = fminf(minw, __shfl_xor_sync(kFull, minw, 2));
        maxw = fmaxf(maxw, __shfl_xor_sync(kFull, maxw, 1));
        maxw = fmaxf(maxw, __shfl_xor_sync(kFull, maxw, 2));
        uint32_t word = 0;                              // this lane's four weights, 4 bits each
        if (!flat) {
            const float inv = __frcp_rn(fmaxf(1e-5f, __fsub_rn(maxw, minw)));
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float wn = __fmul_rn(__fsub_rn(w[j], minw), inv);
                const uint32_t q = rint_u32(__fmul_rn(wn, (float)R));
                word |= (q < R ? q : R) << (4 * j);
            }
        }
        uint32_t words[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) words[l] = __shfl_sync(kFull, word, gbase + l);
#pragma unroll
        for (int i = 0; i < 16; ++i) qw[i] = (words[i & 3] >> (4 * (i >> 2))) & 0xFu;
    }
    const uint4 blk = assemble_block<ALPHA>(q0, q1, qw, s_trits);
    if (lane == 0 && b_req < p.nblocks) p.out[b] = blk;
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
cudaError_t launch_coop_t(const LaunchCoop& p, int threads, cudaStream_t s) {
    constexpr int N = DIM * DIM;
    const int slots = threads / kLanes;
    const size_t smem = (size_t)N * (slots + 1) * sizeof(float4);
    auto kern = astc_encode_blocks_coop<DIM, ALPHA, NORMAL, SRGB>;
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const long long grid = (p.nblocks + slots - 1) / slots;
    return launch_pdl(kern, (unsigned)grid, (unsigned)threads, smem, s, p);
}

template <int DIM, bool ALPHA, bool NORMAL>
cudaError_t coop_srgb(const LaunchCoop& p, bool srgb, int threads, cudaStream_t s) {
    return srgb ? launch_coop_t<DIM, ALPHA, NORMAL, true>(p, threads, s)
                : launch_coop_t<DIM, ALPHA, NORMAL, false>(p, threads, s);
}
template <int DIM, bool ALPHA>
cudaError_t coop_norm(const LaunchCoop& p, bool normal, bool srgb, int threads, cudaStream_t s) {
    return normal ? coop_srgb<DIM, ALPHA, true>(p, srgb, threads, s)
                  : coop_srgb<DIM, ALPHA, false>(p, srgb, threads, s);
}
template <int DIM>
cudaError_t coop_alpha(const LaunchCoop& p, bool alpha, bool normal, bool srgb, int threads, cudaStream_t s) {
    return alpha ? coop_norm<DIM, true>(p, normal, srgb, threads, s)
                 : coop_norm<DIM, false>(p, normal, srgb, threads, s);
}

}  // namespace

cudaError_t launch_encode_coop(const EncodeJob& j, int threads, cudaStream_t stream) {
    if (threads != 64 && threads != 128 && threads != 256) return cudaErrorInvalidValue;
    LaunchCoop p;
    p.tex = make_view(j);
    p.nblocks = (long long)p.tex.nbx * blocks_y(j.height, j.block_dim);
    p.out = reinterpret_cast<uint4*>(j.out);
    const bool alpha = j.has_alpha != 0, normal = j.is_normal != 0, srgb = j.srgb != 0;
    return j.block_dim == 4 ? coop_alpha<4>(p, alpha, normal, srgb, threads, stream)
                            : coop_alpha<6>(p, alpha, normal, srgb, threads, stream);
}

}  // namespace astc
