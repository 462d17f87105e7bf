// astc_encode_h2.cu -- plain (one launch per texture) kernels of the packed
// half2 pipeline (astc_pipeline_h2.cuh), precision ASTC_PRECISION_HALF2.
// One thread per ASTC block, as MainCS (niepp/astc_encoder
// ASTC_Encode.hlsl:553-582).
#include <cuda_runtime.h>
#include <stdint.h>

#include "astc_internal.h"
#include "astc_pipeline_h2.cuh"

namespace astc {
namespace {

constexpr int kH2Threads = 128;

__constant__ TritPack c_trit_pack_h2 = make_trit_pack();
__constant__ SrgbBits c_srgb_bits_h2 = make_srgb_bits();

struct LaunchH2 {
    TextureView tex;
    long long nblocks;
    uint4* out;
};

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
__global__ void __launch_bounds__(kH2Threads) astc_encode_blocks_h2(const LaunchH2 p) {
    constexpr int N = DIM * DIM;
    __shared__ uint8_t s_trits[256];
    __shared__ uint8_t s_lin8[SRGB ? 256 : 1];
    load_cta_tables<false>(c_trit_pack_h2, c_srgb_bits_h2, s_trits, nullptr);
    if (SRGB) load_lin8_table(c_srgb_bits_h2, s_lin8);
    __syncthreads();
    pdl_wait_prior();
    pdl_allow_next();
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblocks) return;
    int bx, by;
    block_coords(p.tex, b, bx, by);
    uint32_t px[N];
    load_block_packed<DIM>(p.tex, bx, by, px);
    p.out[b] = encode_block_h2<DIM, ALPHA, NORMAL, SRGB>(px, s_lin8, s_trits);
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
cudaError_t launch_h2_t(const LaunchH2& p, cudaStream_t s) {
    const long long grid = (p.nblocks + kH2Threads - 1) / kH2Threads;
    return launch_pdl(astc_encode_blocks_h2<DIM, ALPHA, NORMAL, SRGB>, (unsigned)grid, kH2Threads, 0, s, p);
}

template <int DIM, bool ALPHA, bool NORMAL>
cudaError_t h2_srgb(const LaunchH2& p, bool srgb, cudaStream_t s) {
    return srgb ? launch_h2_t<DIM, ALPHA, NORMAL, true>(p, s) : launch_h2_t<DIM, ALPHA, NORMAL, false>(p, s);
}
template <int DIM, bool ALPHA>
cudaError_t h2_norm(const LaunchH2& p, bool normal, bool srgb, cudaStream_t s) {
    return normal ? h2_srgb<DIM, ALPHA, true>(p, srgb, s) : h2_srgb<DIM, ALPHA, false>(p, srgb, s);
}
template <int DIM>
cudaError_t h2_alpha(const LaunchH2& p, bool alpha, bool normal, bool srgb, cudaStream_t s) {
    return alpha ? h2_norm<DIM, true>(p, normal, srgb, s) : h2_norm<DIM, false>(p, normal, srgb, s);
}

}  // namespace

cudaError_t launch_encode_h2(const EncodeJob& j, cudaStream_t stream) {
    LaunchH2 p;
    p.tex = make_view(j);
    p.nblocks = (long long)p.tex.nbx * blocks_y(j.height, j.block_dim);
    p.out = reinterpret_cast<uint4*>(j.out);
    const bool alpha = j.has_alpha != 0, normal = j.is_normal != 0, srgb = j.srgb != 0;
    const cudaError_t e = j.block_dim == 4 ? h2_alpha<4>(p, alpha, normal, srgb, stream)
                                           : h2_alpha<6>(p, alpha, normal, srgb, stream);
    if (e == cudaSuccess) count_launches(1);
    return e;
}

}  // namespace astc
