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
// 64-bit shifts and the weight bit reversal is one __brevll.  Launches use
// programmatic dependent launch (launch_pdl): in a stream of encodes the next
// kernel's CTAs are resident and have their tables loaded when this one ends.
//
// Floating point follows the FP32 oracle's model operation by operation:
// mad = fused (__fmaf_rn), dot(a,b) = a.x*b.x then fused over y, z, w,
// normalize(v) = v * (1/sqrt(dot(v,v))) with correctly rounded sqrt and
// reciprocal, x/N for constant N = x * fl(1/N), round = half-to-even.  The
// file is compiled with --fmad=false so nothing else is contracted; blocks
// are therefore bit-identical to the oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "astc_pipeline_fp32.cuh"
#include "astc_internal.h"

namespace astc {
namespace {

constexpr int kMaxThreads = 256;

__constant__ TritPack c_trit_pack = make_trit_pack();
__constant__ SrgbBits c_srgb_bits = make_srgb_bits();

struct Launch {
    TextureView tex;
    long long nblocks;
    uint4* out;
};

// The shared-memory store caps registers (two 256-thread CTAs per SM, <= 128
// registers) so the compiler re-reads texels from shared memory instead of
// holding all of them in registers across the passes.
template <int DIM, bool ALPHA, bool NORMAL, bool SRGB, int STORE>
__global__ void __launch_bounds__(STORE == kStoreRegistersCapped ? 128 : kMaxThreads,
                                  STORE == kStoreShared ? 2 : (STORE == kStoreRegistersCapped ? 3 : 1))
astc_encode_blocks_fp32(const Launch p) {
    constexpr int N = DIM * DIM;
    extern __shared__ float4 s_texels[];                  // kStoreShared only
    __shared__ uint8_t s_trits[256];
    __shared__ float s_lut[SRGB ? 256 : 1];
    load_cta_tables<SRGB>(c_trit_pack, c_srgb_bits, s_trits, s_lut);
    __syncthreads();
    pdl_wait_prior();
    pdl_allow_next();
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblocks) return;
    int bx, by;
    block_coords(p.tex, b, bx, by);
    uint32_t px[N];
    load_block_packed<DIM>(p.tex, bx, by, px);
    if constexpr (STORE == kStoreShared) {
        SharedTexels<N> st{s_texels + threadIdx.x, (int)blockDim.x};
#pragma unroll
        for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
        p.out[b] = encode_block_fp32<DIM, ALPHA, NORMAL>(st, s_trits);
    } else {
        RegTexels<N> st;
#pragma unroll
        for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
        p.out[b] = encode_block_fp32<DIM, ALPHA, NORMAL>(st, s_trits);
    }
}

// Kernel choice per format and size class: texel store (or the cooperative
// mapping) and CTA size.  Size class 0 holds launches of fewer blocks than
// one wave of the one-thread mappings (SMs x 384 blocks), class 1 the rest.
// Defaults come from measurements on GB300 (profiles/); the autotuner may
// replace them.
struct Choice { int store; int threads; };
Choice g_choice[2][2][2][2][2] = {};     // [class][dim6][alpha][normal][srgb]
bool g_choice_init = false;
std::mutex g_choice_mu;

// GB300 sweep, launches overlapped, 8 distinct textures per step (us per
// launch; store/threads): 2048x2048 4x4 RGB shared/128 23.4, registers/128
// 24.9; 4x4 RGBA sRGB shared/128 23.8, registers/128 24.7; 4096x4096 4x4
// normal map registers/128 50.9, capped/128 50.9, shared/128 53.4; 2048x2048
// 6x6 RGBA sRGB capped/128 19.6, registers/128 23.0, shared/128 34.5; 6x6 RGB
// capped/128 19.2, registers/128 21.6; 4096x4096 6x6 normal map
// registers/128 41.1, capped/128 41.6.  The shared-memory store loses for 6x6
// (its re-reads cost more than the occupancy it gains); capping the register
// store at 168 (no spills) lifts 6x6 from 8 to 12 warps per SM.  Normal maps
// (two varying channels) fit in registers without the cap.
Choice default_choice(int cls, int dim, bool /*alpha*/, bool normal, bool /*srgb*/) {
    (void)cls;
    if (normal) return Choice{kStoreRegisters, 128};
    return dim == 6 ? Choice{kStoreRegistersCapped, 128} : Choice{kStoreShared, 128};
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
    return launch_pdl(kern, (unsigned)grid, (unsigned)threads, smem, s, p);
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB>
cudaError_t launch_store(const Launch& p, const Choice& c, cudaStream_t s) {
    if (c.store == kStoreShared)
        return launch_t<DIM, ALPHA, NORMAL, SRGB, kStoreShared>(p, c.threads, s);
    if (c.store == kStoreRegistersCapped)
        return launch_t<DIM, ALPHA, NORMAL, SRGB, kStoreRegistersCapped>(p, c.threads, s);
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

Choice current_choice(int cls, int dim, bool alpha, bool normal, bool srgb) {
    std::lock_guard<std::mutex> lk(g_choice_mu);
    if (!g_choice_init) {
        for (int c = 0; c < 2; ++c)
            for (int d = 0; d < 2; ++d)
                for (int a = 0; a < 2; ++a)
                    for (int n = 0; n < 2; ++n)
                        for (int r = 0; r < 2; ++r)
                            g_choice[c][d][a][n][r] = default_choice(c, d ? 6 : 4, a, n, r);
        g_choice_init = true;
    }
    return g_choice[cls][dim == 6][alpha][normal][srgb];
}

// SM count of the current device, cached per device index
int sm_count() {
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;
    }
    if (!cache[dev]) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            sms = 152;
        }
        cache[dev] = sms;
    }
    return cache[dev];
}

}  // namespace

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
    block_row_divisor(t.nbx, &t.row_mul, &t.row_shift);
    return t;
}

int encode_size_class(int width, int height, int block_dim) {
    const long long nb = (long long)blocks_x(width, block_dim) * blocks_y(height, block_dim);
    return nb < (long long)sm_count() * 384 ? 0 : 1;
}

cudaError_t launch_encode_variant(const EncodeJob& j, int store, int threads, cudaStream_t stream) {
    if (threads != 32 && threads != 64 && threads != 128 && threads != 256) return cudaErrorInvalidValue;
    if (store == kStoreCoop) {
        const cudaError_t e = launch_encode_coop(j, threads, stream);
        if (e == cudaSuccess) count_launches(1);
        return e;
    }
    if (store != kStoreRegisters && store != kStoreShared && store != kStoreRegistersCapped)
        return cudaErrorInvalidValue;
    if (store == kStoreRegistersCapped && threads > 128) return cudaErrorInvalidValue;
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
    const int cls = encode_size_class(j.width, j.height, j.block_dim);
    const Choice c = current_choice(cls, j.block_dim, j.has_alpha != 0, j.is_normal != 0, j.srgb != 0);
    return launch_encode_variant(j, c.store, c.threads, stream);
}

void set_encode_choice(int dim, bool alpha, bool normal, bool srgb, int store, int threads, int cls) {
    current_choice(0, dim, alpha, normal, srgb);
    std::lock_guard<std::mutex> lk(g_choice_mu);
    for (int c = 0; c < 2; ++c)
        if (cls < 0 || cls == c) g_choice[c][dim == 6][alpha][normal][srgb] = Choice{store, threads};
}

void get_encode_choice(int dim, bool alpha, bool normal, bool srgb, int* store, int* threads, int cls) {
    const Choice c = current_choice(cls, dim, alpha, normal, srgb);
    *store = c.store;
    *threads = c.threads;
}

}  // namespace astc
