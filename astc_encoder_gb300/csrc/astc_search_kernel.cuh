// astc_search_kernel.cuh -- the sm_103a kernel of the FP32 encoder's
// reference-defined alternatives to its fixed pipeline, included by the
// translation units that instantiate it (astc_encode_search.cu: the fixed
// mode with the max-accumulation axis, and the search from one fit;
// astc_encode_thorough.cu: both fits; astc_encode_partitions.cu and
// astc_encode_three.cu: the partition modes), so each compiles in parallel and
// gets its own register allocation:
//   axis   = ASTC_AXIS_MAX_ACCUMULATION: the endpoint fit the reference
//            shader defines but leaves commented out
//            (max_accumulation_pixel_direction, ASTC_Encode.hlsl:170-227, 515);
//   axis   = ASTC_AXIS_BEST with ASTC_QUALITY_SEARCH: both fits, the search
//            from the one whose fixed-mode block decodes with the smaller
//            error (the fixed mode with it has a kernel of its own,
//            astc_encode_best.cu);
//   quality = ASTC_QUALITY_SEARCH: the choose_best_quantmethod the shader
//            sketches at 524-526 -- every single-partition 4x4-grid mode,
//            scored by its exact decode (astc_pipeline_search.cuh);
//   quality = ASTC_QUALITY_THOROUGH: both fits, the search from the one
//            whose fixed-mode block decodes with the smaller error (the
//            PCA on ties), dual-plane candidates (astc_pipeline_dual.cuh);
//   quality = ASTC_QUALITY_PARTITIONS: THOROUGH plus two-partition
//            candidates (astc_pipeline_partition.cuh);
//   quality = ASTC_QUALITY_THREE_PARTITIONS: PARTITIONS plus three-partition
//            candidates for RGB blocks (astc_pipeline_partition3.cuh).
// One thread encodes one block.  Texels stay packed (one register each) and
// are re-decoded per pass, which keeps the 36-texel 6x6 search in registers.
// Compile including units with --fmad=false: blocks are bit-identical to the
// FP32 oracle.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "astc_internal.h"
#include "astc_pipeline_dual.cuh"
#include "astc_pipeline_partition.cuh"
#include "astc_pipeline_partition3.cuh"

namespace astc {
namespace {

constexpr int kSearchThreads = 128;

__device__ const SearchTables g_search = make_search_tables();
__device__ const SrgbBits g_srgb_bits_s = make_srgb_bits();
struct PartitionClasses {
    uint32_t c4[kPartition2Classes4x4Count];   // as in PartSmem
    uint64_t c6[kPartition2Classes6x6Count];
};
constexpr PartitionClasses make_partition_classes() {
    PartitionClasses p{};
    for (int i = 0; i < kPartition2Classes4x4Count; ++i) p.c4[i] = kPartition2Classes4x4[i];
    for (int i = 0; i < kPartition2Classes6x6Count; ++i) p.c6[i] = kPartition2Classes6x6[i];
    return p;
}
__device__ const PartitionClasses g_classes = make_partition_classes();
constexpr Partition3Classes make_partition3_classes() {
    Partition3Classes p{};
    for (int i = 0; i < kPartition3Classes4x4Count; ++i) p.c4[i] = kPartition3Classes4x4[i];
    for (int i = 0; i < kPartition3Classes6x6Count; ++i) {
        p.c6a[i] = kPartition3Classes6x6A[i];
        p.c6b[i] = kPartition3Classes6x6B[i];
    }
    return p;
}
__device__ const Partition3Classes g_classes3 = make_partition3_classes();

struct SearchLaunch {
    TextureView tex;
    long long nblocks;
    uint4* out;
    int axis;     // 0 = PCA, 1 = max accumulation (the kernels with both fits ignore it)
    int search;   // 0 = fixed mode, 1 = the weight-range search
    int dual;     // dual-plane candidates (THOROUGH and above)
};

template <bool ALPHA>
__device__ __forceinline__ void load_dual_smem(DualSmem& ds) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&g_search.color[2][ALPHA][0][0]);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&ds.color[0][0]);
    const int words = g_search.nslots[2][ALPHA] * 128;
    for (int i = tid; i < words; i += nt) dst[i] = src[i];
    if (tid < 12) {
        ds.cq[tid] = g_search.cq[2][ALPHA][tid];
        ds.slot[tid] = g_search.slot[2][ALPHA][tid];
    }
}

__device__ __forceinline__ void load_part3_smem(Part3Smem& p3) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&g_search.color[3][0][0][0]);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&p3.color[0][0]);
    const int words = g_search.nslots[3][0] * 128;
    for (int i = tid; i < words; i += nt) dst[i] = src[i];
    if (tid < 12) {
        p3.cq[tid] = g_search.cq[3][0][tid];
        p3.slot[tid] = g_search.slot[3][0][tid];
    }
}

template <bool ALPHA>
__device__ __forceinline__ void load_partition_smem(PartSmem& pm, int dim) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&g_search.color[1][ALPHA][0][0]);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&pm.color[0][0]);
    const int words = g_search.nslots[1][ALPHA] * 128;
    for (int i = tid; i < words; i += nt) dst[i] = src[i];
    const int n = dim == 6 ? kPartition2Classes6x6Count : kPartition2Classes4x4Count;
    for (int i = tid; i < n; i += nt) {
        if (dim == 6) pm.classes.c6[i] = g_classes.c6[i];
        else pm.classes.c4[i] = g_classes.c4[i];
    }
    if (tid < 12) {
        pm.cq[tid] = g_search.cq[1][ALPHA][tid];
        pm.slot[tid] = g_search.slot[1][ALPHA][tid];
    }
    if (tid == 0) pm.nclasses = n;
}

template <bool ALPHA, bool SRGB>
__device__ __forceinline__ void load_search_smem(SearchSmem& sm) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&g_search.color[0][ALPHA][0][0]);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&sm.color[0][0]);
    const int words = g_search.nslots[0][ALPHA] * 128;
    for (int i = tid; i < words; i += nt) dst[i] = src[i];
    for (int i = tid; i < 12 * 32; i += nt) {
        sm.wval[i >> 5][i & 31] = g_search.wval[i >> 5][i & 31];
        sm.scramble[i >> 5][i & 31] = g_search.scramble[i >> 5][i & 31];
    }
    for (int i = tid; i < 256; i += nt) {
        sm.trits[i] = g_search.trit_pack[i];
        if (i < 128) sm.quints[i] = g_search.quint_pack[i];
        if (SRGB) {
            const float v = __uint_as_float(g_srgb_bits_s.v[i]);
            sm.lut[i] = v;
            sm.tbyte[i] = (uint8_t)rint_u32(v);
        }
    }
    if (tid < 12) {
        sm.cq[tid] = g_search.cq[0][ALPHA][tid];
        sm.slot[tid] = g_search.slot[0][ALPHA][tid];
        sm.wmax[tid] = (float)(quant_levels(tid) - 1);
    }
}

// Endpoint fit on `axis` and the fixed-mode block (encode_block 510-550);
// normal maps take the ZW forms (both axes have zero blue and alpha).
template <int DIM, bool ALPHA, bool NORMAL, class S>
__device__ __forceinline__ uint4 fit_fixed(const S& st, int axis, uint32_t q0[4], uint32_t q1[4],
                                           uint32_t qw[16], const uint8_t* trits) {
    constexpr int N = DIM * DIM;
    const float4 m = block_mean<N, NORMAL>(st);
    const float4 v = axis ? max_accumulation_axis<N, ALPHA>(st, m) : pca_axis<N, NORMAL>(st, m);
    float e0[4], e1[4];
    find_min_max<N, ALPHA, NORMAL>(st, m, v, e0, e1, q0, q1);
    reference_weights<DIM, ALPHA, NORMAL>(st, e0, e1, qw);
    return assemble_block<ALPHA>(q0, q1, qw, trits);
}

// Keeps, of two fits, the one whose fixed-mode block decodes with the
// smaller error (the first on ties).  The second fit is carried as its block
// (its QUANT_256 endpoints are bits 17.. in r0 r1 g0 g1 b0 b1 a0 a1 order)
// and its weights packed 4 bits each.
template <int DIM, bool ALPHA, bool SRGB>
__device__ __forceinline__ void pick_fit(const uint32_t (&tw)[DIM * DIM], const SearchSmem& sm, uint32_t q0[4],
                                         uint32_t q1[4], uint32_t qw[16], uint4& fixed, const uint4 fixed_b,
                                         uint64_t rw_packed) {
    typedef BlockError<DIM, ALPHA, SRGB> Err;
    constexpr int WQ0 = ALPHA ? kQuant6 : kQuant12;
    const uint32_t t2 = Err::target_sq(tw);
    const uint64_t ep = (((uint64_t)fixed_b.y << 32 | fixed_b.x) >> 17) | (((uint64_t)fixed_b.w << 32 | fixed_b.z) << 47);
    uint32_t r0[4], r1[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        r0[c] = (ALPHA || c < 3) ? (uint32_t)(ep >> (16 * c)) & 0xFFu : 255u;
        r1[c] = (ALPHA || c < 3) ? (uint32_t)(ep >> (16 * c + 8)) & 0xFFu : 255u;
    }
    // both fits scored by one copy of the scoring code
    uint32_t ea = 0;
    bool take_b = false;
#pragma unroll 1
    for (int f = 0; f < 2; ++f) {
        int E0[4], E1[4], W[16];
#pragma unroll
        for (int c = 0; c < 4; ++c) { E0[c] = (int)(f ? r0[c] : q0[c]); E1[c] = (int)(f ? r1[c] : q1[c]); }
#pragma unroll
        for (int g = 0; g < 16; ++g)
            W[g] = sm.wval[WQ0][f ? (uint32_t)(rw_packed >> (4 * g)) & 0xFu : qw[g]];
        const uint32_t e = Err::eval(tw, t2, E0, E1, W);
        if (f == 0) ea = e;
        else take_b = e < ea;
    }
    if (take_b) {
#pragma unroll
        for (int c = 0; c < 4; ++c) { q0[c] = r0[c]; q1[c] = r1[c]; }
#pragma unroll
        for (int g = 0; g < 16; ++g) qw[g] = (uint32_t)(rw_packed >> (4 * g)) & 0xFu;
        fixed = fixed_b;
    }
}

// MODE 0: fixed mode (max-accumulation axis) or SEARCH from one fit; 1: both
// fits (ASTC_AXIS_BEST: the fixed mode or the search from the better;
// THOROUGH: the search and dual-plane candidates); 2: THOROUGH plus
// two-partition candidates; 3 (RGB only): 2 plus three-partition candidates.
template <int DIM, bool ALPHA, bool NORMAL, bool SRGB, int MODE>
__global__ void __launch_bounds__(kSearchThreads, 3) astc_encode_blocks_search(const SearchLaunch p) {
    constexpr int N = DIM * DIM;
    constexpr bool thorough = MODE >= 1;
    __shared__ SearchSmem sm;
    static_assert(MODE != 3 || !ALPHA, "three RGBA partitions exceed the format's 18 endpoint values");
    __shared__ typename std::conditional<(MODE >= 2), PartSmem, char>::type pm;
    __shared__ typename std::conditional<(MODE >= 1), DualSmem, char>::type ds;
    __shared__ typename std::conditional<MODE == 3, Part3Smem, char>::type p3;
    // the tables are read-only device constants: loaded before the wait
    load_search_smem<ALPHA, SRGB>(sm);
    if constexpr (MODE >= 1) load_dual_smem<ALPHA>(ds);
    if constexpr (MODE >= 2) load_partition_smem<ALPHA>(pm, DIM);
    if constexpr (MODE == 3) load_part3_smem(p3);
    __syncthreads();
    pdl_wait_prior();
    pdl_allow_next();
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblocks) return;
    int bx, by;
    block_coords(p.tex, b, bx, by);
    uint32_t px[N];
    load_block_packed<DIM>(p.tex, bx, by, px);
    const PackedTexels<N, SRGB, NORMAL> st{px, sm.lut};
    uint32_t q0[4], q1[4], qw[16];
    uint4 fixed = fit_fixed<DIM, ALPHA, NORMAL>(st, thorough ? 0 : p.axis, q0, q1, qw, sm.trits);
    if (!thorough && !p.search) {
        p.out[b] = fixed;
        return;
    }
    uint4 fixed_b = fixed;
    uint64_t rw_packed = 0;
    if constexpr (thorough) {
        uint32_t r0[4], r1[4], rw[16];
        fixed_b = fit_fixed<DIM, ALPHA, NORMAL>(st, 1, r0, r1, rw, sm.trits);
#pragma unroll
        for (int g = 0; g < 16; ++g) rw_packed |= (uint64_t)rw[g] << (4 * g);
    }
    // the 16 grid-point colours every candidate projects: registers for 4x4,
    // a [point][thread] shared array for 6x6 (whose 36 target words and the
    // scoring loop already fill the register budget); then the texels as
    // the bytes the scoring compares with
    uint32_t tw[N];
    uint4 blk;
    uint32_t err = 0;
    if constexpr (DIM == 6) {
#pragma unroll
        for (int k = 0; k < N; ++k) tw[k] = target_word<ALPHA, NORMAL, SRGB>(px[k], sm.tbyte);
        if constexpr (thorough) {
            pick_fit<DIM, ALPHA, SRGB>(tw, sm, q0, q1, qw, fixed, fixed_b, rw_packed);
            if (!p.search) {                       // ASTC_AXIS_BEST, fixed mode
                p.out[b] = fixed;
                return;
            }
        }
        extern __shared__ float4 s_grid[];
        SharedTexels<16> grid{s_grid + threadIdx.x, (int)blockDim.x};
#pragma unroll
        for (int g = 0; g < 16; ++g) grid.put(g, grid_sample<DIM>(st, g));
        blk = search_block<DIM, ALPHA, SRGB>(grid, tw, q0, q1, qw, fixed, sm, &err);
        // an exact block stays: later candidates must decode with less error
        if (err == 0) {
            p.out[b] = blk;
            return;
        }
        if constexpr (thorough)
            if (p.dual)
                blk = dual_plane_block<DIM, ALPHA, SRGB>(st, grid, tw, BlockError<DIM, ALPHA, SRGB>::target_sq(tw),
                                                         err, blk, sm, ds);
        if constexpr (MODE >= 2) {
            // the partition candidates' per-texel weights, [texel][thread],
            // after the grid colours: a region of their own, since their float
            // columns would cross other threads' float4 grid columns (other
            // warps can still be reading theirs)
            SharedFloats<36> tws{reinterpret_cast<float*>(s_grid + 16 * blockDim.x) + threadIdx.x, (int)blockDim.x};
            blk = two_partition_block<DIM, ALPHA, SRGB>(st, tw, BlockError<DIM, ALPHA, SRGB>::target_sq(tw), q0,
                                                        q1, err, blk, sm, pm, tws);
            if constexpr (MODE == 3)
                if (err != 0)
                    blk = three_partition_block<DIM, SRGB>(st, tw, BlockError<DIM, ALPHA, SRGB>::target_sq(tw), err,
                                                           blk, sm, p3, g_classes3, tws);
        }
    } else {
#pragma unroll
        for (int k = 0; k < N; ++k) tw[k] = target_word<ALPHA, NORMAL, SRGB>(px[k], sm.tbyte);
        if constexpr (thorough) {
            pick_fit<DIM, ALPHA, SRGB>(tw, sm, q0, q1, qw, fixed, fixed_b, rw_packed);
            if (!p.search) {                       // ASTC_AXIS_BEST, fixed mode
                p.out[b] = fixed;
                return;
            }
        }
        RegTexels<16> grid;
#pragma unroll
        for (int g = 0; g < 16; ++g) grid.put(g, grid_sample<DIM>(st, g));
        blk = search_block<DIM, ALPHA, SRGB>(grid, tw, q0, q1, qw, fixed, sm, &err);
        if (err == 0) {
            p.out[b] = blk;
            return;
        }
        if constexpr (thorough)
            if (p.dual)
                blk = dual_plane_block<DIM, ALPHA, SRGB>(st, grid, tw, BlockError<DIM, ALPHA, SRGB>::target_sq(tw),
                                                         err, blk, sm, ds);
        if constexpr (MODE >= 2) {
            char none = 0;
            blk = two_partition_block<DIM, ALPHA, SRGB>(st, tw, BlockError<DIM, ALPHA, SRGB>::target_sq(tw), q0,
                                                        q1, err, blk, sm, pm, none);
            if constexpr (MODE == 3)
                if (err != 0)
                    blk = three_partition_block<DIM, SRGB>(st, tw, BlockError<DIM, ALPHA, SRGB>::target_sq(tw), err,
                                                           blk, sm, p3, g_classes3, none);
        }
    }
    p.out[b] = blk;
}

template <int DIM, bool ALPHA, bool NORMAL, bool SRGB, int MODE>
cudaError_t launch_t(const SearchLaunch& p, cudaStream_t s) {
    const long long grid = (p.nblocks + kSearchThreads - 1) / kSearchThreads;
    // 6x6: the grid colours, and for partitions their per-texel weights
    const size_t per_thread = 16 * sizeof(float4) + (MODE >= 2 ? 36 * sizeof(float) : 0);
    const size_t smem = (DIM == 6 && p.search) ? per_thread * kSearchThreads : 0;
    auto* kernel = astc_encode_blocks_search<DIM, ALPHA, NORMAL, SRGB, MODE>;
    if (smem) {
        // with the dual-plane and two-partition tables the total passes the
        // 48 KB default (68.6 KB for two partitions: 3 CTAs still fit an SM);
        // the attribute is per device, so it is set on every launch (a
        // host-side call, against launches of 100+ us)
        const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return launch_pdl(kernel, (unsigned)grid, (unsigned)kSearchThreads, smem, s, p);
}

template <int MODE, int DIM, bool ALPHA, bool NORMAL>
cudaError_t launch_srgb(const SearchLaunch& p, bool srgb, cudaStream_t s) {
    return srgb ? launch_t<DIM, ALPHA, NORMAL, true, MODE>(p, s)
                : launch_t<DIM, ALPHA, NORMAL, false, MODE>(p, s);
}
template <int MODE, int DIM, bool ALPHA>
cudaError_t launch_norm(const SearchLaunch& p, bool normal, bool srgb, cudaStream_t s) {
    return normal ? launch_srgb<MODE, DIM, ALPHA, true>(p, srgb, s)
                  : launch_srgb<MODE, DIM, ALPHA, false>(p, srgb, s);
}
template <int MODE, int DIM>
cudaError_t launch_alpha(const SearchLaunch& p, bool alpha, bool normal, bool srgb, cudaStream_t s) {
    return alpha ? launch_norm<MODE, DIM, true>(p, normal, srgb, s)
                 : launch_norm<MODE, DIM, false>(p, normal, srgb, s);
}

// RGB_ONLY: instantiate the kernels without alpha only (the caller routes
// alpha elsewhere).
template <int MODE, bool RGB_ONLY = false>
cudaError_t launch_search_kernels(const EncodeJob& j, cudaStream_t stream) {
    SearchLaunch p;
    p.tex = make_view(j);
    p.nblocks = (long long)p.tex.nbx * blocks_y(j.height, j.block_dim);
    p.out = reinterpret_cast<uint4*>(j.out);
    p.axis = j.axis;
    p.search = j.quality == ASTC_QUALITY_FAST ? 0 : 1;
    p.dual = j.quality >= ASTC_QUALITY_THOROUGH ? 1 : 0;
    const bool alpha = j.has_alpha != 0, normal = j.is_normal != 0, srgb = j.srgb != 0;
    cudaError_t e;
    if constexpr (RGB_ONLY) {
        if (alpha) return cudaErrorInvalidValue;
        e = j.block_dim == 4 ? launch_norm<MODE, 4, false>(p, normal, srgb, stream)
                             : launch_norm<MODE, 6, false>(p, normal, srgb, stream);
    } else {
        e = j.block_dim == 4 ? launch_alpha<MODE, 4>(p, alpha, normal, srgb, stream)
                             : launch_alpha<MODE, 6>(p, alpha, normal, srgb, stream);
    }
    if (e == cudaSuccess) count_launches(1);
    return e;
}

}  // namespace
}  // namespace astc
