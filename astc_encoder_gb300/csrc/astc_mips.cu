// astc_mips.cu -- box-filtered mip chains on the GPU, the staging step in
// front of the batched encoder.  (The reference encodes a single level,
// main.cpp:33-36 sets MipLevels = 1; this fills the chain a texture pipeline
// encodes next to level 0.)
//
// Level l+1 has size max(1, floor(w_l / 2)) x max(1, floor(h_l / 2)); each of
// its texels is the rounded mean of the 2x2 texels (2x, 2y) .. (2x+1, 2y+1) of
// level l, with the second row/column clamped to the edge for a level of
// width or height 1.  With `srgb` the RGB channels are averaged in linear
// light (sRGB decode, mean, sRGB encode through a 4096-entry table) and alpha
// linearly.  Levels are written back to back in `out`, rows tightly packed.
// Up to six levels come from one launch (astc_mip_pyramid: 64x64 tiles
// reduced in shared memory), so a 2048x2048 chain takes two launches.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <mutex>

#include "astc_block_common.cuh"
#include "astc_internal.h"

namespace astc {
namespace {

struct MipTables {
    float to_linear[256];       // sRGB code -> linear [0, 1]
    uint8_t to_srgb[4096];      // linear quantised to 1/4095 -> nearest sRGB code
};

std::mutex g_mip_mu;
MipTables* g_mip_tables[64] = {};   // per device, created on first sRGB use, kept for the process

// One output texel from its 2x2 parents p0 (x0, y0), p1 (x1, y0), p2 (x0, y1),
// p3 (x1, y1): the rounded mean per channel, RGB in linear light for sRGB.
__device__ __forceinline__ uint32_t box_texel(uint32_t p0, uint32_t p1, uint32_t p2, uint32_t p3,
                                              const float* to_linear, const uint8_t* to_srgb, int srgb) {
    const uint32_t p[4] = {p0, p1, p2, p3};
    uint32_t out = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t v;
        if (srgb && c < 3) {
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k) s += to_linear[(p[k] >> (8 * c)) & 0xFF];
            const int q = min(4095, max(0, __float2int_rn(s * 0.25f * 4095.0f)));
            v = to_srgb[q];
        } else {
            uint32_t sum = 2;
#pragma unroll
            for (int k = 0; k < 4; ++k) sum += (p[k] >> (8 * c)) & 0xFF;
            v = sum >> 2;
        }
        out |= v << (8 * c);
    }
    return out;
}

// Up to six levels per launch from one base level: each CTA reads a 64x64
// tile of the base into shared memory once and reduces it level by level in
// shared memory (64 -> 32 -> ... -> 1), writing every level's texels of that
// tile; the next launch starts from the last level written.  A level's texel
// (x, y) needs texels 2x..2x+1, 2y..2y+1 of the level below, which lie in the
// same tile (clamped to the level's size where it is one texel wide or high).
constexpr int kPyrTile = 64;
constexpr int kPyrLevels = 6;
constexpr int kPyrThreads = 256;

struct PyrLevel {
    uint32_t* dst;
    int w, h;
};
struct PyrParams {
    const uint32_t* src;
    int sw, sh;
    int nlev;
    int tiles_x;                                  // tiles per row of the base level
    PyrLevel lev[kPyrLevels];
    const MipTables* tab;
    int srgb;
};

__global__ void __launch_bounds__(kPyrThreads) astc_mip_pyramid(const PyrParams p) {
    __shared__ uint32_t s_a[kPyrTile * kPyrTile];              // the base tile, then levels 2, 4
    __shared__ uint32_t s_b[(kPyrTile / 2) * (kPyrTile / 2)];  // levels 1, 3, 5
    __shared__ float s_lin[256];
    __shared__ __align__(4) uint8_t s_srgb[4096];
    if (p.srgb) {
        for (int i = threadIdx.x; i < 256; i += kPyrThreads) s_lin[i] = __ldg(&p.tab->to_linear[i]);
        const uint32_t* t4 = reinterpret_cast<const uint32_t*>(p.tab->to_srgb);
        for (int i = threadIdx.x; i < 1024; i += kPyrThreads)
            reinterpret_cast<uint32_t*>(s_srgb)[i] = __ldg(t4 + i);
    }
    // the tables are read-only: loaded before waiting for the previous kernel
    // on the stream (the level this launch starts from may be its output)
    pdl_wait_prior();
    pdl_allow_next();
    const int ty = (int)(blockIdx.x / (unsigned)p.tiles_x), tx = (int)blockIdx.x - ty * p.tiles_x;
    const int ox = tx * kPyrTile, oy = ty * kPyrTile;
    for (int i = threadIdx.x; i < kPyrTile * kPyrTile; i += kPyrThreads) {
        const int x = ox + (i & (kPyrTile - 1)), y = oy + i / kPyrTile;
        s_a[i] = (x < p.sw && y < p.sh) ? __ldg(p.src + (size_t)y * p.sw + x) : 0u;
    }
    __syncthreads();
    uint32_t* cur = s_a;
    uint32_t* nxt = s_b;
    int cw = p.sw, ch = p.sh, ct = kPyrTile;
    for (int l = 0; l < p.nlev; ++l) {
        const int nw = p.lev[l].w, nh = p.lev[l].h, nt = ct / 2;
        const int cox = ox >> l, coy = oy >> l;                 // tile origin at the current level
        const int nox = cox >> 1, noy = coy >> 1;               // and at the next
        for (int i = threadIdx.x; i < nt * nt; i += kPyrThreads) {
            const int lx = i % nt, ly = i / nt;
            const int x = nox + lx, y = noy + ly;
            if (x >= nw || y >= nh) continue;
            const int x0 = min(2 * x, cw - 1) - cox, x1 = min(2 * x + 1, cw - 1) - cox;
            const int y0 = min(2 * y, ch - 1) - coy, y1 = min(2 * y + 1, ch - 1) - coy;
            const uint32_t v = box_texel(cur[y0 * ct + x0], cur[y0 * ct + x1], cur[y1 * ct + x0], cur[y1 * ct + x1],
                                         s_lin, s_srgb, p.srgb);
            nxt[ly * nt + lx] = v;
            p.lev[l].dst[(size_t)y * nw + x] = v;
        }
        __syncthreads();
        uint32_t* t = cur;
        cur = nxt;
        nxt = t;
        cw = nw;
        ch = nh;
        ct = nt;
    }
}

}  // namespace
}  // namespace astc

using namespace astc;

extern "C" {

int astc_mip_levels(int width, int height) {
    if (width <= 0 || height <= 0) return 0;
    int levels = 1;
    while (width > 1 || height > 1) {
        width = width > 1 ? width / 2 : 1;
        height = height > 1 ? height / 2 : 1;
        ++levels;
    }
    return levels;
}

size_t astc_mip_chain_bytes(int width, int height, int levels) {
    size_t bytes = 0;
    for (int l = 1; l < levels && (width > 1 || height > 1); ++l) {
        width = width > 1 ? width / 2 : 1;
        height = height > 1 ? height / 2 : 1;
        bytes += (size_t)width * height * 4;
    }
    return bytes;
}

astc_status astc_generate_mips(const uint8_t* rgba8, int width, int height, int levels, int srgb,
                               uint8_t* out, void* stream) {
    if (!rgba8 || !out) return set_error(ASTC_ERR_INVALID_ARG, "NULL pointer");
    if (width <= 0 || height <= 0 || levels < 1 || levels > astc_mip_levels(width, height))
        return set_error(ASTC_ERR_INVALID_ARG, "levels must be 1..astc_mip_levels(width, height)");
    if (reinterpret_cast<uintptr_t>(rgba8) % 4 || reinterpret_cast<uintptr_t>(out) % 4)
        return set_error(ASTC_ERR_INVALID_ARG, "images must be 4-byte aligned");
    for (const void* p : {static_cast<const void*>(rgba8), static_cast<const void*>(out)}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess ||
            (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_error(ASTC_ERR_INVALID_ARG, "mip buffers must be device memory");
        }
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(ASTC_ERR_UNSUPPORTED, "device index out of range");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MipTables* s_tab = nullptr;
    std::lock_guard<std::mutex> lk(g_mip_mu);
    if (srgb && g_mip_tables[dev]) s_tab = g_mip_tables[dev];
    if (srgb && !s_tab) {
        MipTables h;
        for (int c = 0; c < 256; ++c) {
            const double x = c / 255.0;
            h.to_linear[c] = (float)(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4));
        }
        for (int q = 0; q < 4096; ++q) {
            const double l = q / 4095.0;
            const double v = l <= 0.0031308 ? l * 12.92 : 1.055 * std::pow(l, 1.0 / 2.4) - 0.055;
            const long c = std::lround(v * 255.0);
            h.to_srgb[q] = (uint8_t)(c < 0 ? 0 : c > 255 ? 255 : c);
        }
        MipTables* d = nullptr;
        if ((e = cudaMalloc(reinterpret_cast<void**>(&d), sizeof(MipTables))) != cudaSuccess)
            return cuda_error(e, "cudaMalloc of the sRGB mip tables");
        if ((e = cudaMemcpy(d, &h, sizeof(h), cudaMemcpyHostToDevice)) != cudaSuccess) {
            cudaFree(d);
            return cuda_error(e, "upload of the sRGB mip tables");
        }
        g_mip_tables[dev] = s_tab = d;
    }
    // levels 1..levels-1, up to six per launch, each launch starting from the
    // last level the previous one wrote
    const uint32_t* src = reinterpret_cast<const uint32_t*>(rgba8);
    uint32_t* dst = reinterpret_cast<uint32_t*>(out);
    int w = width, h = height;
    for (int l = 1; l < levels;) {
        PyrParams pp;
        pp.src = src;
        pp.sw = w;
        pp.sh = h;
        pp.tab = s_tab;
        pp.srgb = srgb ? 1 : 0;
        pp.nlev = 0;
        int lw = w, lh = h;
        while (pp.nlev < kPyrLevels && l < levels) {
            lw = lw > 1 ? lw / 2 : 1;
            lh = lh > 1 ? lh / 2 : 1;
            pp.lev[pp.nlev++] = PyrLevel{dst, lw, lh};
            dst += (size_t)lw * lh;
            ++l;
        }
        pp.tiles_x = (w + kPyrTile - 1) / kPyrTile;
        const long long tiles = (long long)pp.tiles_x * ((h + kPyrTile - 1) / kPyrTile);
        if ((e = launch_pdl(astc_mip_pyramid, (unsigned)tiles, kPyrThreads, 0, s, pp)) != cudaSuccess)
            return cuda_error(e, "mip kernel launch");
        count_launches(1);
        src = pp.lev[pp.nlev - 1].dst;
        w = lw;
        h = lh;
    }
    if (!stream && (e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_error(e, "mips");
    return ASTC_OK;
}

}  // extern "C"
