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
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <mutex>

#include "astc_internal.h"

namespace astc {
namespace {

struct MipTables {
    float to_linear[256];       // sRGB code -> linear [0, 1]
    uint8_t to_srgb[4096];      // linear quantised to 1/4095 -> nearest sRGB code
};

std::mutex g_mip_mu;
MipTables* g_mip_tables[64] = {};   // per device, created on first sRGB use, kept for the process

__global__ void astc_mip_box2x2(const uint32_t* __restrict__ src, int sw, int sh, uint32_t* __restrict__ dst,
                                int dw, int dh, const MipTables* __restrict__ tab, int srgb) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)dw * dh) return;
    const int x = (int)(i % dw), y = (int)(i / dw);
    const int x0 = min(2 * x, sw - 1), x1 = min(2 * x + 1, sw - 1);
    const int y0 = min(2 * y, sh - 1), y1 = min(2 * y + 1, sh - 1);
    const uint32_t p[4] = {__ldg(src + (size_t)y0 * sw + x0), __ldg(src + (size_t)y0 * sw + x1),
                           __ldg(src + (size_t)y1 * sw + x0), __ldg(src + (size_t)y1 * sw + x1)};
    uint32_t out = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t v;
        if (srgb && c < 3) {
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k) s += tab->to_linear[(p[k] >> (8 * c)) & 0xFF];
            const int q = min(4095, max(0, __float2int_rn(s * 0.25f * 4095.0f)));
            v = tab->to_srgb[q];
        } else {
            uint32_t s = 2;
#pragma unroll
            for (int k = 0; k < 4; ++k) s += (p[k] >> (8 * c)) & 0xFF;
            v = s >> 2;
        }
        out |= v << (8 * c);
    }
    dst[i] = out;
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
    const uint32_t* src = reinterpret_cast<const uint32_t*>(rgba8);
    uint32_t* dst = reinterpret_cast<uint32_t*>(out);
    int w = width, h = height;
    for (int l = 1; l < levels; ++l) {
        const int dw = w > 1 ? w / 2 : 1, dh = h > 1 ? h / 2 : 1;
        const long long n = (long long)dw * dh;
        astc_mip_box2x2<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, w, h, dst, dw, dh, s_tab, srgb);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "mip kernel launch");
        count_launches(1);
        src = dst;
        dst += n;
        w = dw;
        h = dh;
    }
    if (!stream && (e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_error(e, "mips");
    return ASTC_OK;
}

}  // extern "C"
