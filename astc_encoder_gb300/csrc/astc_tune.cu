// astc_tune.cu -- autotuner for the encode kernel variants.
//
// Two mappings of blocks to threads: one thread per ASTC block (the
// reference's, ASTC_Encode.hlsl:553-561) with three ways to keep a block's
// decoded texels -- registers, a [texel][thread] shared-memory array, or
// registers with the count capped near 168 (6x6: 36 float4 per block
// otherwise hold the register count near 255 and the SM near 8 warps) -- and
// the cooperative mapping, four lanes per block (astc_encode_coop.cu), whose
// shorter per-block path pays for launches that do not fill the GPU.  The CTA
// size trades scheduling slack against shared memory.  astc_autotune times
// every (mapping/store, CTA size) candidate for a format on a synthetic
// texture of the caller's size on the current device and installs the
// fastest for that format and size class (under one wave of the one-thread
// mappings, or not) in this process -- unless it beats the current choice by
// less than 3%, which then stays (timing noise, e.g. under a profiler that
// serialises launches, does not move the choice).
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "astc_internal.h"

namespace astc {
namespace {

// Deterministic test texture: smooth gradients, hash noise and flat patches.
__global__ void astc_tune_fill(uint32_t* px, int w, int h) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)w * h) return;
    const int x = (int)(i % w), y = (int)(i / w);
    uint32_t s = (uint32_t)x * 0x9E3779B1u ^ (uint32_t)y * 0x85EBCA77u;
    s ^= s >> 15; s *= 0x2C1B3C6Du; s ^= s >> 12;
    const bool flat = ((x >> 5) + (y >> 5)) % 3 == 0;
    const uint32_t r = flat ? 90u : (uint32_t)((x + (s & 15)) & 255);
    const uint32_t g = flat ? 140u : (uint32_t)((y + ((s >> 4) & 15)) & 255);
    const uint32_t b = flat ? 200u : (uint32_t)((x + y + ((s >> 8) & 31)) & 255);
    const uint32_t a = ((x >> 4) & 1) ? 255u : (uint32_t)(((s >> 16) & 255));
    px[i] = r | (g << 8) | (b << 16) | (a << 24);
}

}  // namespace
}  // namespace astc

using namespace astc;

extern "C" {

astc_status astc_set_kernel_choice(int block_dim, int has_alpha, int is_normal, int srgb, int store,
                                   int threads) {
    if (block_dim != 4 && block_dim != 6) return set_error(ASTC_ERR_INVALID_ARG, "block_dim must be 4 or 6");
    if (store < 0 || store > 3) return set_error(ASTC_ERR_INVALID_ARG, "store must be 0, 1, 2 or 3");
    if (store == 2 && threads > 128)
        return set_error(ASTC_ERR_INVALID_ARG, "the capped-register store takes at most 128 threads");
    if (threads != 32 && threads != 64 && threads != 128 && threads != 256)
        return set_error(ASTC_ERR_INVALID_ARG, "threads must be 32, 64, 128 or 256");
    if (store == 3 && threads < 64)
        return set_error(ASTC_ERR_INVALID_ARG, "the cooperative mapping takes 64, 128 or 256 threads");
    set_encode_choice(block_dim, has_alpha != 0, is_normal != 0, srgb != 0, store, threads, -1);
    return ASTC_OK;
}

astc_status astc_get_kernel_choice_for_size(int block_dim, int has_alpha, int is_normal, int srgb, int width,
                                            int height, int* store, int* threads) {
    if (block_dim != 4 && block_dim != 6) return set_error(ASTC_ERR_INVALID_ARG, "block_dim must be 4 or 6");
    if (!store || !threads) return set_error(ASTC_ERR_INVALID_ARG, "NULL pointer");
    if (width <= 0 || height <= 0) return set_error(ASTC_ERR_INVALID_ARG, "bad size");
    get_encode_choice(block_dim, has_alpha != 0, is_normal != 0, srgb != 0, store, threads,
                      encode_size_class(width, height, block_dim));
    return ASTC_OK;
}

astc_status astc_get_kernel_choice(int block_dim, int has_alpha, int is_normal, int srgb, int* store,
                                   int* threads) {
    if (block_dim != 4 && block_dim != 6) return set_error(ASTC_ERR_INVALID_ARG, "block_dim must be 4 or 6");
    if (!store || !threads) return set_error(ASTC_ERR_INVALID_ARG, "NULL pointer");
    get_encode_choice(block_dim, has_alpha != 0, is_normal != 0, srgb != 0, store, threads, 1);
    return ASTC_OK;
}

astc_status astc_autotune(int block_dim, int has_alpha, int is_normal, int srgb, int width, int height,
                          astc_tune_result* result) {
    if (block_dim != 4 && block_dim != 6) return set_error(ASTC_ERR_INVALID_ARG, "block_dim must be 4 or 6");
    if (width <= 0 || height <= 0 || (long long)width * height > (1LL << 28))
        return set_error(ASTC_ERR_INVALID_ARG, "tuning texture must be 1..2^28 texels");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    const size_t in_bytes = (size_t)width * height * 4;
    const size_t out_bytes = astc_encoded_size(width, height, block_dim);
    uint8_t* d_in = nullptr;
    uint8_t* d_out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    astc_status st = ASTC_OK;
    do {
        if ((e = cudaMalloc(&d_in, in_bytes)) != cudaSuccess) { st = cuda_error(e, "cudaMalloc"); break; }
        if ((e = cudaMalloc(&d_out, out_bytes)) != cudaSuccess) { st = cuda_error(e, "cudaMalloc"); break; }
        if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) {
            st = cuda_error(e, "cudaStreamCreate");
            break;
        }
        if ((e = cudaEventCreate(&ev0)) != cudaSuccess || (e = cudaEventCreate(&ev1)) != cudaSuccess) {
            st = cuda_error(e, "cudaEventCreate");
            break;
        }
        const long long n = (long long)width * height;
        astc_tune_fill<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(reinterpret_cast<uint32_t*>(d_in), width,
                                                                   height);
        if ((e = cudaGetLastError()) != cudaSuccess) { st = cuda_error(e, "fill kernel"); break; }
        count_launches(1);
        EncodeJob job;
        job.in = d_in;
        job.pitch = (size_t)width * 4;
        job.width = width;
        job.height = height;
        job.block_dim = block_dim;
        job.has_alpha = has_alpha;
        job.is_normal = is_normal;
        job.srgb = srgb;
        job.border = ASTC_BORDER_CLAMP;
        job.precision = ASTC_PRECISION_FP32;
        job.out = d_out;
        const int cls = encode_size_class(width, height, block_dim);
        int def_store = 0, def_threads = 128;
        get_encode_choice(block_dim, has_alpha != 0, is_normal != 0, srgb != 0, &def_store, &def_threads, cls);
        const int stores[4] = {0, 1, 2, 3};
        const int sizes[3] = {64, 128, 256};
        float best = 1e30f, def_us = -1.0f;
        int best_store = def_store, best_threads = def_threads;
        for (int si = 0; si < 4 && st == ASTC_OK; ++si)
            for (int ti = 0; ti < 3 && st == ASTC_OK; ++ti) {
                if (stores[si] == 2 && sizes[ti] > 128) continue;      // capped store: <= 128 threads
                for (int w = 0; w < 2; ++w)
                    if ((e = launch_encode_variant(job, stores[si], sizes[ti], s)) != cudaSuccess) break;
                if (e != cudaSuccess) { st = cuda_error(e, "variant launch"); break; }
                // best of 3 bursts of 8 back-to-back launches: the queue runs
                // ahead of the GPU, so launch latency does not pad the timing
                constexpr int kBurst = 8;
                float ms_best = 1e30f;
                for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
                    cudaEventRecord(ev0, s);
                    for (int k = 0; k < kBurst && e == cudaSuccess; ++k)
                        e = launch_encode_variant(job, stores[si], sizes[ti], s);
                    if (e != cudaSuccess) break;
                    cudaEventRecord(ev1, s);
                    if ((e = cudaEventSynchronize(ev1)) != cudaSuccess) break;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, ev0, ev1);
                    ms /= kBurst;
                    ms_best = ms < ms_best ? ms : ms_best;
                }
                if (e != cudaSuccess) { st = cuda_error(e, "variant timing"); break; }
                const float us = ms_best * 1000.0f;
                if (stores[si] == def_store && sizes[ti] == def_threads) def_us = us;
                if (us < best) { best = us; best_store = stores[si]; best_threads = sizes[ti]; }
            }
        if (st != ASTC_OK) break;
        if (def_us > 0.0f && best > 0.97f * def_us) {
            best_store = def_store;
            best_threads = def_threads;
            best = def_us;
        }
        set_encode_choice(block_dim, has_alpha != 0, is_normal != 0, srgb != 0, best_store, best_threads, cls);
        if (result) {
            result->store = best_store;
            result->threads = best_threads;
            result->best_us = best;
            result->default_us = def_us;
        }
    } while (false);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (s) { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    if (d_in) cudaFree(d_in);
    if (d_out) cudaFree(d_out);
    return st;
}

}  // extern "C"
