// astc_noalloc.cu -- astc_sse_gpu_noalloc: the per-channel SSE reduction of
// astc_sse_gpu, for callers that may not allocate device memory.
//
// Who needs it: applications that own the whole device-memory budget through
// their own allocator and forbid a library from allocating behind their back
// (game engines, texture-streaming and serving processes that admit work by
// memory), and real-time loops where a cudaMalloc/cudaFree would synchronise
// the device in the middle of a frame.  astc_sse_gpu allocates its
// accumulator (and, for host memory, staging) the first time it runs; this
// entry point allocates nothing.
//
// How: the scratch -- one partial sum (4 x u64) per chunk of texels (8,192
// or, for images above 2^25 texels, 1/4096 of the image rounded up to 1,024;
// at most 65,536), one CTA per chunk -- is a file-scope static __device__
// array of fixed size (4096 chunks, 128 KiB),
// which every GPU that loads this library holds until the process exits.  The
// inputs (two RGBA8 images in device memory) and the output (4 x u64 in device
// memory) are the caller's.  The first call on a device looks up the array's
// device address with cudaGetSymbolAddress (with that device current) and
// caches it; that first call should come before any stream capture.  All calls
// share the array: two calls whose kernels overlap on the GPU race on it.
// Each chunk's CTA overwrites its own partial and counts itself done in the
// array's last word; the CTA that counts last reads only the partials of the
// current call, writes the totals and sets the count back to zero, so one
// launch does the whole reduction.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "astc_block_common.cuh"
#include "astc_internal.h"
#include "astc_sse.cuh"

namespace astc {
namespace {

constexpr int kNoAllocMaxChunks = 4096;
constexpr size_t kNoAllocChunkTexels = size_t(1) << 16;                          // the largest chunk
constexpr size_t kNoAllocMinChunkTexels = size_t(1) << 13;
constexpr size_t kNoAllocMaxTexels = kNoAllocMaxChunks * kNoAllocChunkTexels;   // 2^28
constexpr int kNoAllocThreads = 256;

// the partials, then one counter: CTAs of the current call that have written
// theirs (the last one totals them and sets it back to zero)
static __device__ __align__(256) unsigned long long g_noalloc_partials[kNoAllocMaxChunks * 4 + 1];

constexpr int kMaxDevicesNoAlloc = 64;
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_ptr[kMaxDevicesNoAlloc] = {};

__device__ __forceinline__ unsigned long long block_sum(unsigned long long v, unsigned long long* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    unsigned long long s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kNoAllocThreads / 32; ++w) s += red[w];
    return s;
}

// One CTA per chunk of `chunk` texels (a multiple of 1,024): writes the
// chunk's R, G, B, A sums of squared differences, then counts itself done;
// the CTA that counts last totals every chunk's partials into `out` and sets
// the counter back to zero for the next call (the fence before the count
// makes each partial visible before it is counted).
__global__ void __launch_bounds__(kNoAllocThreads)
astc_sse_chunks_static(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, size_t n, size_t chunk,
                       unsigned long long* __restrict__ partials, unsigned long long* __restrict__ out) {
    __shared__ unsigned long long red[kNoAllocThreads / 32];
    __shared__ bool last;
    // a launch may start while the previous kernel on the stream finishes; the
    // scratch and the images are touched only after it has completed
    pdl_wait_prior();
    pdl_allow_next();
    const size_t begin = (size_t)blockIdx.x * chunk;
    const size_t end = begin + chunk < n ? begin + chunk : n;
    SseAcc acc;
    if (begin < end) sse_range(a, b, begin, end, threadIdx.x, kNoAllocThreads, acc);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const unsigned long long s = block_sum(acc.hi[c], red);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * 4 + c] = s;
    }
    unsigned long long* counter = partials + (size_t)kNoAllocMaxChunks * 4;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1ull) == (unsigned long long)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    unsigned long long tot[4] = {0, 0, 0, 0};
    for (unsigned i = threadIdx.x; i < gridDim.x; i += kNoAllocThreads)
#pragma unroll
        for (int c = 0; c < 4; ++c) tot[c] += __ldcg(partials + (size_t)i * 4 + c);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const unsigned long long s = block_sum(tot[c], red);
        if (threadIdx.x == 0) out[c] = s;
    }
    if (threadIdx.x == 0) *counter = 0ull;
}

astc_status noalloc_scratch(unsigned long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevicesNoAlloc)
        return set_error(ASTC_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);   // with `dev` current
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress of the static scratch");
        g_noalloc_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return ASTC_OK;
}

}  // namespace
}  // namespace astc

using namespace astc;

extern "C" astc_status astc_sse_gpu_noalloc(const uint8_t* a, const uint8_t* b, size_t texels,
                                            void* stream, uint64_t* sse_rgba) {
    try {
        if (!a || !b || !sse_rgba) return set_error(ASTC_ERR_INVALID_ARG, "NULL pointer");
        if (texels > kNoAllocMaxTexels)
            return set_error(ASTC_ERR_INVALID_ARG,
                             "astc_sse_gpu_noalloc: " + std::to_string(texels) +
                                 " texels exceed the static scratch limit of " +
                                 std::to_string(kNoAllocMaxTexels) +
                                 " (4096 chunks of 65536); use astc_sse_gpu");
        if (reinterpret_cast<uintptr_t>(a) % 4 || reinterpret_cast<uintptr_t>(b) % 4 ||
            reinterpret_cast<uintptr_t>(sse_rgba) % 8)
            return set_error(ASTC_ERR_INVALID_ARG,
                             "images must be 4-byte and the output 8-byte aligned");
        astc_status st;
        // device memory of the current device, each extent inside its allocation
        if ((st = check_device_span(a, texels * 4, "a", false, nullptr)) != ASTC_OK) return st;
        if ((st = check_device_span(b, texels * 4, "b", false, nullptr)) != ASTC_OK) return st;
        if ((st = check_device_span(sse_rgba, 4 * sizeof(uint64_t), "sse_rgba", false, nullptr)) != ASTC_OK)
            return st;
        unsigned long long* scratch = nullptr;
        if ((st = noalloc_scratch(&scratch)) != ASTC_OK) return st;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        // chunks of at least 8,192 texels, at most 4096 of them
        size_t chunk = (texels + kNoAllocMaxChunks - 1) / kNoAllocMaxChunks;
        chunk = (chunk + 1023) / 1024 * 1024;
        if (chunk < kNoAllocMinChunkTexels) chunk = kNoAllocMinChunkTexels;
        const int chunks = (int)((texels + chunk - 1) / chunk);
        // one CTA at least, so an empty call still writes its zero sums
        cudaError_t e = launch_pdl(astc_sse_chunks_static, (unsigned)(chunks > 0 ? chunks : 1), kNoAllocThreads, 0, s,
                                   reinterpret_cast<const uint32_t*>(a), reinterpret_cast<const uint32_t*>(b),
                                   texels, chunk, scratch, reinterpret_cast<unsigned long long*>(sse_rgba));
        if (e != cudaSuccess) return cuda_error(e, "sse kernel launch");
        count_launches(1);
        return ASTC_OK;
    } catch (...) {
        return set_error(ASTC_ERR_CUDA, "unexpected exception");
    }
}
