// astc_sse.cuh -- per-channel sums of squared differences of two RGBA8
// images, the inner loop of astc_sse_gpu and astc_sse_gpu_noalloc.
//
// Four texel pairs at a time: the byte-wise absolute differences
// (__vabsdiffu4) are transposed into one word per channel and each channel's
// four squares summed by one __dp4a.  Sums are exact integers in any order;
// a thread's 32-bit partial sums are moved into 64-bit ones before they could
// wrap (every 4,096 rounds of four texels: at most 4 x 4,096 x 255^2 < 2^32).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace astc {

// byte c of words p0..p3 gathered into word c
__device__ __forceinline__ void transpose_bytes4(uint32_t p0, uint32_t p1, uint32_t p2, uint32_t p3, uint32_t& r,
                                                 uint32_t& g, uint32_t& b, uint32_t& a) {
    const uint32_t lo01 = __byte_perm(p0, p1, 0x5140);   // r0 r1 g0 g1
    const uint32_t hi01 = __byte_perm(p0, p1, 0x7362);   // b0 b1 a0 a1
    const uint32_t lo23 = __byte_perm(p2, p3, 0x5140);
    const uint32_t hi23 = __byte_perm(p2, p3, 0x7362);
    r = __byte_perm(lo01, lo23, 0x5410);
    g = __byte_perm(lo01, lo23, 0x7632);
    b = __byte_perm(hi01, hi23, 0x5410);
    a = __byte_perm(hi01, hi23, 0x7632);
}

struct SseAcc {
    uint32_t lo[4] = {0, 0, 0, 0};
    unsigned long long hi[4] = {0, 0, 0, 0};
    int rounds = 0;

    __device__ __forceinline__ void flush() {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            hi[c] += lo[c];
            lo[c] = 0;
        }
        rounds = 0;
    }
    __device__ __forceinline__ void add4(uint4 x, uint4 y) {
        uint32_t r, g, b, a;
        transpose_bytes4(__vabsdiffu4(x.x, y.x), __vabsdiffu4(x.y, y.y), __vabsdiffu4(x.z, y.z),
                         __vabsdiffu4(x.w, y.w), r, g, b, a);
        lo[0] = __dp4a(r, r, lo[0]);
        lo[1] = __dp4a(g, g, lo[1]);
        lo[2] = __dp4a(b, b, lo[2]);
        lo[3] = __dp4a(a, a, lo[3]);
        if (++rounds == 4096) flush();
    }
    __device__ __forceinline__ void add1(uint32_t x, uint32_t y) {
        const uint32_t d = __vabsdiffu4(x, y);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const uint32_t v = (d >> (8 * c)) & 0xFFu;
            lo[c] += v * v;
        }
        if (++rounds == 4096) flush();
    }
};

// Texels [begin, end) of a and b, thread `t` of `nt`: 16-byte loads (two
// in flight per round) when both images are 16-byte aligned at `begin`, else
// 4-byte loads.  begin is a multiple of 4 texels in the 16-byte case.
__device__ __forceinline__ void sse_range(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                                          size_t begin, size_t end, size_t t, size_t nt, SseAcc& acc) {
    const bool v16 = ((reinterpret_cast<uintptr_t>(a + begin) | reinterpret_cast<uintptr_t>(b + begin)) & 15u) == 0;
    size_t i = begin;
    if (v16) {
        const size_t quads = (end - begin) / 4;
        const uint4* a4 = reinterpret_cast<const uint4*>(a + begin);
        const uint4* b4 = reinterpret_cast<const uint4*>(b + begin);
        size_t q = t;
        for (; q + nt < quads; q += 2 * nt) {
            const uint4 x0 = __ldg(a4 + q), y0 = __ldg(b4 + q);
            const uint4 x1 = __ldg(a4 + q + nt), y1 = __ldg(b4 + q + nt);
            acc.add4(x0, y0);
            acc.add4(x1, y1);
        }
        if (q < quads) acc.add4(__ldg(a4 + q), __ldg(b4 + q));
        i = begin + quads * 4;
        for (size_t k = i + t; k < end; k += nt) acc.add1(__ldg(a + k), __ldg(b + k));
    } else {
        for (size_t k = i + t; k < end; k += nt) acc.add1(__ldg(a + k), __ldg(b + k));
    }
    acc.flush();
}

}  // namespace astc
