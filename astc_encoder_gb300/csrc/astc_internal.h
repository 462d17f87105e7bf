// astc_internal.h -- declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

#include "../../include/astc_gb300.h"

namespace astc {

// One texture to encode, everything already on the device.
struct EncodeJob {
    const uint8_t* in;    // RGBA8, 4-byte aligned
    size_t pitch;         // bytes between rows, multiple of 4
    int width, height;
    int block_dim;        // 4 or 6
    int has_alpha, is_normal, srgb, border, precision;
    int axis = ASTC_AXIS_PCA, quality = ASTC_QUALITY_FAST;
    uint8_t* out;         // 16 * nblocks bytes, 16-byte aligned
};

// Launch with programmatic dependent launch (PDL): the kernel may be started
// while the previous kernel on the stream is still finishing, once every CTA
// of that kernel has passed its own wait and allowed it (pdl_allow_next); it
// loads its constant tables and then waits in pdl_wait_prior until the
// previous kernel has completed and its writes are visible, before it reads
// or writes any global memory.  Stream order is unchanged for every caller;
// what overlaps is the launch gap and the table set-up (a kernel that does not
// allow it, or a copy, delays the launch to its completion as usual).  On
// GB300 this took a 2048x2048 6x6 launch from 23.9 to 20.0 us in a stream of
// encodes.  While the stream is being captured into a graph the launch is a
// plain one (the waits then return at once).
template <class... P, class... A>
cudaError_t launch_pdl(void (*kern)(P...), unsigned grid, unsigned threads, size_t smem, cudaStream_t s,
                       A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    const cudaError_t e = cudaStreamIsCapturing(s, &capture);
    if (e != cudaSuccess) return e;
    cfg.attrs = attr;
    cfg.numAttrs = capture == cudaStreamCaptureStatusNone ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<A&&>(args)...);
}

inline int blocks_x(int w, int dim) { return (w + dim - 1) / dim; }
inline int blocks_y(int h, int dim) { return (h + dim - 1) / dim; }

// The cooperative mapping (four lanes per block; astc_encode_coop.cu),
// threads per CTA 64/128/256.
cudaError_t launch_encode_coop(const EncodeJob& job, int threads, cudaStream_t stream);

// Kernel launchers (astc_encode.cu).  Return cudaSuccess or the launch error.
cudaError_t launch_encode(const EncodeJob& job, cudaStream_t stream);
// One explicit kernel variant: store 0 = texels in registers, 1 = in shared
// memory; threads per CTA 32/64/128/256.
cudaError_t launch_encode_variant(const EncodeJob& job, int store, int threads, cudaStream_t stream);
// The variant launch_encode uses for a format (process-wide; set by the autotuner).
// Size class of a texture: 0 = fewer blocks than one wave of the
// one-thread-per-block mappings (SMs x 384), 1 = the rest.  Choices are kept
// per format and class; cls -1 in set_encode_choice sets both classes.
int encode_size_class(int width, int height, int block_dim);
void set_encode_choice(int dim, bool alpha, bool normal, bool srgb, int store, int threads, int cls);
void get_encode_choice(int dim, bool alpha, bool normal, bool srgb, int* store, int* threads, int cls);
struct TextureView;
TextureView make_view(const EncodeJob& job);
// Packed-half2 pipeline (astc_encode_h2.cu).
cudaError_t launch_encode_h2(const EncodeJob& job, cudaStream_t stream);
// FP32 with the max-accumulation axis and/or the mode search (astc_encode_search.cu);
// the search from the better of both fits (astc_encode_thorough.cu).
cudaError_t launch_encode_search(const EncodeJob& job, cudaStream_t stream);
cudaError_t launch_encode_thorough(const EncodeJob& job, cudaStream_t stream);
// THOROUGH plus two-partition candidates (astc_encode_partitions.cu).
cudaError_t launch_encode_partitions(const EncodeJob& job, cudaStream_t stream);
cudaError_t launch_encode_three(const EncodeJob& job, cudaStream_t stream);
cudaError_t launch_encode_best(const EncodeJob& job, cudaStream_t stream);

// Decoder / SSE launchers (astc_decode.cu).
cudaError_t launch_decode(const uint8_t* blocks, int width, int height, int bw, int bh,
                          int srgb, uint8_t* out, cudaStream_t stream);
cudaError_t launch_normal_sse(const uint8_t* a, const uint8_t* b, size_t texels, double* d_sse,
                              cudaStream_t stream);
cudaError_t launch_sse(const uint8_t* a, const uint8_t* b, size_t texels,
                       unsigned long long* d_sse4, cudaStream_t stream);

// Pointer checks (astc_capi.cu).  check_device_span accepts [p, p + bytes)
// when it is device memory of the current device or managed memory (and,
// with allow_host_view, the device view of pinned host memory), lying inside
// one allocation.  `seen` (may be NULL) collects the allocation ranges already
// checked, so a call that passes many pointers into the same allocations
// queries each allocation once; keep it for one call only (an address that is
// freed and reused between calls is checked again).
struct SpanCache {
    struct Range { uintptr_t lo, hi; };
    Range r[256];
    int n = 0;
    int last = 0;      // the range that matched last (pointers tend to repeat it)
};
astc_status check_device_span(const void* p, size_t bytes, const char* what, bool allow_host_view,
                              SpanCache* seen);

// Error plumbing (astc_capi.cu).
astc_status set_error(astc_status st, const std::string& msg);
astc_status cuda_error(cudaError_t e, const char* what);
void count_launches(uint64_t n);
// The address at which the current device reaches a host buffer: the device
// view of pinned memory (pinned = true), or the pointer itself for pageable
// memory on a device that reads the host's page tables; ptr NULL otherwise.
struct HostView {
    const void* ptr = nullptr;
    bool pinned = false;
};
HostView host_device_view(const void* host);
// Whether pageable host memory is accessed in place on the current device.
bool pageable_in_place_available();

}  // namespace astc
