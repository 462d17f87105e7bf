// astc_capi.cu -- the C ABI (include/astc_gb300.h): argument checks, pooled
// device staging, host<->device copies, .astc file I/O and error reporting.
//
// Replaces the D3D11 host side of niepp/astc_encoder:
//   encode_astc        astc_encode.h:87-194 (SRV/UAV/cbuffer setup, grid
//                      math 124-134, Dispatch 190)  -> astc_encode_gpu
//   read_gpu           astc_save.h:34-50 (staging buffer + Map)
//                                                   -> cudaMemcpyAsync D2H
//   save_astc          astc_save.h:52-76            -> astc_save_file
// Unlike the reference, every failure returns a status (the reference leaked
// its D3D objects on each error path and never checked fopen).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <new>
#include <string>

#include "astc_internal.h"

namespace astc {
namespace {

thread_local std::string t_last_error;
std::atomic<uint64_t> g_launches{0};

// Upload ring for large host inputs the device reaches in place: the copy
// engine (pinned input) or a copy kernel (pageable input read through the
// host page tables) uploads the texture (in equal bands of whole block rows
// when it is larger than a slot) into kRingSlots device slots on the ring's
// own stream, while encode kernels on the caller's stream consume earlier
// uploads.  `filled[k]` (copy stream)
// orders a band's kernel after its upload, `drained[k]` (caller's stream)
// orders the slot's next upload after that kernel, so uploads run back to
// back across calls and the kernels hide under them: the host link stays busy
// instead of alternating between the kernels' load and compute phases.  On
// GB300 (2048x2048 6x6 RGBA, 16 calls per sync) the ring moves the host-memory
// path from 44.9 (in-place reads) to 49.5 Gtexel/s against a ~52 Gtexel/s
// link bound; smaller slots lose (8 MiB: 47.1, 2 MiB: 33.7) because each band
// costs a kernel launch of less than a wave.
constexpr int kRingSlots = 3;
constexpr size_t kRingSlotBytes = (size_t)32 << 20;
constexpr size_t kRingMinBytes = (size_t)4 << 20;   // smaller inputs are read in place

// Rows of a pageable host buffer that the device reads through the host's
// page tables, copied into a ring slot by the SMs: four independent T-sized
// loads per thread per round keep enough of the link's latency covered.
template <typename T>
__global__ void __launch_bounds__(256) astc_copy_rows(const uint8_t* __restrict__ src, size_t src_pitch,
                                                      uint8_t* __restrict__ dst, size_t dst_pitch,
                                                      size_t row_elems, size_t total) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += 4 * stride) {
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t k = i + u * stride;
            if (k < total) {
                const size_t r = k / row_elems;
                v[u] = reinterpret_cast<const T*>(src + r * src_pitch)[k - r * row_elems];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t k = i + u * stride;
            if (k < total) {
                const size_t r = k / row_elems;
                reinterpret_cast<T*>(dst + r * dst_pitch)[k - r * row_elems] = v[u];
            }
        }
    }
}

// `rows` rows of `row_bytes` from `src` (pitch `src_pitch`, 4-byte aligned)
// to `dst` (pitch `dst_pitch`, 16-byte aligned) on stream s.
cudaError_t copy_rows_by_sms(const uint8_t* src, size_t src_pitch, uint8_t* dst, size_t dst_pitch,
                             size_t row_bytes, int rows, int sms, cudaStream_t s) {
    const bool v16 = reinterpret_cast<uintptr_t>(src) % 16 == 0 && src_pitch % 16 == 0 && row_bytes % 16 == 0 &&
                     dst_pitch % 16 == 0;
    const size_t elem = v16 ? 16 : 4;
    const size_t row_elems = row_bytes / elem, total = row_elems * (size_t)rows;
    if (total == 0) return cudaSuccess;
    const unsigned grid = (unsigned)(2 * (sms > 0 ? sms : 1));
    if (v16)
        astc_copy_rows<uint4><<<grid, 256, 0, s>>>(src, src_pitch, dst, dst_pitch, row_elems, total);
    else
        astc_copy_rows<uint32_t><<<grid, 256, 0, s>>>(src, src_pitch, dst, dst_pitch, row_elems, total);
    return cudaGetLastError();
}

struct UploadRing {
    bool ready = false;
    int sms = 0;                              // multiprocessors of the ring's device
    cudaStream_t copy = nullptr;
    uint8_t* slot[kRingSlots] = {};
    cudaEvent_t filled[kRingSlots] = {};
    cudaEvent_t drained[kRingSlots] = {};
    int next = 0;
};

// Per-device pool: one stream and grow-only staging buffers for host-memory
// calls.  Calls on one device serialise on its mutex while they use the pool.
struct DevicePool {
    std::mutex mu;
    bool ready = false;
    cudaStream_t stream = nullptr;
    uint8_t* d_in = nullptr;
    size_t in_cap = 0;
    uint8_t* d_out = nullptr;
    size_t out_cap = 0;
    unsigned long long* d_sse = nullptr;
    UploadRing ring;
};

constexpr int kMaxDevices = 64;
DevicePool g_pools[kMaxDevices];

astc_status grow(uint8_t** p, size_t* cap, size_t need) {
    if (*cap >= need) return ASTC_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t want = need < (1u << 20) ? (1u << 20) : need;
    want = (want + 255) & ~(size_t)255;
    const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(ASTC_ERR_OUT_OF_MEMORY,
                         std::string("cudaMalloc of staging buffer failed: ") + cudaGetErrorString(e));
    }
    *cap = want;
    return ASTC_OK;
}

astc_status pool_for_current(DevicePool** out, int* dev_out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return set_error(ASTC_ERR_UNSUPPORTED, "device index out of range");
    DevicePool& p = g_pools[dev];
    *out = &p;
    *dev_out = dev;
    return ASTC_OK;
}

astc_status pool_init_locked(DevicePool& p, int dev) {
    if (p.ready) return ASTC_OK;
    // a blocking stream: calls without a stream of their own are ordered after
    // earlier work on the legacy default stream (where callers usually filled
    // their device buffers)
    cudaError_t e = cudaStreamCreate(&p.stream);
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamCreateWithFlags");
    (void)dev;
    p.ready = true;
    return ASTC_OK;
}

void ring_release(UploadRing& r) {
    if (r.copy) cudaStreamSynchronize(r.copy);
    for (int k = 0; k < kRingSlots; ++k) {
        if (r.slot[k]) cudaFree(r.slot[k]);
        if (r.filled[k]) cudaEventDestroy(r.filled[k]);
        if (r.drained[k]) cudaEventDestroy(r.drained[k]);
        r.slot[k] = nullptr;
        r.filled[k] = r.drained[k] = nullptr;
    }
    if (r.copy) cudaStreamDestroy(r.copy);
    r.copy = nullptr;
    r.next = 0;
    r.ready = false;
}

astc_status ring_init_locked(UploadRing& r) {
    if (r.ready) return ASTC_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r.sms, cudaDevAttrMultiProcessorCount, dev);
    for (int k = 0; k < kRingSlots && e == cudaSuccess; ++k) {
        e = cudaMalloc(reinterpret_cast<void**>(&r.slot[k]), kRingSlotBytes);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r.filled[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r.drained[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(r.drained[k], r.copy);   // every slot starts free
    }
    if (e != cudaSuccess) {
        const astc_status st = cuda_error(e, "upload ring set-up");
        ring_release(r);
        return st;
    }
    r.ready = true;
    return ASTC_OK;
}

// ASTC_GB300_UPLOAD_RING=0 reads large pinned inputs in place instead.
bool upload_ring_enabled() {
    static const bool on = [] {
        const char* v = getenv("ASTC_GB300_UPLOAD_RING");
        return !(v && v[0] == '0');
    }();
    return on;
}

astc_status check_device_pointer(const void* ptr, size_t bytes, const char* what) {
    return check_device_span(ptr, bytes, what, false, nullptr);
}

// Device view of a pinned (page-locked, device-mapped) host buffer, or NULL
// for any other buffer.  Under unified addressing every pinned allocation is
// mapped; ASTC_GB300_ZERO_COPY=0 turns the zero-copy path off.
bool zero_copy_enabled() {
    static const bool on = [] {
        const char* v = getenv("ASTC_GB300_ZERO_COPY");
        return !(v && v[0] == '0');
    }();
    return on;
}

}  // namespace

// cuPointerGetAttributes through the runtime's driver entry point (no link
// against the driver library); NULL where the driver does not provide it.
using PointerAttrsFn = CUresult (*)(unsigned, CUpointer_attribute*, void**, CUdeviceptr);
static PointerAttrsFn pointer_attrs_fn() {
    static const PointerAttrsFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttributes", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<PointerAttrsFn>(f);
    }();
    return fn;
}

astc_status check_device_span(const void* p, size_t bytes, const char* what, bool allow_host_view,
                              SpanCache* seen) {
    const uintptr_t lo = reinterpret_cast<uintptr_t>(p), hi = lo + bytes;
    if (hi < lo) return set_error(ASTC_ERR_INVALID_ARG, std::string(what) + ": extent overflows");
    if (seen && seen->n) {
        if (lo >= seen->r[seen->last].lo && hi <= seen->r[seen->last].hi) return ASTC_OK;
        for (int i = 0; i < seen->n; ++i)
            if (lo >= seen->r[i].lo && hi <= seen->r[i].hi) {
                seen->last = i;
                return ASTC_OK;
            }
    }
    cudaPointerAttributes a;
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(ASTC_ERR_INVALID_ARG, std::string(what) + " is not a CUDA pointer");
    }
    // pageable host memory that the device reads through the host's page
    // tables: accessed in place like pinned memory (it has no allocation
    // range to check the extent against)
    if (allow_host_view && a.type == cudaMemoryTypeUnregistered && pageable_in_place_available()) return ASTC_OK;
    const bool host_view = allow_host_view && a.type == cudaMemoryTypeHost && a.devicePointer == p;
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged && !host_view)
        return set_error(ASTC_ERR_INVALID_ARG,
                         std::string(what) + (allow_host_view ? " is not device-accessible memory"
                                                              : " is not device memory (memory = ASTC_MEMORY_DEVICE)"));
    if (a.type == cudaMemoryTypeDevice) {
        int cur = 0;
        if (cudaGetDevice(&cur) == cudaSuccess && a.device != cur)
            return set_error(ASTC_ERR_INVALID_ARG, std::string(what) + " is memory of device " +
                                                       std::to_string(a.device) + ", not of the current device " +
                                                       std::to_string(cur));
    }
    // the allocation that holds p: the whole extent must lie inside it
    if (PointerAttrsFn fn = pointer_attrs_fn()) {
        CUpointer_attribute attrs[2] = {CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, CU_POINTER_ATTRIBUTE_RANGE_SIZE};
        CUdeviceptr start = 0;
        size_t size = 0;
        void* data[2] = {&start, &size};
        if (fn(2, attrs, data, (CUdeviceptr)lo) == CUDA_SUCCESS && size > 0) {
            if (hi > (uintptr_t)start + size)
                return set_error(ASTC_ERR_INVALID_ARG, std::string(what) + ": " + std::to_string(bytes) +
                                                           " bytes from the pointer run past the end of its allocation");
            if (seen && seen->n < (int)(sizeof(seen->r) / sizeof(seen->r[0]))) {
                seen->last = seen->n;
                seen->r[seen->n++] = {(uintptr_t)start, (uintptr_t)start + size};
            }
        }
    }
    return ASTC_OK;
}

// ASTC_GB300_PAGEABLE_IN_PLACE=0 stages pageable host buffers even where the
// device could access them in place.
bool pageable_in_place_enabled() {
    static const bool on = [] {
        const char* v = getenv("ASTC_GB300_PAGEABLE_IN_PLACE");
        return !(v && v[0] == '0');
    }();
    return on;
}

// Whether the current device reads and writes pageable host memory through
// the host's page tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables:
// address translation over NVLink-C2C on Grace systems), cached per device.
bool pageable_host_access() {
    static std::atomic<int> cache[kMaxDevices] = {};   // 0 unknown, 1 no, 2 yes
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return false;
    }
    int c = cache[dev].load(std::memory_order_relaxed);
    if (!c) {
        int a = 0, b = 0;
        const bool ok = cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
                        cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
                            cudaSuccess;
        if (!ok) cudaGetLastError();
        c = ok && a && b ? 2 : 1;
        cache[dev].store(c, std::memory_order_relaxed);
    }
    return c == 2;
}

bool pageable_in_place_available() { return pageable_in_place_enabled() && pageable_host_access(); }

HostView host_device_view(const void* host) {
    HostView v;
    if (!host) return v;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return v;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer && zero_copy_enabled()) {
        v.ptr = a.devicePointer;
        v.pinned = true;
    } else if (a.type == cudaMemoryTypeUnregistered && pageable_in_place_available()) {
        v.ptr = host;                                  // the same virtual address on the device
    }
    return v;
}


namespace {

astc_status validate_opts(const astc_opts* o, int w, int h) {
    if (!o) return set_error(ASTC_ERR_INVALID_ARG, "opts is NULL");
    if (o->block_dim != 4 && o->block_dim != 6)
        return set_error(ASTC_ERR_INVALID_ARG, "block_dim must be 4 or 6");
    if (o->border != ASTC_BORDER_ZERO && o->border != ASTC_BORDER_CLAMP)
        return set_error(ASTC_ERR_INVALID_ARG, "border must be ASTC_BORDER_ZERO or ASTC_BORDER_CLAMP");
    if (o->precision != ASTC_PRECISION_FP32 && o->precision != ASTC_PRECISION_HALF2)
        return set_error(ASTC_ERR_INVALID_ARG, "precision must be FP32 or HALF2");
    if (o->memory != ASTC_MEMORY_HOST && o->memory != ASTC_MEMORY_DEVICE)
        return set_error(ASTC_ERR_INVALID_ARG, "memory must be ASTC_MEMORY_HOST or ASTC_MEMORY_DEVICE");
    if (o->axis != ASTC_AXIS_PCA && o->axis != ASTC_AXIS_MAX_ACCUMULATION && o->axis != ASTC_AXIS_BEST)
        return set_error(ASTC_ERR_INVALID_ARG, "axis must be ASTC_AXIS_PCA, _MAX_ACCUMULATION or _BEST");
    if (o->quality < ASTC_QUALITY_FAST || o->quality > ASTC_QUALITY_THREE_PARTITIONS)
        return set_error(ASTC_ERR_INVALID_ARG,
                         "quality must be ASTC_QUALITY_FAST, _SEARCH, _THOROUGH, _PARTITIONS or _THREE_PARTITIONS");
    if (o->precision == ASTC_PRECISION_HALF2 && (o->axis != ASTC_AXIS_PCA || o->quality != ASTC_QUALITY_FAST))
        return set_error(ASTC_ERR_UNSUPPORTED, "the other axes and the quality modes are FP32 only");
    if (w <= 0 || h <= 0) return set_error(ASTC_ERR_INVALID_ARG, "width and height must be positive");
    if (w > 0xFFFFFF || h > 0xFFFFFF)
        return set_error(ASTC_ERR_INVALID_ARG, "width and height must fit the 24-bit .astc size fields");
    const long long nb = (long long)blocks_x(w, o->block_dim) * blocks_y(h, o->block_dim);
    if (nb > (1LL << 31)) return set_error(ASTC_ERR_INVALID_ARG, "image has more than 2^31 blocks");
    return ASTC_OK;
}

}  // namespace

astc_status set_error(astc_status st, const std::string& msg) {
    t_last_error = msg;
    return st;
}

astc_status cuda_error(cudaError_t e, const char* what) {
    const std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? ASTC_ERR_OUT_OF_MEMORY : ASTC_ERR_CUDA, msg);
}

void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace astc

using namespace astc;

namespace {

// Shared body of the SSE reductions: stages host images through the pool,
// zeroes the 32-byte accumulator, runs `launch(a, b, accumulator, stream)` and
// reads the accumulator back into `result` (`result_bytes` of it).
template <class Launch>
astc_status sse_common(const uint8_t* a, const uint8_t* b, size_t texels, int memory, void* stream,
                       void* result, size_t result_bytes, Launch launch) {
    try {
        if (!a || !b || !result) return set_error(ASTC_ERR_INVALID_ARG, "NULL pointer");
        if (memory != ASTC_MEMORY_HOST && memory != ASTC_MEMORY_DEVICE)
            return set_error(ASTC_ERR_INVALID_ARG, "bad memory kind");
        if (texels > SIZE_MAX / 4) return set_error(ASTC_ERR_INVALID_ARG, "texel count overflows the byte size");
        DevicePool* pool = nullptr;
        int dev = 0;
        astc_status st;
        if ((st = pool_for_current(&pool, &dev)) != ASTC_OK) return st;
        std::lock_guard<std::mutex> lk(pool->mu);
        if ((st = pool_init_locked(*pool, dev)) != ASTC_OK) return st;
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : pool->stream;
        if (!pool->d_sse) {
            cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&pool->d_sse), 4 * sizeof(unsigned long long));
            if (e != cudaSuccess) return cuda_error(e, "cudaMalloc of the SSE accumulator");
        }
        const uint8_t* da = a;
        const uint8_t* db = b;
        if (memory == ASTC_MEMORY_HOST) {
            const size_t bytes = texels * 4;
            if ((st = grow(&pool->d_in, &pool->in_cap, bytes)) != ASTC_OK) return st;
            if ((st = grow(&pool->d_out, &pool->out_cap, bytes)) != ASTC_OK) return st;
            cudaError_t e = cudaMemcpyAsync(pool->d_in, a, bytes, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(pool->d_out, b, bytes, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return cuda_error(e, "host-to-device copy");
            da = pool->d_in;
            db = pool->d_out;
        } else {
            if ((st = check_device_pointer(a, texels * 4, "a")) != ASTC_OK) return st;
            if ((st = check_device_pointer(b, texels * 4, "b")) != ASTC_OK) return st;
            if (reinterpret_cast<uintptr_t>(a) % 4 != 0 || reinterpret_cast<uintptr_t>(b) % 4 != 0)
                return set_error(ASTC_ERR_INVALID_ARG, "images must be 4-byte aligned");
        }
        cudaError_t e = cudaMemsetAsync(pool->d_sse, 0, 4 * sizeof(unsigned long long), s);
        if (e != cudaSuccess) return cuda_error(e, "cudaMemsetAsync");
        e = launch(da, db, pool->d_sse, s);
        if (e != cudaSuccess) return cuda_error(e, "sse kernel launch");
        unsigned long long h[4];
        e = cudaMemcpyAsync(h, pool->d_sse, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_error(e, "sse");
        memcpy(result, h, result_bytes);
        return ASTC_OK;
    } catch (...) {
        return set_error(ASTC_ERR_CUDA, "unexpected exception");
    }
}

}  // namespace

extern "C" {

void astc_opts_init(astc_opts* o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->block_dim = 4;                 // encode_option(): is4x4 = true
    o->border = ASTC_BORDER_ZERO;
    o->precision = ASTC_PRECISION_FP32;
    o->memory = ASTC_MEMORY_HOST;
}

size_t astc_encoded_size(int width, int height, int block_dim) {
    if (width <= 0 || height <= 0 || (block_dim != 4 && block_dim != 6)) return 0;
    return (size_t)16 * blocks_x(width, block_dim) * blocks_y(height, block_dim);
}

astc_status astc_encode_gpu_pitched(const uint8_t* rgba8, int width, int height, size_t row_pitch,
                                    const astc_opts* opts, uint8_t* out) {
    try {
        astc_status st = validate_opts(opts, width, height);
        if (st != ASTC_OK) return st;
        if (!rgba8 || !out) return set_error(ASTC_ERR_INVALID_ARG, "rgba8 and out must be non-NULL");
        if (row_pitch < (size_t)width * 4 || row_pitch % 4 != 0)
            return set_error(ASTC_ERR_INVALID_ARG, "row_pitch must be >= 4*width and a multiple of 4");
        auto launch = [&](const EncodeJob& j, cudaStream_t st_) {
            if (opts->precision == ASTC_PRECISION_HALF2) return launch_encode_h2(j, st_);
            if (j.axis != ASTC_AXIS_PCA || j.quality != ASTC_QUALITY_FAST) return launch_encode_search(j, st_);
            return launch_encode(j, st_);
        };
        DevicePool* pool = nullptr;
        int dev = 0;
        if ((st = pool_for_current(&pool, &dev)) != ASTC_OK) return st;
        std::lock_guard<std::mutex> lk(pool->mu);
        if ((st = pool_init_locked(*pool, dev)) != ASTC_OK) return st;

        const size_t out_bytes = astc_encoded_size(width, height, opts->block_dim);
        const size_t in_bytes = row_pitch * (size_t)(height - 1) + (size_t)width * 4;
        cudaStream_t s = opts->stream ? static_cast<cudaStream_t>(opts->stream) : pool->stream;

        EncodeJob job;
        job.width = width;
        job.height = height;
        job.block_dim = opts->block_dim;
        job.has_alpha = opts->has_alpha;
        job.is_normal = opts->is_normal;
        job.srgb = opts->srgb;
        job.border = opts->border;
        job.precision = opts->precision;
        job.axis = opts->axis;
        job.quality = opts->quality;

        if (opts->memory == ASTC_MEMORY_DEVICE) {
            if ((st = check_device_pointer(rgba8, in_bytes, "rgba8")) != ASTC_OK) return st;
            if ((st = check_device_pointer(out, out_bytes, "out")) != ASTC_OK) return st;
            if (reinterpret_cast<uintptr_t>(rgba8) % 4 != 0)
                return set_error(ASTC_ERR_INVALID_ARG, "device rgba8 must be 4-byte aligned");
            if (reinterpret_cast<uintptr_t>(out) % 16 != 0)
                return set_error(ASTC_ERR_INVALID_ARG, "device out must be 16-byte aligned");
            job.in = rgba8;
            job.pitch = row_pitch;
            job.out = out;
            cudaError_t e = launch(job, s);
            if (e != cudaSuccess) return cuda_error(e, "encode kernel launch");
            if (!opts->stream) {
                e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) return cuda_error(e, "encode");
            }
            return ASTC_OK;
        }

        // host memory the device can address -- pinned buffers through their
        // device view, and pageable buffers on a device that reads the host's
        // page tables -- is accessed over the host link: an input of
        // kRingMinBytes or more streams through the upload ring, a smaller one
        // is read in place (zero-copy); the output is written in place.  Other
        // buffers are staged through the pool (tight rows on the device).
        (void)in_bytes;
        const size_t tight = (size_t)width * 4;
        const HostView in_hv = host_device_view(rgba8), out_hv = host_device_view(out);
        const void* in_view = in_hv.ptr;
        void* out_view = const_cast<void*>(out_hv.ptr);
        if (out_view && reinterpret_cast<uintptr_t>(out_view) % 16 != 0) out_view = nullptr;
        // only a call whose buffers are both pinned may return before the
        // blocks are in `out` (pinned memory is the caller's to keep alive;
        // pageable buffers keep the synchronous contract of other host memory)
        const bool may_return_early = opts->stream && in_hv.pinned && out_hv.pinned;
        cudaError_t e = cudaSuccess;
        const int dim = opts->block_dim;
        const bool use_ring = in_view && upload_ring_enabled() && tight * (size_t)height >= kRingMinBytes &&
                              tight * (size_t)dim <= kRingSlotBytes;
        if (use_ring) {
            // banded upload through the ring; the bands' kernels write `out`
            if ((st = ring_init_locked(pool->ring)) != ASTC_OK) return st;
            if (out_view) {
                job.out = static_cast<uint8_t*>(out_view);
            } else {
                if ((st = grow(&pool->d_out, &pool->out_cap, out_bytes)) != ASTC_OK) return st;
                job.out = pool->d_out;
            }
            UploadRing& r = pool->ring;
            // equal bands of whole block rows, each at most one slot
            const int block_rows = blocks_y(height, dim);
            const int max_band = (int)(kRingSlotBytes / (tight * (size_t)dim));
            // a pageable input is copied into the slots by the SMs, which read it
            // through the host page tables at the link's rate (the copy engine
            // takes pageable sources more slowly: 2048x2048 6x6 RGBA, 16
            // synchronous calls, 35.5 against 32.6 Gtexel/s end to end)
            const bool sm_copy = !in_hv.pinned && reinterpret_cast<uintptr_t>(rgba8) % 4 == 0;
            const int nbands = (block_rows + max_band - 1) / max_band;
            const int band_rows = ((block_rows + nbands - 1) / nbands) * dim;          // texel rows
            const size_t band_row_bytes = (size_t)blocks_x(width, dim) * 16;
            for (int y0 = 0; y0 < height; y0 += band_rows) {
                const int rows = height - y0 < band_rows ? height - y0 : band_rows;
                const int k = r.next;
                r.next = (r.next + 1) % kRingSlots;
                if ((e = cudaStreamWaitEvent(r.copy, r.drained[k], 0)) != cudaSuccess)
                    return cuda_error(e, "upload ring wait");
                const uint8_t* src = rgba8 + (size_t)y0 * row_pitch;
                if (sm_copy) {
                    // pageable source: the SMs read it through the host page tables
                    e = copy_rows_by_sms(src, row_pitch, r.slot[k], tight, tight, rows, r.sms, r.copy);
                    if (e == cudaSuccess) count_launches(1);
                } else {
                    e = row_pitch == tight
                            ? cudaMemcpyAsync(r.slot[k], src, tight * (size_t)rows, cudaMemcpyHostToDevice, r.copy)
                            : cudaMemcpy2DAsync(r.slot[k], tight, src, row_pitch, tight, rows,
                                                cudaMemcpyHostToDevice, r.copy);
                }
                if (e != cudaSuccess) return cuda_error(e, "host-to-device band copy");
                if ((e = cudaEventRecord(r.filled[k], r.copy)) != cudaSuccess) return cuda_error(e, "event record");
                if ((e = cudaStreamWaitEvent(s, r.filled[k], 0)) != cudaSuccess)
                    return cuda_error(e, "upload ring wait");
                EncodeJob band = job;
                band.in = r.slot[k];
                band.pitch = tight;
                band.height = rows;
                band.out = job.out + (size_t)(y0 / dim) * band_row_bytes;
                if ((e = launch(band, s)) != cudaSuccess) return cuda_error(e, "encode kernel launch");
                if ((e = cudaEventRecord(r.drained[k], s)) != cudaSuccess) return cuda_error(e, "event record");
            }
            if (!out_view) {
                e = cudaMemcpyAsync(out, pool->d_out, out_bytes, cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) return cuda_error(e, "device-to-host copy");
            }
            // the ring's slots are ordered by events, so with a caller's stream and
            // pinned buffers the call stays asynchronous
            if (out_view && may_return_early) return ASTC_OK;
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return cuda_error(e, "encode");
            return ASTC_OK;
        }
        if (in_view && reinterpret_cast<uintptr_t>(in_view) % 4 == 0) {
            job.in = static_cast<const uint8_t*>(in_view);
            job.pitch = row_pitch;
        } else {
            if ((st = grow(&pool->d_in, &pool->in_cap, tight * height)) != ASTC_OK) return st;
            e = cudaMemcpy2DAsync(pool->d_in, tight, rgba8, row_pitch, tight, height, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return cuda_error(e, "host-to-device copy");
            job.in = pool->d_in;
            job.pitch = tight;
        }
        if (out_view) {
            job.out = static_cast<uint8_t*>(out_view);
        } else {
            if ((st = grow(&pool->d_out, &pool->out_cap, out_bytes)) != ASTC_OK) return st;
            job.out = pool->d_out;
        }
        e = launch(job, s);
        if (e != cudaSuccess) return cuda_error(e, "encode kernel launch");
        if (!out_view) {
            e = cudaMemcpyAsync(out, pool->d_out, out_bytes, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) return cuda_error(e, "device-to-host copy");
        }
        // Fully zero-copy calls on pinned buffers touch no pooled buffer, so with
        // a caller's stream they stay asynchronous; otherwise the pool is reused
        // by the next call, or the buffers are pageable, and the call finishes
        // before returning.
        if (job.in != pool->d_in && out_view && may_return_early) return ASTC_OK;
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_error(e, "encode");
        return ASTC_OK;
    } catch (const std::bad_alloc&) {
        return set_error(ASTC_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (...) {
        return set_error(ASTC_ERR_CUDA, "unexpected exception");
    }
}

astc_status astc_encode_gpu(const uint8_t* rgba8, int width, int height, const astc_opts* opts,
                            uint8_t* out) {
    if (width <= 0) return astc_encode_gpu_pitched(rgba8, width, height, 4, opts, out);
    return astc_encode_gpu_pitched(rgba8, width, height, (size_t)width * 4, opts, out);
}

astc_status astc_save_file(const char* path, int bdx, int bdy, int width, int height,
                           const uint8_t* blocks, size_t blocks_size) {
    if (!path || !blocks) return set_error(ASTC_ERR_INVALID_ARG, "path and blocks must be non-NULL");
    if (bdx < 2 || bdx > 12 || bdy < 2 || bdy > 12)
        return set_error(ASTC_ERR_INVALID_ARG, "block dimensions must be 2..12");
    if (width <= 0 || height <= 0 || width > 0xFFFFFF || height > 0xFFFFFF)
        return set_error(ASTC_ERR_INVALID_ARG, "image size must be 1..2^24-1");
    const size_t need = (size_t)16 * ((width + bdx - 1) / bdx) * ((height + bdy - 1) / bdy);
    if (blocks_size != need)
        return set_error(ASTC_ERR_INVALID_ARG, "blocks_size does not match the image and block size");
    // astc_header (astc_save.h:5-14): magic 0x5CA1AB13 little-endian, block
    // dims, 24-bit little-endian x/y/z sizes in texels, z = 1.
    uint8_t hdr[16];
    const uint32_t magic = 0x5CA1AB13u;
    for (int i = 0; i < 4; ++i) hdr[i] = (uint8_t)(magic >> (8 * i));
    hdr[4] = (uint8_t)bdx;
    hdr[5] = (uint8_t)bdy;
    hdr[6] = 1;
    for (int i = 0; i < 3; ++i) {
        hdr[7 + i] = (uint8_t)(width >> (8 * i));
        hdr[10 + i] = (uint8_t)(height >> (8 * i));
    }
    hdr[13] = 1; hdr[14] = 0; hdr[15] = 0;
    FILE* f = fopen(path, "wb");
    if (!f) return set_error(ASTC_ERR_IO, std::string("cannot open for writing: ") + path);
    const bool ok = fwrite(hdr, 1, 16, f) == 16 && fwrite(blocks, 1, blocks_size, f) == blocks_size;
    const bool closed = fclose(f) == 0;
    if (!ok || !closed) return set_error(ASTC_ERR_IO, std::string("write failed: ") + path);
    return ASTC_OK;
}

astc_status astc_load_file(const char* path, int* bdx, int* bdy, int* width, int* height,
                           uint8_t* blocks, size_t capacity, size_t* blocks_size) {
    if (!path || !bdx || !bdy || !width || !height || !blocks_size)
        return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    FILE* f = fopen(path, "rb");
    if (!f) return set_error(ASTC_ERR_IO, std::string("cannot open: ") + path);
    uint8_t hdr[16];
    if (fread(hdr, 1, 16, f) != 16) {
        fclose(f);
        return set_error(ASTC_ERR_FORMAT, "file shorter than the 16-byte header");
    }
    const uint32_t magic = hdr[0] | (hdr[1] << 8) | (hdr[2] << 16) | ((uint32_t)hdr[3] << 24);
    if (magic != 0x5CA1AB13u) {
        fclose(f);
        return set_error(ASTC_ERR_FORMAT, "bad magic (expected 0x5CA1AB13)");
    }
    const int x = hdr[7] | (hdr[8] << 8) | (hdr[9] << 16);
    const int y = hdr[10] | (hdr[11] << 8) | (hdr[12] << 16);
    const int z = hdr[13] | (hdr[14] << 8) | (hdr[15] << 16);
    if (hdr[4] < 2 || hdr[5] < 2 || hdr[6] != 1 || x <= 0 || y <= 0 || z != 1) {
        fclose(f);
        return set_error(ASTC_ERR_FORMAT, "unsupported header (only 2-D, z = 1)");
    }
    const size_t need = (size_t)16 * ((x + hdr[4] - 1) / hdr[4]) * ((y + hdr[5] - 1) / hdr[5]);
    *bdx = hdr[4];
    *bdy = hdr[5];
    *width = x;
    *height = y;
    *blocks_size = need;
    astc_status st = ASTC_OK;
    if (blocks) {
        if (capacity < need) {
            st = set_error(ASTC_ERR_INVALID_ARG, "capacity smaller than the block data");
        } else if (fread(blocks, 1, need, f) != need) {
            st = set_error(ASTC_ERR_FORMAT, "file truncated");
        }
    }
    fclose(f);
    return st;
}

astc_status astc_decode_gpu(const uint8_t* blocks, int width, int height, int block_w, int block_h,
                            int srgb, int memory, void* stream, uint8_t* out_rgba8) {
    try {
        if (!blocks || !out_rgba8) return set_error(ASTC_ERR_INVALID_ARG, "NULL pointer");
        if (width <= 0 || height <= 0 || width > 0xFFFFFF || height > 0xFFFFFF)
            return set_error(ASTC_ERR_INVALID_ARG, "bad image size");
        if (block_w < 4 || block_w > 12 || block_h < 4 || block_h > 12)
            return set_error(ASTC_ERR_INVALID_ARG, "block footprint must be 4..12 per axis");
        if (memory != ASTC_MEMORY_HOST && memory != ASTC_MEMORY_DEVICE)
            return set_error(ASTC_ERR_INVALID_ARG, "bad memory kind");
        DevicePool* pool = nullptr;
        int dev = 0;
        astc_status st;
        if ((st = pool_for_current(&pool, &dev)) != ASTC_OK) return st;
        std::lock_guard<std::mutex> lk(pool->mu);
        if ((st = pool_init_locked(*pool, dev)) != ASTC_OK) return st;
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : pool->stream;
        const size_t nblk = (size_t)((width + block_w - 1) / block_w) * ((height + block_h - 1) / block_h);
        const size_t in_bytes = 16 * nblk, out_bytes = (size_t)width * height * 4;
        if (memory == ASTC_MEMORY_DEVICE) {
            if ((st = check_device_pointer(blocks, in_bytes, "blocks")) != ASTC_OK) return st;
            if ((st = check_device_pointer(out_rgba8, out_bytes, "out_rgba8")) != ASTC_OK) return st;
            if (reinterpret_cast<uintptr_t>(blocks) % 16 != 0 || reinterpret_cast<uintptr_t>(out_rgba8) % 4 != 0)
                return set_error(ASTC_ERR_INVALID_ARG, "blocks must be 16-byte and out 4-byte aligned");
            cudaError_t e = launch_decode(blocks, width, height, block_w, block_h, srgb, out_rgba8, s);
            if (e != cudaSuccess) return cuda_error(e, "decode kernel launch");
            if (!stream && (e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_error(e, "decode");
            return ASTC_OK;
        }
        if ((st = grow(&pool->d_in, &pool->in_cap, in_bytes)) != ASTC_OK) return st;
        if ((st = grow(&pool->d_out, &pool->out_cap, out_bytes)) != ASTC_OK) return st;
        cudaError_t e = cudaMemcpyAsync(pool->d_in, blocks, in_bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_error(e, "host-to-device copy");
        e = launch_decode(pool->d_in, width, height, block_w, block_h, srgb, pool->d_out, s);
        if (e != cudaSuccess) return cuda_error(e, "decode kernel launch");
        e = cudaMemcpyAsync(out_rgba8, pool->d_out, out_bytes, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_error(e, "device-to-host copy");
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_error(e, "decode");
        return ASTC_OK;
    } catch (...) {
        return set_error(ASTC_ERR_CUDA, "unexpected exception");
    }
}

astc_status astc_sse_gpu(const uint8_t* a, const uint8_t* b, size_t texels, int memory, void* stream,
                         uint64_t sse_rgba[4]) {
    return sse_common(a, b, texels, memory, stream, sse_rgba, 4 * sizeof(uint64_t),
                      [texels](const uint8_t* da, const uint8_t* db, unsigned long long* acc, cudaStream_t s) {
                          return launch_sse(da, db, texels, acc, s);
                      });
}

astc_status astc_normal_sse_gpu(const uint8_t* a, const uint8_t* b, size_t texels, int memory, void* stream,
                                double* sse) {
    static_assert(sizeof(double) <= 4 * sizeof(unsigned long long), "accumulator size");
    return sse_common(a, b, texels, memory, stream, sse, sizeof(double),
                      [texels](const uint8_t* da, const uint8_t* db, unsigned long long* acc, cudaStream_t s) {
                          return launch_normal_sse(da, db, texels, reinterpret_cast<double*>(acc), s);
                      });
}

astc_status astc_get_device_caps(astc_device_caps* caps) {
    if (!caps) return set_error(ASTC_ERR_INVALID_ARG, "NULL caps");
    memset(caps, 0, sizeof(*caps));
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    struct Q { cudaDeviceAttr a; int* v; } qs[] = {
        {cudaDevAttrMultiProcessorCount, &caps->sm_count},
        {cudaDevAttrL2CacheSize, &caps->l2_bytes},
        {cudaDevAttrUnifiedAddressing, &caps->unified_addressing},
        {cudaDevAttrCanMapHostMemory, &caps->can_map_host_memory},
        {cudaDevAttrPageableMemoryAccess, &caps->pageable_memory_access},
        {cudaDevAttrPageableMemoryAccessUsesHostPageTables, &caps->pageable_uses_host_page_tables},
    };
    for (const Q& q : qs)
        if ((e = cudaDeviceGetAttribute(q.v, q.a, dev)) != cudaSuccess) return cuda_error(e, "cudaDeviceGetAttribute");
    caps->zero_copy = zero_copy_enabled() && caps->unified_addressing && caps->can_map_host_memory;
    caps->pageable_in_place = pageable_in_place_enabled() && caps->pageable_memory_access &&
                              caps->pageable_uses_host_page_tables;
    return ASTC_OK;
}

const char* astc_last_error(void) { return t_last_error.c_str(); }

const char* astc_status_string(astc_status s) {
    switch (s) {
    case ASTC_OK: return "ok";
    case ASTC_ERR_INVALID_ARG: return "invalid argument";
    case ASTC_ERR_UNSUPPORTED: return "unsupported";
    case ASTC_ERR_CUDA: return "CUDA error";
    case ASTC_ERR_OUT_OF_MEMORY: return "out of memory";
    case ASTC_ERR_IO: return "I/O error";
    case ASTC_ERR_TIMEOUT: return "timeout";
    case ASTC_ERR_BUSY: return "busy";
    case ASTC_ERR_CANCELLED: return "cancelled";
    case ASTC_ERR_FORMAT: return "bad .astc format";
    }
    return "unknown status";
}

uint64_t astc_kernel_launch_count(void) { return g_launches.load(); }

void astc_shutdown(void) {
    int cur = 0;
    const bool have = cudaGetDevice(&cur) == cudaSuccess;
    for (int d = 0; d < kMaxDevices; ++d) {
        DevicePool& p = g_pools[d];
        std::lock_guard<std::mutex> lk(p.mu);
        if (!p.ready && !p.d_in && !p.d_out && !p.d_sse && !p.ring.ready) continue;
        if (cudaSetDevice(d) != cudaSuccess) { cudaGetLastError(); continue; }
        if (p.stream) cudaStreamSynchronize(p.stream);
        ring_release(p.ring);
        if (p.d_in) cudaFree(p.d_in);
        if (p.d_out) cudaFree(p.d_out);
        if (p.d_sse) cudaFree(p.d_sse);
        if (p.stream) cudaStreamDestroy(p.stream);
        p.d_in = p.d_out = nullptr;
        p.d_sse = nullptr;
        p.in_cap = p.out_cap = 0;
        p.stream = nullptr;
        p.ready = false;
    }
    if (have) cudaSetDevice(cur);
    cudaGetLastError();
}

}  // extern "C"
