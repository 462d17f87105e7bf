// astc_batch.cu -- batched encode: one CUDA-graph launch encodes a whole
// list of textures (different sizes, mip levels and formats).
//
// The reference dispatches one texture per call (astc_encode.h:87-194,
// Dispatch at 190); small textures and mip levels then cost a launch each and
// leave most of the GPU idle.  Here the host splits every texture into work
// items of up to 128 blocks, groups the items by format, and uploads the
// texture descriptors and items in one copy; one persistent kernel per format
// present (16 formats: 4x4/6x6 x alpha x normal x sRGB, per precision) drains
// its format's queue: a CTA takes the next item with one atomicAdd on a
// device counter and encodes its blocks, one thread per block, exactly as the
// plain kernels do (so a texture's blocks are the same whether it is encoded
// alone or in a batch).  The kernels are captured once per (precision, set
// of formats) into a CUDA graph and replayed; each call uploads exactly its
// queue header, descriptors and items (two copies) and launches the graph.
// Batch sizes and contents are read from device memory at run time, so one
// graph serves every batch that fits the handle.
//
// No kernel here waits on another CTA or kernel: the only synchronisation is
// the atomicAdd that hands out items.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "astc_internal.h"
#include "astc_pipeline_fp32.cuh"
#include "astc_pipeline_h2.cuh"

namespace astc {
namespace {

constexpr int kBatchThreads = 128;      // blocks per work item = threads per CTA
constexpr int kFormats = 16;

__constant__ TritPack c_trit_pack_b = make_trit_pack();
__constant__ SrgbBits c_srgb_bits_b = make_srgb_bits();

struct BatchJob {
    TextureView tex;
    uint4* out;
    int item_start;     // index of the job's first work item (items grouped by format)
    int nblocks;
};

struct WorkItem {
    int job;
    int first;
    int count;
    int pad;
};

struct QueueState {
    int counter[kFormats];
    int begin[kFormats];
    int end[kFormats];
    int njobs;
    int pad[kFormats - 1];
};

// Expands the jobs into their work items of <= 128 blocks on the device (the
// host uploads only the per-texture descriptors, O(textures) per call).
__global__ void __launch_bounds__(kBatchThreads)
astc_batch_expand(const BatchJob* __restrict__ jobs, WorkItem* __restrict__ items, const QueueState* __restrict__ q) {
    const int njobs = q->njobs;
    for (int j = blockIdx.x; j < njobs; j += gridDim.x) {
        const int start = jobs[j].item_start, nb = jobs[j].nblocks;
        const int n = (nb + kBatchThreads - 1) / kBatchThreads;
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            WorkItem w;
            w.job = j;
            w.first = t * kBatchThreads;
            w.count = nb - w.first < kBatchThreads ? nb - w.first : kBatchThreads;
            w.pad = 0;
            items[start + t] = w;
        }
    }
}

inline int format_index(int dim, bool alpha, bool normal, bool srgb) {
    return (dim == 6 ? 8 : 0) | (alpha ? 4 : 0) | (normal ? 2 : 0) | (srgb ? 1 : 0);
}

// Register caps: <= 128 registers (4 CTAs of 128 per SM) for everything but
// the FP32 6x6 pipeline, whose 36 FP32 texels spill heavily at 128; it takes
// 3 CTAs per SM (<= 168 registers; the queue loop leaves 80-250 bytes of
// L1-resident spill in the colour formats), which on GB300 ran the mixed
// 256-texture batch at 211 Gtexel/s against 206 with one CTA per SM.
template <int DIM, bool ALPHA, bool NORMAL, bool SRGB, int PREC>
__global__ void __launch_bounds__(kBatchThreads, (PREC == ASTC_PRECISION_FP32 && DIM == 6) ? 3 : 4)
astc_encode_persistent(const BatchJob* __restrict__ jobs, const WorkItem* __restrict__ items,
                       QueueState* __restrict__ q, int fmt) {
    constexpr int N = DIM * DIM;
    extern __shared__ float4 s_texels[];            // FP32 4x4 keeps texels in shared memory
    __shared__ uint8_t s_trits[256];
    __shared__ float s_lut[(SRGB && PREC == ASTC_PRECISION_FP32) ? 256 : 1];
    __shared__ uint8_t s_lin8[(SRGB && PREC == ASTC_PRECISION_HALF2) ? 256 : 1];
    __shared__ int s_item;
    load_cta_tables<SRGB && PREC == ASTC_PRECISION_FP32>(c_trit_pack_b, c_srgb_bits_b, s_trits, s_lut);
    if (SRGB && PREC == ASTC_PRECISION_HALF2) load_lin8_table(c_srgb_bits_b, s_lin8);
    const int end = q->end[fmt];
    const int begin = q->begin[fmt];
    for (;;) {
        if (threadIdx.x == 0) s_item = begin + atomicAdd(&q->counter[fmt], 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= end) break;
        const WorkItem w = items[it];
        if ((int)threadIdx.x < w.count) {
            const BatchJob j = jobs[w.job];
            const int b = w.first + threadIdx.x;
            int bx, by;
            block_coords(j.tex, b, bx, by);
            uint32_t px[N];
            load_block_packed<DIM>(j.tex, bx, by, px);
            uint4 r;
            if constexpr (PREC == ASTC_PRECISION_HALF2) {
                r = encode_block_h2<DIM, ALPHA, NORMAL, SRGB>(px, s_lin8, s_trits);
            } else if constexpr (DIM == 4) {
                SharedTexels<N> st{s_texels + threadIdx.x, kBatchThreads};
#pragma unroll
                for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
                r = encode_block_fp32<DIM, ALPHA, NORMAL>(st, s_trits);
            } else {
                RegTexels<N> st;
#pragma unroll
                for (int k = 0; k < N; ++k) st.put(k, decode_texel<SRGB, NORMAL>(px[k], s_lut));
                r = encode_block_fp32<DIM, ALPHA, NORMAL>(st, s_trits);
            }
            j.out[b] = r;
        }
    }
}

using KernelFn = void (*)(const BatchJob*, const WorkItem*, QueueState*, int);

template <int PREC>
KernelFn kernel_for(int f) {
    switch (f) {
#define ASTC_K(F, D, A, NM, S) case F: return astc_encode_persistent<D, A, NM, S, PREC>;
        ASTC_K(0, 4, false, false, false) ASTC_K(1, 4, false, false, true)
        ASTC_K(2, 4, false, true, false)  ASTC_K(3, 4, false, true, true)
        ASTC_K(4, 4, true, false, false)  ASTC_K(5, 4, true, false, true)
        ASTC_K(6, 4, true, true, false)   ASTC_K(7, 4, true, true, true)
        ASTC_K(8, 6, false, false, false) ASTC_K(9, 6, false, false, true)
        ASTC_K(10, 6, false, true, false) ASTC_K(11, 6, false, true, true)
        ASTC_K(12, 6, true, false, false) ASTC_K(13, 6, true, false, true)
        ASTC_K(14, 6, true, true, false)  ASTC_K(15, 6, true, true, true)
#undef ASTC_K
    }
    return nullptr;
}

size_t dyn_smem(int f, int prec) {
    return (prec == ASTC_PRECISION_FP32 && f < 8) ? (size_t)16 * kBatchThreads * sizeof(float4) : 0;
}

}  // namespace
}  // namespace astc

using namespace astc;

struct astc_batch {
    std::mutex mu;
    int device = 0;
    int max_items = 0;
    long long max_blocks = 0;
    int max_work = 0;
    int sms = 0;
    // device: [QueueState][BatchJob x max_items][WorkItem x max_work]
    uint8_t* d_buf = nullptr;
    uint8_t* h_buf = nullptr;       // pinned staging of [QueueState][BatchJob x max_items]
    size_t buf_bytes = 0;
    cudaStream_t capture_stream = nullptr;
    // per-format branches of the captured graph (created with the first graph)
    cudaStream_t branch[kFormats] = {};
    cudaEvent_t fork = nullptr, join[kFormats] = {};
    cudaEvent_t done = nullptr;       // the last batch's graph has finished
    cudaEvent_t uploaded = nullptr;   // the last batch's descriptors have left h_buf
    bool pending = false;
    std::map<unsigned, cudaGraphExec_t> graphs;   // key: precision << 16 | format mask
};

namespace {

size_t jobs_offset() { return (sizeof(QueueState) + 255) & ~(size_t)255; }
size_t items_offset(int max_items) {
    return (jobs_offset() + (size_t)max_items * sizeof(BatchJob) + 255) & ~(size_t)255;
}

// Checks item i of a batch call and adds its block count to *blocks.
astc_status validate_item(const astc_batch_item& t, int i, long long* blocks, SpanCache* seen) {
    if (t.block_dim != 4 && t.block_dim != 6)
        return set_error(ASTC_ERR_INVALID_ARG, "item " + std::to_string(i) + ": block_dim must be 4 or 6");
    if (t.width <= 0 || t.height <= 0 || t.width > 0xFFFFFF || t.height > 0xFFFFFF)
        return set_error(ASTC_ERR_INVALID_ARG, "item " + std::to_string(i) + ": bad size");
    if (t.border != ASTC_BORDER_ZERO && t.border != ASTC_BORDER_CLAMP)
        return set_error(ASTC_ERR_INVALID_ARG, "item " + std::to_string(i) + ": bad border");
    const size_t pitch = t.row_pitch ? t.row_pitch : (size_t)t.width * 4;
    if (pitch < (size_t)t.width * 4 || pitch % 4)
        return set_error(ASTC_ERR_INVALID_ARG, "item " + std::to_string(i) + ": bad row_pitch");
    if (!t.rgba8 || !t.out || reinterpret_cast<uintptr_t>(t.rgba8) % 4 || reinterpret_cast<uintptr_t>(t.out) % 16)
        return set_error(ASTC_ERR_INVALID_ARG,
                         "item " + std::to_string(i) + ": rgba8 must be 4-byte and out 16-byte aligned");
    const long long nb = (long long)blocks_x(t.width, t.block_dim) * blocks_y(t.height, t.block_dim);
    if (nb > (1LL << 31)) return set_error(ASTC_ERR_INVALID_ARG, "texture has more than 2^31 blocks");
    astc_status st = check_device_span(t.rgba8, pitch * (size_t)(t.height - 1) + (size_t)t.width * 4, "rgba8",
                                       true, seen);
    if (st == ASTC_OK) st = check_device_span(t.out, (size_t)nb * 16, "out", true, seen);
    if (st != ASTC_OK) return set_error(st, "item " + std::to_string(i) + ": " + astc_last_error());
    *blocks += nb;
    return ASTC_OK;
}

// ASTC_GB300_BATCH_SERIAL=1 captures the formats' kernels one after another
// on one stream instead of as parallel branches (for comparison).
bool batch_serial() {
    static const bool on = [] {
        const char* v = getenv("ASTC_GB300_BATCH_SERIAL");
        return v && v[0] == '1';
    }();
    return on;
}

// Captures one persistent kernel per format in `mask` (the descriptor upload
// is issued before the launch with the exact sizes of each batch).  The
// kernels are parallel branches of the graph: each fills every SM slot it
// can get and drains its own format's queue, and the CTAs of the other
// formats take the slots as they free up, so no format's tail leaves the
// GPU idle before the next one starts.
astc_status build_graph(astc_batch* b, unsigned mask, int prec, cudaGraphExec_t* out) {
    cudaError_t e = cudaSuccess;
    if (!b->fork) {
        e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
        for (int f = 0; f < kFormats && e == cudaSuccess; ++f) {
            e = cudaStreamCreateWithFlags(&b->branch[f], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[f], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) return cuda_error(e, "batch branch streams");
    }
    const bool serial = batch_serial();
    cudaStream_t s = b->capture_stream;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamBeginCapture");
    auto* q = reinterpret_cast<QueueState*>(b->d_buf);
    auto* jobs = reinterpret_cast<BatchJob*>(b->d_buf + jobs_offset());
    auto* items = reinterpret_cast<WorkItem*>(b->d_buf + items_offset(b->max_items));
    astc_batch_expand<<<4 * b->sms, kBatchThreads, 0, s>>>(jobs, items, q);
    e = cudaGetLastError();
    if (!serial && e == cudaSuccess) e = cudaEventRecord(b->fork, s);
    for (int f = 0; f < kFormats && e == cudaSuccess; ++f) {
        if (!(mask & (1u << f))) continue;
        KernelFn k = prec == ASTC_PRECISION_HALF2 ? kernel_for<ASTC_PRECISION_HALF2>(f)
                                                  : kernel_for<ASTC_PRECISION_FP32>(f);
        const size_t smem = dyn_smem(f, prec);
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBatchThreads, smem);
        if (e != cudaSuccess) break;
        const int grid = (occ > 0 ? occ : 1) * b->sms;
        cudaStream_t ks = serial ? s : b->branch[f];
        if (!serial && (e = cudaStreamWaitEvent(ks, b->fork, 0)) != cudaSuccess) break;
        k<<<grid, kBatchThreads, smem, ks>>>(jobs, items, q, f);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if (!serial) {
            if ((e = cudaEventRecord(b->join[f], ks)) != cudaSuccess) break;
            e = cudaStreamWaitEvent(s, b->join[f], 0);
        }
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_error(e != cudaSuccess ? e : e2, "batch graph capture");
    }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphInstantiate");
    return ASTC_OK;
}

}  // namespace

extern "C" {

astc_status astc_batch_create(int max_textures, long long max_blocks, astc_batch** out) {
    if (!out) return set_error(ASTC_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (max_textures <= 0 || max_blocks <= 0 || max_blocks > (1LL << 36))
        return set_error(ASTC_ERR_INVALID_ARG, "max_textures and max_blocks must be positive");
    const long long work = max_blocks / kBatchThreads + max_textures + 1;
    if (work > (1LL << 30)) return set_error(ASTC_ERR_INVALID_ARG, "batch too large");
    astc_batch* b = new (std::nothrow) astc_batch();
    if (!b) return set_error(ASTC_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->max_items = max_textures;
    b->max_blocks = max_blocks;
    b->max_work = (int)work;
    b->buf_bytes = items_offset(max_textures) + (size_t)b->max_work * sizeof(WorkItem);
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_buf), b->buf_bytes);
    // the host stages the queue header and descriptors only (items are built on the device)
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&b->h_buf), items_offset(max_textures));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->uploaded, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        const astc_status st = cuda_error(e, "batch allocation");
        astc_batch_destroy(b);
        return st;
    }
    memset(b->h_buf, 0, items_offset(max_textures));
    *out = b;
    return ASTC_OK;
}

astc_status astc_batch_encode(astc_batch* b, const astc_batch_item* in, int count, int precision,
                              void* stream) {
    if (!b || (!in && count > 0)) return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    if (count < 0 || count > b->max_items)
        return set_error(ASTC_ERR_INVALID_ARG, "count exceeds the batch's max_textures");
    if (precision != ASTC_PRECISION_FP32 && precision != ASTC_PRECISION_HALF2)
        return set_error(ASTC_ERR_INVALID_ARG, "precision must be FP32 or HALF2");
    try {
        std::lock_guard<std::mutex> lk(b->mu);
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
        if (dev != b->device) return set_error(ASTC_ERR_INVALID_ARG, "batch was created on another device");
        // plan: validate, count work items per format
        long long blocks = 0;
        int per_fmt[kFormats] = {};
        SpanCache seen;
        for (int i = 0; i < count; ++i) {
            const astc_batch_item& t = in[i];
            const long long before = blocks;
            const astc_status st = validate_item(t, i, &blocks, &seen);
            if (st != ASTC_OK) return st;
            per_fmt[format_index(t.block_dim, t.has_alpha, t.is_normal, t.srgb)] +=
                (int)((blocks - before + kBatchThreads - 1) / kBatchThreads);
        }
        if (blocks > b->max_blocks) return set_error(ASTC_ERR_INVALID_ARG, "batch exceeds max_blocks");
        // the previous batch's upload must have left the pinned staging buffer
        // (the host waits for that only; its kernels may still be running)
        if (b->pending) {
            if ((e = cudaEventSynchronize(b->uploaded)) != cudaSuccess) return cuda_error(e, "previous batch");
        }
        auto* q = reinterpret_cast<QueueState*>(b->h_buf);
        auto* jobs = reinterpret_cast<BatchJob*>(b->h_buf + jobs_offset());
        unsigned mask = 0;
        int cursor[kFormats];
        int total = 0;
        for (int f = 0; f < kFormats; ++f) {
            q->counter[f] = 0;
            q->begin[f] = total;
            cursor[f] = total;
            total += per_fmt[f];
            q->end[f] = total;
            if (per_fmt[f]) mask |= 1u << f;
        }
        for (int i = 0; i < count; ++i) {
            const astc_batch_item& t = in[i];
            EncodeJob j;
            j.in = t.rgba8;
            j.pitch = t.row_pitch ? t.row_pitch : (size_t)t.width * 4;
            j.width = t.width;
            j.height = t.height;
            j.block_dim = t.block_dim;
            j.has_alpha = t.has_alpha;
            j.is_normal = t.is_normal;
            j.srgb = t.srgb;
            j.border = t.border;
            j.precision = precision;
            j.out = t.out;
            jobs[i].tex = make_view(j);
            jobs[i].out = reinterpret_cast<uint4*>(t.out);
            const int nb = blocks_x(t.width, t.block_dim) * blocks_y(t.height, t.block_dim);
            int& c = cursor[format_index(t.block_dim, t.has_alpha, t.is_normal, t.srgb)];
            jobs[i].item_start = c;
            jobs[i].nblocks = nb;
            c += (nb + kBatchThreads - 1) / kBatchThreads;
        }
        q->njobs = count;
        if (!mask) return ASTC_OK;
        const unsigned key = ((unsigned)precision << 16) | mask;
        auto it = b->graphs.find(key);
        if (it == b->graphs.end()) {
            cudaGraphExec_t g = nullptr;
            astc_status st = build_graph(b, mask, precision, &g);
            if (st != ASTC_OK) return st;
            it = b->graphs.emplace(key, g).first;
        }
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        // the device buffers are rewritten only after the previous batch's
        // kernels have finished with them, whatever stream each call uses
        if (b->pending && (e = cudaStreamWaitEvent(s, b->done, 0)) != cudaSuccess)
            return cuda_error(e, "cudaStreamWaitEvent");
        // upload exactly this batch's queue header + descriptors; the graph's
        // first kernel expands them into work items
        const size_t head = jobs_offset() + (size_t)count * sizeof(BatchJob);
        if ((e = cudaMemcpyAsync(b->d_buf, b->h_buf, head, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_error(e, "descriptor upload");
        if ((e = cudaEventRecord(b->uploaded, s)) != cudaSuccess) return cuda_error(e, "cudaEventRecord");
        if ((e = cudaGraphLaunch(it->second, s)) != cudaSuccess) return cuda_error(e, "cudaGraphLaunch");
        if ((e = cudaEventRecord(b->done, s)) != cudaSuccess) return cuda_error(e, "cudaEventRecord");
        b->pending = true;
        int kernels = 1;                                  // the item expansion
        for (int f = 0; f < kFormats; ++f) kernels += (mask >> f) & 1;
        count_launches((uint64_t)kernels);
        if (!stream) {
            if ((e = cudaEventSynchronize(b->done)) != cudaSuccess) return cuda_error(e, "batch encode");
            b->pending = false;
        }
        return ASTC_OK;
    } catch (const std::bad_alloc&) {
        return set_error(ASTC_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (...) {
        return set_error(ASTC_ERR_CUDA, "unexpected exception");
    }
}

astc_status astc_batch_encode_quality(astc_batch* b, const astc_batch_item* in, int count, int precision,
                                      int quality, void* stream) {
    if (quality == ASTC_QUALITY_FAST) return astc_batch_encode(b, in, count, precision, stream);
    if (!b || (!in && count > 0)) return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    if (quality < ASTC_QUALITY_FAST || quality > ASTC_QUALITY_THREE_PARTITIONS)
        return set_error(ASTC_ERR_INVALID_ARG, "bad quality");
    if (precision != ASTC_PRECISION_FP32)
        return set_error(ASTC_ERR_UNSUPPORTED, "the quality modes are FP32 only");
    if (count < 0 || count > b->max_items)
        return set_error(ASTC_ERR_INVALID_ARG, "count exceeds the batch's max_textures");
    try {
        std::lock_guard<std::mutex> lk(b->mu);
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
        if (dev != b->device) return set_error(ASTC_ERR_INVALID_ARG, "batch was created on another device");
        long long blocks = 0;
        SpanCache seen;
        for (int i = 0; i < count; ++i) {
            const astc_status st = validate_item(in[i], i, &blocks, &seen);
            if (st != ASTC_OK) return st;
        }
        if (blocks > b->max_blocks) return set_error(ASTC_ERR_INVALID_ARG, "batch exceeds max_blocks");
        // one quality-mode kernel per texture on the stream (these kernels run
        // for tens of microseconds or more, so launches do not dominate)
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        for (int i = 0; i < count; ++i) {
            const astc_batch_item& t = in[i];
            EncodeJob j;
            j.in = t.rgba8;
            j.pitch = t.row_pitch ? t.row_pitch : (size_t)t.width * 4;
            j.width = t.width;
            j.height = t.height;
            j.block_dim = t.block_dim;
            j.has_alpha = t.has_alpha;
            j.is_normal = t.is_normal;
            j.srgb = t.srgb;
            j.border = t.border;
            j.precision = ASTC_PRECISION_FP32;
            j.quality = quality;
            j.out = t.out;
            if ((e = launch_encode_search(j, s)) != cudaSuccess) return cuda_error(e, "quality kernel launch");
        }
        if (!stream && (e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_error(e, "batch encode");
        return ASTC_OK;
    } catch (...) {
        return set_error(ASTC_ERR_CUDA, "unexpected exception");
    }
}

astc_status astc_batch_destroy(astc_batch* b) {
    if (!b) return ASTC_OK;
    int cur = 0;
    const bool have = cudaGetDevice(&cur) == cudaSuccess;
    cudaSetDevice(b->device);
    if (b->pending && b->done) cudaEventSynchronize(b->done);
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    for (int f = 0; f < kFormats; ++f) {
        if (b->branch[f]) cudaStreamDestroy(b->branch[f]);
        if (b->join[f]) cudaEventDestroy(b->join[f]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->done) cudaEventDestroy(b->done);
    if (b->uploaded) cudaEventDestroy(b->uploaded);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    if (b->d_buf) cudaFree(b->d_buf);
    if (b->h_buf) cudaFreeHost(b->h_buf);
    if (have) cudaSetDevice(cur);
    cudaGetLastError();
    delete b;
    return ASTC_OK;
}

}  // extern "C"
