/*
 * astc_gb300.h -- C ABI of the GB300 (sm_103a) ASTC LDR block encoder.
 *
 * Plain pointers and sizes only; no CUDA, torch or C++ types in any
 * signature (streams are passed as void*, i.e. a cudaStream_t).
 *
 * Reference interfaces replaced (niepp/astc_encoder):
 *   encode_option                 astc_encode.h:14-28   -> astc_opts
 *   encode_astc + Dispatch        astc_encode.h:87-194  -> astc_encode_gpu
 *   read_gpu (staging + Map)      astc_save.h:34-50     -> the D2H copy inside
 *                                                          astc_encode_gpu
 *   astc_header / save_astc       astc_save.h:5-14,52-76 -> astc_save_file
 *   MainCS (one block per thread) ASTC_Encode.hlsl:553-582 -> the CUDA kernels
 *                                                          behind astc_encode_gpu
 *
 * Errors: every entry point returns an astc_status; a human-readable message
 * for the last failure on the calling thread is in astc_last_error().  No
 * entry point aborts the process or lets a C++ exception escape.
 */
#ifndef ASTC_GB300_H
#define ASTC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASTC_GB300_VERSION_MAJOR 1
#define ASTC_GB300_VERSION_MINOR 0

typedef enum astc_status {
    ASTC_OK = 0,
    ASTC_ERR_INVALID_ARG = 1,    /* bad pointer, size or option            */
    ASTC_ERR_UNSUPPORTED = 2,    /* option combination not implemented     */
    ASTC_ERR_CUDA = 3,           /* a CUDA runtime call failed             */
    ASTC_ERR_OUT_OF_MEMORY = 4,  /* device or pinned allocation failed     */
    ASTC_ERR_IO = 5,             /* file open / read / write failed        */
    ASTC_ERR_TIMEOUT = 6,        /* a bounded device wait ran out          */
    ASTC_ERR_BUSY = 7,           /* admission refused (no memory / slots)  */
    ASTC_ERR_CANCELLED = 8,      /* request cancelled before it ran        */
    ASTC_ERR_FORMAT = 9          /* malformed .astc file                   */
} astc_status;

typedef enum astc_border {
    ASTC_BORDER_ZERO = 0,        /* texels outside the image read as 0
                                    (the reference's Texture2D.Load rule,
                                    ASTC_Encode.hlsl:574)                   */
    ASTC_BORDER_CLAMP = 1        /* texels outside repeat the edge texel    */
} astc_border;

typedef enum astc_precision {
    ASTC_PRECISION_FP32 = 0,     /* the reference's FP32 math, bit-exact
                                    with the FP32 oracle                    */
    ASTC_PRECISION_HALF2 = 1     /* per-texel projections in packed half2,
                                    FP32 accumulation                       */
} astc_precision;

typedef enum astc_memory {
    ASTC_MEMORY_HOST = 0,        /* input and output are host pointers      */
    ASTC_MEMORY_DEVICE = 1       /* input and output are device pointers    */
} astc_memory;

typedef enum astc_axis {
    ASTC_AXIS_PCA = 0,           /* principal_component_analysis, the
                                    reference's fit (ASTC_Encode.hlsl:514)   */
    ASTC_AXIS_MAX_ACCUMULATION = 1, /* max_accumulation_pixel_direction,
                                    the reference's alternative fit, defined
                                    but commented out (170-227, 515)         */
    ASTC_AXIS_BEST = 2           /* both fits; the one whose fixed-mode
                                    block decodes with the smaller squared
                                    error against the texels rounded to
                                    bytes (the PCA on ties) is kept, or with
                                    ASTC_QUALITY_SEARCH searched from.  Most
                                    of THOROUGH's gain on alpha cut-outs at
                                    4-6 times THOROUGH's speed (40-55% of
                                    the fixed mode's); FP32 only (THOROUGH
                                    and above use both fits whatever the
                                    axis)                                   */
} astc_axis;

typedef enum astc_quality {
    ASTC_QUALITY_FAST = 0,       /* the reference's fixed mode (518-522):
                                    QUANT_12 (RGB) / QUANT_6 (RGBA) weights,
                                    QUANT_256 endpoints                     */
    ASTC_QUALITY_SEARCH = 1,     /* the fixed-mode block and every single-
                                    partition 4x4-grid mode (weight ranges
                                    QUANT_3..QUANT_32, each with the largest
                                    endpoint range that fits), keeping the
                                    one whose decode has the least squared
                                    error against the texels rounded to
                                    bytes in the fit space; the
                                    choose_best_quantmethod the
                                    reference sketches (524-526).  Never
                                    worse than FAST; FP32 only              */
    ASTC_QUALITY_THOROUGH = 2,   /* SEARCH from the better of the two fits
                                    (PCA and max accumulation both run; the
                                    one whose fixed-mode block decodes with
                                    less error is searched from, PCA on
                                    ties; opts.axis is ignored), plus
                                    single-partition dual-plane blocks: one
                                    channel on its own weight plane (the one
                                    whose removal leaves the least off-axis
                                    variance), the others fitted without it,
                                    every legal weight range scored (the
                                    reference writes the dual-plane bit as 0,
                                    ASTC_Encode.hlsl:446-473).  Recovers the
                                    blocks the reference's PCA collapses
                                    (flat colour, varying alpha) and
                                    decorrelated channels; FP32 only        */
    ASTC_QUALITY_PARTITIONS = 3, /* THOROUGH plus two-partition blocks: the
                                    partition index whose pattern best
                                    matches the split along the kept fit,
                                    each partition fitted on its own, every
                                    legal weight range scored by its exact
                                    decode (the reference has only a
                                    commented-out layout stub for partitions,
                                    ASTC_Encode.hlsl:422-431); FP32 only    */
    ASTC_QUALITY_THREE_PARTITIONS = 4  /* PARTITIONS plus three-partition
                                    blocks for RGB input (three RGBA
                                    partitions would need 24 colour endpoint
                                    values, above the format's 18): the
                                    four pattern classes that best match an
                                    integer three-colour labelling of the
                                    texels, each partition fitted on its own,
                                    every legal weight range scored.  For
                                    flat-colour graphics (UI, sprites);
                                    RGBA input is encoded as PARTITIONS;
                                    FP32 only                               */
} astc_quality;

/* Encoder options: the reference's encode_option (astc_encode.h:14-28) plus
 * the GPU-side controls.  Use astc_opts_init() for the reference defaults. */
typedef struct astc_opts {
    int block_dim;   /* 4 (ASTC 4x4) or 6 (ASTC 6x6)               is4x4   */
    int has_alpha;   /* CEM 12 + QUANT_6 weights, else CEM 8 + QUANT_12    */
    int is_normal;   /* normal map: blue and alpha forced to 1.0           */
    int srgb;        /* input is sRGB-encoded: RGB are linearised before
                        the fit (R8G8B8A8_UNORM_SRGB sampling, main.cpp:38) */
    int border;      /* astc_border                                        */
    int precision;   /* astc_precision                                     */
    int memory;      /* astc_memory: where `rgba8` and `out` live          */
    void* stream;    /* cudaStream_t to run on asynchronously; NULL = the
                        library's own stream (ordered after earlier work on
                        the legacy default stream), and the call returns
                        when the result is in `out` (for asynchronous work
                        on the legacy default stream pass cudaStreamLegacy,
                        (void*)0x1, not NULL)                               */
    int axis;        /* astc_axis (FP32 only)                               */
    int quality;     /* astc_quality (FP32 only)                            */
} astc_opts;

/* Fills the reference defaults: 4x4, no alpha, not a normal map, linear,
 * zero border, FP32, host memory, synchronous, PCA axis, fixed mode. */
void astc_opts_init(astc_opts* opts);

/* Bytes of ASTC blocks for a w x h image: 16 * ceil(w/dim) * ceil(h/dim). */
size_t astc_encoded_size(int width, int height, int block_dim);

/* Encode one RGBA8 image (tightly packed rows, row 0 first, 4 bytes per
 * texel) into 16-byte ASTC blocks in row-major block order.
 * Replaces encode_astc (astc_encode.h:87) + read_gpu (astc_save.h:34).
 * `out` must hold astc_encoded_size(width, height, opts->block_dim) bytes.
 * Host memory: pinned buffers are accessed in place by the kernel
 * (zero-copy), and so are pageable buffers on a device that reads the host's
 * page tables (astc_device_caps.pageable_in_place: Grace systems over
 * NVLink-C2C); other buffers are staged.  The call returns when `out` is
 * written, except when both buffers are pinned and opts->stream is set --
 * then it is asynchronous on that stream like a device-memory call.  A host
 * buffer the device accesses in place must hold its whole extent, writable
 * for `out`: the device faults where a host copy would have.  Pages of a
 * pageable `out` that the host has never touched are faulted in by the
 * device's first write to them, which is slow (reuse or fill such buffers). */
astc_status astc_encode_gpu(const uint8_t* rgba8, int width, int height,
                            const astc_opts* opts, uint8_t* out);

/* As astc_encode_gpu with an explicit input row pitch in bytes (>= 4*width,
 * a multiple of 4). */
astc_status astc_encode_gpu_pitched(const uint8_t* rgba8, int width, int height,
                                    size_t row_pitch, const astc_opts* opts,
                                    uint8_t* out);

/* ---- batched encode (one CUDA-graph launch for many textures) -----------
 * The reference encodes one texture per Dispatch (astc_encode.h:190).  A
 * batch encodes any list of textures -- different sizes, mip levels and
 * formats -- in one graph launch: the blocks are split into work items of
 * 128 blocks, grouped by format, and persistent kernels drain the items from
 * a device work queue.  Every texture's blocks are identical to what
 * astc_encode_gpu returns for it with the same precision. */
typedef struct astc_batch_item {
    const uint8_t* rgba8;   /* device memory, 4-byte aligned (or host memory
                               the device reaches in place: pinned, or
                               pageable where astc_device_caps.
                               pageable_in_place; the caller keeps it alive
                               until the stream has run the batch)          */
    size_t row_pitch;       /* bytes between rows; 0 = 4 * width             */
    int width, height;
    int block_dim, has_alpha, is_normal, srgb, border;   /* as astc_opts     */
    uint8_t* out;           /* the same kinds of memory, 16-byte aligned,
                               16 B / block                                  */
} astc_batch_item;

typedef struct astc_batch astc_batch;   /* opaque; owns descriptor buffers,
                                           a pinned staging copy and the
                                           captured graphs               */

/* Capacity: up to max_textures items and max_blocks blocks per call. */
astc_status astc_batch_create(int max_textures, long long max_blocks, astc_batch** out);
/* Encode `count` items with `precision` on `stream` (asynchronous; NULL =
 * the legacy default stream, and the call returns when the blocks are
 * written).  A call waits for the previous call's descriptor upload before
 * it reuses the staging buffer.  Not thread-safe per handle across streams. */
astc_status astc_batch_encode(astc_batch* batch, const astc_batch_item* items, int count,
                              int precision, void* stream);
/* The same with a quality mode (astc_quality).  ASTC_QUALITY_FAST is
 * astc_batch_encode; the search modes (FP32 only) launch one quality-mode
 * kernel per item on `stream`; every texture's blocks equal its
 * astc_encode_gpu result with that quality. */
astc_status astc_batch_encode_quality(astc_batch* batch, const astc_batch_item* items, int count,
                                      int precision, int quality, void* stream);
astc_status astc_batch_destroy(astc_batch* batch);

/* ---- serving: continuous batching of single-texture requests -----------
 * (No counterpart in the reference, a one-shot command line tool.)  A server
 * owns a device staging pool and a worker thread.  Requests (host buffers)
 * queue in arrival order; whenever an in-flight slot is free the worker
 * admits queued requests, in order, while their inputs and outputs fit in
 * the free pool memory (admission by memory) and the batch has room, copies
 * them in, encodes them with one batched graph launch (or, in per-request
 * mode, one plain kernel launch each) and copies the blocks back, all on the
 * slot's stream.  Up to `inflight` slots run at once, so requests arriving
 * while others are on the GPU are admitted as memory and slots free up, and
 * their copies and kernels overlap with the work in flight.  A request's
 * blocks are the same as astc_encode_gpu's for it, alone or in any mix. */
typedef enum astc_serve_mode {
    ASTC_SERVE_BATCHED = 0,       /* continuous batching through astc_batch */
    ASTC_SERVE_PER_REQUEST = 1    /* one plain launch per request           */
} astc_serve_mode;

typedef struct astc_server_config {
    size_t pool_bytes;   /* device staging pool for inputs + outputs           */
    int max_batch;       /* requests per batch (batched mode)                   */
    int inflight;        /* slots (batches or requests) in flight, 1..16        */
    int precision;       /* astc_precision                                      */
    int mode;            /* astc_serve_mode                                     */
    int quality;         /* astc_quality of every request (FP32 for the search
                            modes)                                              */
} astc_server_config;

typedef struct astc_request {
    const uint8_t* rgba8;   /* host memory, read in place when the device reaches
                               it (pinned, or pageable where astc_device_caps.
                               pageable_in_place), else staged through the pool */
    size_t row_pitch;       /* 0 = 4 * width                                     */
    int width, height;
    int block_dim, has_alpha, is_normal, srgb, border;
    uint8_t* out;           /* host memory, astc_encoded_size() bytes            */
} astc_request;

typedef struct astc_request_stats {
    double submit_us, admit_us, done_us;   /* server clock, microseconds        */
    int status;                            /* astc_status of the request        */
} astc_request_stats;

typedef struct astc_server astc_server;

astc_status astc_server_create(const astc_server_config* config, astc_server** out);
/* Queues a request (non-blocking); *ticket identifies it.  Requests larger
 * than the whole pool are rejected with ASTC_ERR_BUSY. */
astc_status astc_server_submit(astc_server* server, const astc_request* request, uint64_t* ticket);
/* Waits up to timeout_ms (< 0: no limit) for a request; ASTC_ERR_TIMEOUT if
 * it is not done yet (the ticket stays valid), else the request's status
 * (the ticket is then released). */
astc_status astc_server_wait(astc_server* server, uint64_t ticket, int timeout_ms,
                             astc_request_stats* stats);
/* Cancels a request that is still queued (ASTC_ERR_BUSY once admitted). */
astc_status astc_server_cancel(astc_server* server, uint64_t ticket);
/* Load replay: submits request i at arrival_us[i] after the start (open
 * loop), waits for all, and returns each request's latency from its
 * scheduled arrival to its completion, plus the wall time. */
astc_status astc_server_replay(astc_server* server, const astc_request* requests,
                               const double* arrival_us, int count, double* latency_us,
                               double* wall_s);
/* Device-side record of the slot launches retired since the last reset
 * (timing events recorded on each slot's stream before its first copy and
 * after its last): how busy the device was and how much the slots' work
 * overlapped.  The record holds at most the most recent 2^20 launches.
 * (No counterpart in the reference.) */
typedef struct astc_server_stats {
    long long launches;          /* slot launches (batches, or requests)       */
    long long requests;          /* requests they carried                      */
    int max_requests_per_launch;
    double device_busy_s;        /* union of the launches' device intervals    */
    double device_overlap_s;     /* time with two or more slots on the device  */
    double device_slot_s;        /* sum of the intervals (busy x mean depth)   */
    double device_span_s;        /* first interval start to last interval end  */
} astc_server_stats;
astc_status astc_server_get_stats(astc_server* server, int reset, astc_server_stats* out);
/* Waits for the work in flight, then frees the server. */
astc_status astc_server_destroy(astc_server* server);

/* ---- mip chains (staging in front of the batched encoder) --------------
 * (No counterpart in the reference, which encodes one level: main.cpp:36.)
 * Level l+1 is max(1, w/2) x max(1, h/2); each texel is the rounded mean of
 * the 2x2 texels below it (edge-clamped for a width or height of 1); with
 * `srgb` the RGB channels are averaged in linear light.  Levels 1..levels-1
 * are written back to back into `out` (device memory, tight rows). */
int astc_mip_levels(int width, int height);            /* full chain length   */
size_t astc_mip_chain_bytes(int width, int height, int levels);
astc_status astc_generate_mips(const uint8_t* rgba8, int width, int height, int levels,
                               int srgb, uint8_t* out, void* stream);

/* Write a .astc file: the 16-byte header of astc_save.h:5-14 (magic
 * 0x5CA1AB13, block dims, 24-bit x/y/z sizes, z = 1) then the blocks.
 * Replaces save_astc (astc_save.h:52-76), which did not check fopen. */
astc_status astc_save_file(const char* path, int block_dim_x, int block_dim_y,
                           int width, int height, const uint8_t* blocks,
                           size_t blocks_size);

/* Read a .astc file written by astc_save_file (or any 2-D .astc).  On
 * ASTC_OK the width, height and block dimensions are stored through their
 * pointers; when `blocks` is
 * non-NULL up to `capacity` block bytes are copied.  *blocks_size receives
 * the block byte count.  (No counterpart in the reference, which only
 * writes.) */
astc_status astc_load_file(const char* path, int* block_dim_x, int* block_dim_y,
                           int* width, int* height, uint8_t* blocks,
                           size_t capacity, size_t* blocks_size);

/* Integer-only ASTC LDR decode of `blocks` (block_w x block_h footprint) to
 * tightly packed RGBA8 on the GPU; memory/stream as in astc_opts.  Error
 * blocks decode to magenta.  (No counterpart in the reference.) */
astc_status astc_decode_gpu(const uint8_t* blocks, int width, int height,
                            int block_w, int block_h, int srgb, int memory,
                            void* stream, uint8_t* out_rgba8);

/* Sum of squared differences between two RGBA8 images per channel (R, G, B,
 * A), reduced on the GPU; both images in `memory`.  (No counterpart in the
 * reference.) */
astc_status astc_sse_gpu(const uint8_t* a, const uint8_t* b, size_t texels,
                         int memory, void* stream, uint64_t sse_rgba[4]);

/* Squared error of two normal maps in the -norm layout (the reference keeps
 * X and Y in R and G, ASTC_Encode.hlsl:575-578), measured on the rebuilt unit
 * normals: x, y = code * 2/255 - 1, z = sqrt(max(0, 1 - x^2 - y^2)); each
 * component's difference is scaled by 127.5 so an 8-bit peak of 255 applies
 * to PSNR over 3 * texels values.  Reduced on the GPU in FP64; memory/stream
 * as in astc_sse_gpu.  (No counterpart in the reference.) */
astc_status astc_normal_sse_gpu(const uint8_t* a, const uint8_t* b, size_t texels,
                                int memory, void* stream, double* sse);

/* Kernel variant of a format: where a block's decoded texels live
 * (store 0 = registers, 1 = shared memory, 2 = registers with the count
 * capped for occupancy, at most 128 threads) or, store 3, the cooperative
 * mapping: four lanes of a warp share one block (a warp encodes eight
 * blocks; texels staged in a shared-memory tile; 64/128/256 threads), which
 * shortens each block's path for launches too small to fill the GPU; and
 * the CTA size (32/64/128/256).  Every variant produces identical blocks;
 * they differ in speed only.  Choices are kept per format and per size
 * class: textures with fewer blocks than one wave of the one-thread
 * mappings (SMs x 384 blocks) and the rest.  (No counterpart in the
 * reference, whose shader has one fixed mapping, one thread per block,
 * [numthreads(8,8,1)] at ASTC_Encode.hlsl:553-561.) */
typedef struct astc_tune_result {
    int store;
    int threads;
    float best_us;      /* fastest variant, microseconds per launch       */
    float default_us;   /* the variant that was installed before tuning   */
} astc_tune_result;

/* Time every variant for a format on a synthetic width x height texture on
 * the current device and install the fastest for that format and that
 * size class in this process (it allocates its own test buffers). */
astc_status astc_autotune(int block_dim, int has_alpha, int is_normal, int srgb,
                          int width, int height, astc_tune_result* result);
/* Install a variant for a format, for every texture size. */
astc_status astc_set_kernel_choice(int block_dim, int has_alpha, int is_normal, int srgb,
                                   int store, int threads);
/* The variant installed for a format's textures of one wave or more. */
astc_status astc_get_kernel_choice(int block_dim, int has_alpha, int is_normal, int srgb,
                                   int* store, int* threads);
/* The variant astc_encode_gpu uses for a texture of this size. */
astc_status astc_get_kernel_choice_for_size(int block_dim, int has_alpha, int is_normal, int srgb,
                                            int width, int height, int* store, int* threads);

/* astc_sse_gpu for callers that may not allocate device memory (no
 * counterpart in the reference).  Some hosts own the whole device-memory
 * budget through their own allocator and forbid a library from allocating
 * behind their back (game engines, texture-streaming and serving processes
 * that admit work by memory); in real-time loops a cudaMalloc/cudaFree would
 * also synchronise the device mid-frame.  This entry point calls no
 * cudaMalloc/cudaFree: `a` and `b` (RGBA8, 4-byte aligned) and `sse_rgba`
 * (4 x uint64, 8-byte aligned) are all caller-owned DEVICE memory, and its
 * scratch is a fixed static device array (one partial per chunk of 8,192 to
 * 65,536 texels, 4096 partials = 128 KiB) that every GPU loading this
 * library holds until exit.  Limit: texels <= 2^28 (268,435,456); larger calls return
 * ASTC_ERR_INVALID_ARG.  Asynchronous on `stream` (NULL = the legacy default
 * stream).  The first call on a device looks up the scratch address with
 * that device current; make that first call before any stream capture.
 * Calls share the scratch: calls whose kernels overlap on the GPU race. */
astc_status astc_sse_gpu_noalloc(const uint8_t* a, const uint8_t* b, size_t texels,
                                 void* stream, uint64_t* sse_rgba);

/* What the current device offers the host-memory paths.  (No counterpart in
 * the reference.)  With `zero_copy` set, host-memory calls whose buffers are
 * pinned (page-locked and device-mapped) let the kernels read texels and
 * write blocks directly through the host link instead of staging them in
 * device memory; with `pageable_in_place` set, ordinary pageable buffers
 * (malloc, new, numpy) are accessed the same way; other host buffers are
 * staged. */
typedef struct astc_device_caps {
    int sm_count;
    int l2_bytes;
    int unified_addressing;          /* pinned host memory has a device view    */
    int can_map_host_memory;
    int pageable_memory_access;
    int pageable_uses_host_page_tables;
    int zero_copy;                   /* the library uses zero-copy for pinned buffers */
    int pageable_in_place;           /* ... and accesses pageable buffers in place */
} astc_device_caps;
astc_status astc_get_device_caps(astc_device_caps* caps);

/* Message for the last failed call on this thread ("" if none). */
const char* astc_last_error(void);
const char* astc_status_string(astc_status status);

/* Number of kernels this library has launched in this process. */
uint64_t astc_kernel_launch_count(void);

/* Free the library's pooled device and pinned memory and streams. */
void astc_shutdown(void);

#ifdef __cplusplus
}
#endif
#endif
