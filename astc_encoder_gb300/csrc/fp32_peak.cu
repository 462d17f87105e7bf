// fp32_peak.cu -- FP32 fused multiply-add throughput of the GPU, the
// denominator of the encoder's FP32-issue roofline (libastc_fp32_peak.so,
// loaded by the benchmark only; not part of the encoder library).
//
// Every thread runs 8 independent FMA chains (x = x * a + b) for `iters`
// rounds, unrolled by 4, so the FMA pipe is the only busy unit; 4 CTAs of 256
// threads per SM.  The chains' sum is written only if it equals a value it
// cannot reach, which keeps the work from being removed.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) fma_chains(float* sink, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = (float)(threadIdx.x + j) * 1e-3f;
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = __fmaf_rn(x[j], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == -1.0f) sink[blockIdx.x] = s;
}

}  // namespace

// Best of `reps` timed launches, in TFLOP/s (an FMA counts as 2 FLOPs).
// Returns 0 on success, else the CUDA error code.
extern "C" int astc_fp32_fma_peak(int reps, double* tflops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    const int threads = 256, grid = sms * 4, iters = 8192;
    float* sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if ((e = cudaMalloc(&sink, sizeof(float) * grid)) != cudaSuccess) return (int)e;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    double best = 0.0;
    for (int r = -1; r < reps && e == cudaSuccess; ++r) {          // r = -1: warm-up
        cudaEventRecord(t0, s);
        fma_chains<<<grid, threads, 0, s>>>(sink, iters, 0.999f, 1e-3f);
        cudaEventRecord(t1, s);
        if ((e = cudaEventSynchronize(t1)) != cudaSuccess) break;
        float ms = 0.0f;
        if ((e = cudaEventElapsedTime(&ms, t0, t1)) != cudaSuccess) break;
        const double flops = 2.0 * 8.0 * iters * (double)grid * threads;
        if (r >= 0 && ms > 0.0f) best = best > flops / (ms * 1e-3) / 1e12 ? best : flops / (ms * 1e-3) / 1e12;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (s) cudaStreamDestroy(s);
    cudaFree(sink);
    if (e != cudaSuccess) return (int)e;
    *tflops = best;
    return 0;
}
