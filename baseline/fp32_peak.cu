// FP32 throughput probe: the FP32-pipe roofline denominator of this device,
// for bench.py (measurement infrastructure; the renderer never loads it).
// Every thread runs eight independent fused multiply-add chains on registers
// (no memory traffic inside the loop), with enough warps per SM to cover the
// FFMA latency.  FLOPs = 2 per FMA.  Best of several timed launches.
#include <cuda_runtime.h>

namespace {

constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) k_ffma(float* out, float a, float b)
{
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.0f, x2 = x0 + 2.0f, x3 = x0 + 3.0f;
    float x4 = x0 + 4.0f, x5 = x0 + 5.0f, x6 = x0 + 6.0f, x7 = x0 + 7.0f;
#pragma unroll 16
    for (int i = 0; i < kIters; ++i) {
        x0 = __fmaf_rn(x0, a, b); x1 = __fmaf_rn(x1, a, b); x2 = __fmaf_rn(x2, a, b); x3 = __fmaf_rn(x3, a, b);
        x4 = __fmaf_rn(x4, a, b); x5 = __fmaf_rn(x5, a, b); x6 = __fmaf_rn(x6, a, b); x7 = __fmaf_rn(x7, a, b);
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

// Returns a cudaError_t as int; *tflops = FP32 TFLOP/s of the device.
extern "C" __attribute__((visibility("default"))) int fp32_peak_tflops(int device, double* tflops)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return e;
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) return e;
    const int threads = 256;
    const int blocks = prop.multiProcessorCount * 8;
    float* out = nullptr;
    e = cudaMalloc(&out, sizeof(float) * threads * blocks);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double best = 0.0;
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
        cudaEventRecord(a);
        k_ffma<<<blocks, threads>>>(out, 0.999999f, 1e-7f);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && rep > 0 && ms > 0.0f) {
            const double flops = 2.0 * 8.0 * kIters * (double)threads * blocks;
            const double t = flops / (ms * 1e-3) / 1e12;
            if (t > best) best = t;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return e;
    *tflops = best;
    return cudaGetLastError();
}
