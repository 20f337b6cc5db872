// Throughput probes of the arithmetic units the dense Cholesky can use, the
// denominators of its roofline: FP64 fused multiply-add (DFMA), the FP64
// tensor instruction mma.sync m8n8k4 (DMMA) and the BF16 tensor instruction
// mma.sync m16n8k16 that the error-free split update issues. Each kernel
// keeps every SM busy with independent dependency chains (enough in flight
// to cover the unit's latency), is timed with CUDA events after a warm-up
// launch, and folds its registers into one store that never happens, so
// the compiler keeps the work.
#include <cuda_bf16.h>

#include "kernels.cuh"

namespace sfmba {

namespace {

constexpr int kPeakIters = 4096;

__global__ void __launch_bounds__(256) k_peak_dfma(double seed, double *sink) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x + k;
    const double b = 0.999999, c = 1e-7;
    for (int it = 0; it < kPeakIters; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == -1.0) *sink = s;
}

__global__ void __launch_bounds__(256) k_peak_dmma(double seed, double *sink) {
    double acc[4][2];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = 0.0;
    const double a = seed + 1e-3 * (threadIdx.x & 31), b = seed - 1e-3 * (threadIdx.x & 7);
    for (int it = 0; it < kPeakIters; ++it)
#pragma unroll
        for (int k = 0; k < 4; ++k)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                         : "+d"(acc[k][0]), "+d"(acc[k][1])
                         : "d"(a), "d"(b));
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) s += acc[k][0] + acc[k][1];
    if (s == -1.0) *sink = s;
}

__global__ void __launch_bounds__(256) k_peak_bf16(float seed, double *sink) {
    float acc[8][4];
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[k][e] = 0.0f;
    const __nv_bfloat162 v = __floats2bfloat162_rn(seed, seed * 0.5f);
    const unsigned a = *reinterpret_cast<const unsigned *>(&v);
    for (int it = 0; it < kPeakIters; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k)
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %4, %4, %4}, {%4, %4}, "
                "{%0, %1, %2, %3};\n"
                : "+f"(acc[k][0]), "+f"(acc[k][1]), "+f"(acc[k][2]), "+f"(acc[k][3])
                : "r"(a));
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += acc[k][0] + acc[k][1] + acc[k][2] + acc[k][3];
    if (s == -1.0f) *sink = s;
}

template <typename K, typename... Args>
double time_kernel(K kernel, int blocks, cudaStream_t s, Args... args) {
    cudaEvent_t e0, e1;
    SFMBA_CUDA(cudaEventCreate(&e0));
    SFMBA_CUDA(cudaEventCreate(&e1));
    kernel<<<blocks, 256, 0, s>>>(args...);  // warm-up
    SFMBA_LAUNCH_CHECK();
    SFMBA_CUDA(cudaEventRecord(e0, s));
    kernel<<<blocks, 256, 0, s>>>(args...);
    SFMBA_LAUNCH_CHECK();
    SFMBA_CUDA(cudaEventRecord(e1, s));
    SFMBA_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    SFMBA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms * 1e-3;
}

}  // namespace

PeakRates measure_peaks(cudaStream_t s, double *sink) {
    int dev = 0, sms = 0;
    SFMBA_CUDA(cudaGetDevice(&dev));
    SFMBA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8;
    const double threads = (double)blocks * 256, warps = threads / 32;
    PeakRates r;
    r.dfma_tflops = 2.0 * 8 * kPeakIters * threads / time_kernel(k_peak_dfma, blocks, s, 1.0, sink) * 1e-12;
    r.dmma_tflops = 2.0 * 256 * 4 * kPeakIters * warps / time_kernel(k_peak_dmma, blocks, s, 1.0, sink) * 1e-12;
    r.bf16_mma_tflops =
        2.0 * 4096 * 8 * kPeakIters * warps / time_kernel(k_peak_bf16, blocks, s, 1.0f, sink) * 1e-12;
    return r;
}

}  // namespace sfmba
