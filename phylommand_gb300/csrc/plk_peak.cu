// plk_measure_fp32_peak: the FP32 multiply-add rate this GPU sustains, the
// denominator of the post-order passes' FP32 roofline (packed = 2: the FP64
// rate, the denominator of the FP64 plain form's).
//
// Every thread runs kChains independent multiply-add chains (enough to cover
// the pipe latency with a few warps per scheduler), either as scalar
// fma.rn.f32 or as packed fma.rn.f32x2 (two lanes per instruction), over a
// grid of a whole number of CTAs per SM.  Timed with CUDA events around one
// launch after a warm-up launch; flops = 2 per lane-FMA.  The chains converge
// to a fixed point (x <- x * b + c with 0 < b < 1), so no value overflows or
// turns subnormal, and the result is stored only under a condition the host
// never meets, which keeps the chains live without memory traffic.
#include <cuda_runtime.h>

#include "plk_internal.h"

namespace {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;
constexpr int kPeakCtasPerSm = 4;

typedef unsigned long long u64;

__device__ __forceinline__ u64 peak_fma2(u64 a, u64 b, u64 c) {
    u64 d;
    asm volatile("fma.rn.f32x2 %0, %1, %2, %3;\n" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

template <bool PACKED>
__global__ void __launch_bounds__(kPeakThreads) fp32_peak_kernel(int iters, float b, float c, float* sink, int flag) {
    if constexpr (PACKED) {
        u64 a[kChains];
        u64 bb, cc;
        asm("mov.b64 %0, {%1, %2};\n" : "=l"(bb) : "f"(b), "f"(b));
        asm("mov.b64 %0, {%1, %2};\n" : "=l"(cc) : "f"(c), "f"(c));
#pragma unroll
        for (int k = 0; k < kChains; ++k) {
            const float x = (float)(threadIdx.x + k);
            asm("mov.b64 %0, {%1, %2};\n" : "=l"(a[k]) : "f"(x), "f"(x + 0.5f));
        }
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int k = 0; k < kChains; ++k) a[k] = peak_fma2(a[k], bb, cc);
        }
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < kChains; ++k) {
            float lo, hi;
            asm("mov.b64 {%0, %1}, %2;\n" : "=f"(lo), "=f"(hi) : "l"(a[k]));
            s += lo + hi;
        }
        if (flag == 12345) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
    } else {
        float a[2 * kChains];
#pragma unroll
        for (int k = 0; k < 2 * kChains; ++k) a[k] = (float)(threadIdx.x + k);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int k = 0; k < 2 * kChains; ++k) a[k] = __fmaf_rn(a[k], b, c);
        }
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < 2 * kChains; ++k) s += a[k];
        if (flag == 12345) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
    }
}

// FP64 multiply-adds: 2 kChains independent fma.rn.f64 chains per thread,
// the lane-FMA count per iteration of the FP32 forms
__global__ void __launch_bounds__(kPeakThreads) fp64_peak_kernel(int iters, double b, double c, double* sink,
                                                                 int flag) {
    double a[2 * kChains];
#pragma unroll
    for (int k = 0; k < 2 * kChains; ++k) a[k] = (double)(threadIdx.x + k);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int k = 0; k < 2 * kChains; ++k) a[k] = __fma_rn(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 2 * kChains; ++k) s += a[k];
    if (flag == 12345) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" plk_status plk_measure_fp32_peak(int device, int packed, int iters, double* tflops_out, double* ms_out) {
    if (tflops_out == nullptr || iters < 1 || iters > (1 << 24) || packed < 0 || packed > 2)
        return plk::report_error(PLK_ERR_ARG, "plk_measure_fp32_peak: bad arguments");
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0)
        return plk::report_error(PLK_ERR_NODEV, "plk_measure_fp32_peak: no CUDA device");
    if (device < 0 || device >= n_dev) return plk::report_error(PLK_ERR_ARG, "plk_measure_fp32_peak: bad device");
    if (cudaSetDevice(device) != cudaSuccess) return plk::report_error(PLK_ERR_CUDA, "cudaSetDevice failed");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * kPeakCtasPerSm;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return plk::report_error(PLK_ERR_CUDA, "cudaStreamCreate failed");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto launch = [&](int n) {
        if (packed == 2) fp64_peak_kernel<<<blocks, kPeakThreads, 0, st>>>(n, 0.999, 1e-3, nullptr, 0);
        else if (packed) fp32_peak_kernel<true><<<blocks, kPeakThreads, 0, st>>>(n, 0.999f, 1e-3f, nullptr, 0);
        else fp32_peak_kernel<false><<<blocks, kPeakThreads, 0, st>>>(n, 0.999f, 1e-3f, nullptr, 0);
    };
    launch(iters / 8 + 1);  // warm-up
    cudaEventRecord(e0, st);
    launch(iters);
    cudaEventRecord(e1, st);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err == cudaSuccess) err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (err != cudaSuccess) return plk::report_error(PLK_ERR_CUDA, cudaGetErrorString(err));
    // lane-FMAs per thread per iteration: 4 rounds x kChains chains x 2 lanes
    // (packed) or 4 rounds x 2 kChains scalar chains: the same count
    const double fmas = (double)blocks * kPeakThreads * (double)iters * 4.0 * 2.0 * kChains;
    *tflops_out = 2.0 * fmas / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return PLK_OK;
}
