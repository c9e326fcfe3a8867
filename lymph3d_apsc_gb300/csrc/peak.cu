// peak.cu -- the FP64 FMA rate of the device, measured: the denominator of
// the plain FP64 step kernel's roofline (the step kernel is bound by the FP64
// pipe, which the copy-bandwidth and BF16 figures do not describe).

#include "common.cuh"

namespace {

// 8 independent FMA chains per thread in registers, `iters` rounds; the
// result is written only so that the chains are not removed.  The FMA's
// multiplier and addend are kernel arguments: with literal constants the
// probe measured 1.06 TFLOP/s on a GB300, with register operands 1.25 (the
// pipe's rate; the step kernel's FMAs take their operands from registers
// too).
__global__ void __launch_bounds__(256) k_fp64_fma(int iters, double seed, double b, double c, double* sink) {
    double a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = seed + threadIdx.x * 1e-9 + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fma(a[j], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == 12345.678) sink[blockIdx.x] = s;  // practically never true
}

}  // namespace

extern "C" {

// FP64 FMA throughput of device 0's current device in TFLOP/s (2 FLOP per
// FMA): one launch of 8 x SMs CTAs x 256 threads x 8 chains x `iters` FMAs,
// timed with CUDA events after a warm-up launch.
int lymph_fp64_peak(int32_t iters, double* tflops) {
    if (!tflops || iters < 1) return LYMPH_ERR_INVALID;
    int dev = 0, sms = 0;
    LYMPH_CUDA_TRY(cudaGetDevice(&dev));
    LYMPH_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* sink = nullptr;
    LYMPH_CUDA_TRY(cudaMalloc(&sink, sizeof(double) * 8 * (size_t)sms));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int grid = 8 * sms;
    k_fp64_fma<<<grid, 256>>>(iters / 4 + 1, 1.0, 0.999999, 1e-7, sink);
    cudaEventRecord(e0);
    k_fp64_fma<<<grid, 256>>>(iters, 1.0, 0.999999, 1e-7, sink);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) {
        lymph_set_error(std::string("lymph_fp64_peak: ") + cudaGetErrorString(e));
        return LYMPH_ERR_CUDA;
    }
    *tflops = 2.0 * 8.0 * 256.0 * grid * (double)iters / (ms * 1e-3) / 1e12;
    return LYMPH_OK;
}

}  // extern "C"
