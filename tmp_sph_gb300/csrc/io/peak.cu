// peak.cu — the FP32 arithmetic peak of the GPU, measured: the denominator of the solver's
// FP32 roofline fraction (no reference counterpart; the reference records no peaks).
//
// One launch of blocks x 256 threads, each thread running `iters` rounds of eight independent
// FP32 fused multiply-adds (eight chains keep the FMA pipes busy between dependent issues),
// 2 flops each.  The chains' results are summed into `sink`, so nothing is dead code.  Timed
// by CUDA events on the given stream after one warm-up launch.
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_CHAINS = 8;

__global__ void __launch_bounds__(PEAK_THREADS) k_fma_peak(float* sink, int iters, float a,
                                                           float b) {
    float v[PEAK_CHAINS];
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) v[c] = (float)(threadIdx.x + c) * 1e-3f;
#pragma unroll 1
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int r = 0; r < 16; r++)
#pragma unroll
            for (int c = 0; c < PEAK_CHAINS; c++) v[c] = __fmaf_rn(v[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) s += v[c];
    sink[blockIdx.x * PEAK_THREADS + threadIdx.x] = s;
}

}  // namespace

extern "C" int sph_measure_fp32_peak(float* sink, int blocks, int iters, double* flops,
                                     double* ms, void* stream) {
    if (!sink || blocks < 1 || iters < 1 || !flops || !ms) return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return SPH_ERR_CUDA;
    }
    // a and b keep the chains bounded (|v| stays below b / (1 - a))
    k_fma_peak<<<blocks, PEAK_THREADS, 0, s>>>(sink, iters, 0.999f, 1e-3f);
    cudaEventRecord(e0, s);
    k_fma_peak<<<blocks, PEAK_THREADS, 0, s>>>(sink, iters, 0.999f, 1e-3f);
    cudaEventRecord(e1, s);
    float t = 0.f;
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return SPH_ERR_CUDA;
    *ms = t;
    *flops = 2.0 * 16.0 * PEAK_CHAINS * (double)iters * (double)PEAK_THREADS * (double)blocks;
    return SPH_OK;
}
