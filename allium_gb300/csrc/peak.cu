// FP64 multiply-add throughput probe: the denominator of the FP64 sweep's
// compute roofline, measured on the GPU the library runs on (the FP64 rate is
// the bound of the FP64 sweep on GB300, where it is 1/64 of the FP32 rate).
#include <cuda_runtime.h>

#include "../../include/allium_sweep.h"

namespace {

constexpr int kChains = 8;   // independent FMA chains per thread (hides the DFMA latency)

__global__ void k_dfma_probe(long long iters, double a, double b, double* sink) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1e-3;
    for (long long i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;   // keeps the chains alive
}

}  // namespace

extern "C" int allium_fp64_fma_probe(int blocks, int threads, long long iters, double* sink, void* stream) {
    if (blocks < 1 || threads < 32 || threads > 1024 || iters < 1 || !sink) return ALLIUM_ERR_ARG;
    // a = 1 - 2^-20, b small: the chains stay finite for any iteration count
    k_dfma_probe<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, 1.0 - 9.5367431640625e-7, 1e-6, sink);
    return cudaGetLastError() == cudaSuccess ? ALLIUM_OK : ALLIUM_ERR_CUDA;
}
