// Throughput probe of the FP64 FMA pipe: the denominator for kernels that the FP64 pipe, not HBM,
// bounds on this chip (the FP64 row GEMV and the FP64 Green's-function assembly). Each thread runs
// kChains independent dependent FMA chains (enough independent work to cover the pipe's latency)
// for iters iterations; the caller times the launch with CUDA events and divides the FLOPs
// (2 per FMA) by the time.
#include <cuda_runtime.h>

#include "gbc_internal.cuh"

namespace gbc {

constexpr int kChains = 8;

__global__ void k_probe_fp64_fma(double* __restrict__ out, long long iters, double b, double c) {
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (long long i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    out[blockIdx.x * (long long)blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace gbc

using namespace gbc;

extern "C" int gbc_probe_fp64_fma(double* out_dev, int blocks, int threads, long long iters, void* stream,
                                  double* flops) {
    if (!out_dev || blocks <= 0 || threads <= 0 || threads > 1024 || (threads & 31) || iters <= 0)
        return fail(GBC_EINVAL, "gbc_probe_fp64_fma: bad launch shape");
    // a = a*b + c with |b| < 1 stays bounded (fixed point c / (1 - b)), so no value overflows
    k_probe_fp64_fma<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(out_dev, iters, 0.999999, 1e-6);
    GBC_CUDA(cudaGetLastError());
    count_launches(1);
    if (flops) *flops = 2.0 * kChains * (double)iters * blocks * threads;
    return 0;
}
