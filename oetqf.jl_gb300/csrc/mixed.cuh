// Device pieces of the block-scaled 16-bit path shared by the single-model right-hand side
// (mixed.cu) and the shared-geometry sweep (sweep.cu): the 16-bit unpack and the shared-memory
// fault rows (FP32 Toeplitz sum + the G21 part + FP64 friction).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>

#include "rhs.cuh"

namespace gbc {

// eight 16-bit entries (one 16-byte load) to FP32
template <int MODE>
__device__ __forceinline__ void unpack8(const uint4 v, float (&f)[8]) {
    if (MODE == GBC_PREC_BF16) {
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            f[2 * i] = __uint_as_float(w[i] << 16);
            f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
        }
    } else {
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            __half2 h;
            memcpy(&h, &w[i], 4);
            const float2 t = __half22float2(h);
            f[2 * i] = t.x;
            f[2 * i + 1] = t.y;
        }
    }
}

// Fault rows through shared memory: one CTA per (16 along-strike patches ii0..ii0+15, depth row j),
// cta = j * ceil(nx / 16) + ii0 / 16, 256 threads, fsm = fault_rows_smem_bytes(N, nx, nxi) bytes of
// dynamic shared memory. The CTA stages x = v - vpl for the whole fault and the Toeplitz columns
// st32[:, j, l] for every source row l (2 N floats); thread (ii, t) sums over source rows
// l ≡ t (mod 16) and all k, the 16 partials of a patch are added in order t = 0..15, and the
// patch's FP64 friction follows with the G21 part a.y32[i] added when the model has a mantle.
constexpr int kFR_II = 16, kFR_L = 16;
__device__ __forceinline__ void fault_rows_cta(const RhsArgs& a, const double* __restrict__ u, double* __restrict__ du,
                                               const StateLayout& L, int cta, float* fsm) {
    const int nx = a.nx, nxi = a.nxi, N = a.N;
    float* xs = fsm;      // N: x[k + nx l]
    float* ts = fsm + N;  // nx * nxi: st32[d + nx (j + nxi l)] for this j, as ts[d + nx l]
    __shared__ float part[kFR_L][kFR_II + 1];
    const int nb = (nx + kFR_II - 1) / kFR_II;
    const int j = cta / nb, ii0 = (cta % nb) * kFR_II;
    for (int t = threadIdx.x; t < N; t += blockDim.x) xs[t] = (float)(u[L.v + t] - a.vpl);
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        const int d = t % nx, l = t / nx;
        ts[t] = a.st32[d + (size_t)nx * (j + (size_t)nxi * l)];
    }
    __syncthreads();
    const int il = threadIdx.x % kFR_II, tl = threadIdx.x / kFR_II;
    const int ii = ii0 + il;
    float acc = 0.f;
    if (ii < nx)
        for (int l = tl; l < nxi; l += kFR_L) {
            const float* x = xs + nx * l;
            const float* tt = ts + nx * l;
            float a0 = 0.f, a1 = 0.f;
            int k = 0;
            for (; k + 1 < nx; k += 2) {
                a0 = fmaf(tt[ii > k ? ii - k : k - ii], x[k], a0);
                a1 = fmaf(tt[ii > k + 1 ? ii - k - 1 : k + 1 - ii], x[k + 1], a1);
            }
            if (k < nx) a0 = fmaf(tt[ii > k ? ii - k : k - ii], x[k], a0);
            acc += a0 + a1;
        }
    part[tl][il] = acc;
    __syncthreads();
    if (tl == 0 && ii < nx) {
        float s = 0.f;
        for (int t = 0; t < kFR_L; ++t) s += part[t][il];
        const int i = ii + nx * j;
        fault_friction(a, u, du, L, i, (double)s + (a.ne > 0 ? (double)a.y32[i] : 0.0));
    }
}

size_t fault_rows_smem_bytes(int N, int nx, int nxi);

}  // namespace gbc
