// FP64 right-hand side on the device.
//
// Viscoelastic ode (equation.jl:185-205) as two launches:
//   1. prologue, one thread per mantle cell / fault patch: update_strain_rate! (:207-222) writes
//      dϵ into du, relative_strain_rate! (:224-230) and relative_velocity! (:35-42) fill the
//      scratch vector x = [v - vpl; dϵ - dϵ₀];
//   2. one warp per receiver row: mantle rows compute dσ = [G12 | G22] x (:202-203) as a single
//      GEMV; fault rows compute the Toeplitz traction rate sum_{k,l} st[|i-k|, j, l] (v - vpl)[k,l]
//      (the FFT convolution of :44-61 applied directly) plus G21 (dϵ - dϵ₀) (:201), then the
//      friction epilogue update_fault! (:233-246) in the same warp.
// Fault-only ode (:156-166) is the second launch alone, with v - vpl formed on the fly.
// Each row's sum is reduced in a fixed order (lane partials, then a shuffle tree), so results
// are bitwise reproducible run to run.
#include <cuda_runtime.h>

#include "gbc_internal.cuh"
#include "rhs.cuh"

namespace gbc {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// sum_c A[c] * x[c] over c in [0, n) by one warp; A and x 16-byte aligned
__device__ __forceinline__ double warp_dot(const double* __restrict__ A, const double* __restrict__ x,
                                           long long n, int lane) {
    const double2* A2 = reinterpret_cast<const double2*>(A);
    const double2* x2 = reinterpret_cast<const double2*>(x);
    const long long n2 = n >> 1;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    long long c = lane;
    for (; c + 32 < n2; c += 64) {
        const double2 a0 = __ldcs(A2 + c), a1 = __ldcs(A2 + c + 32);
        const double2 x0 = __ldg(x2 + c), x1 = __ldg(x2 + c + 32);
        s0 = fma(a0.x, x0.x, s0);
        s1 = fma(a0.y, x0.y, s1);
        s2 = fma(a1.x, x1.x, s2);
        s3 = fma(a1.y, x1.y, s3);
    }
    for (; c < n2; c += 32) {
        const double2 a0 = __ldcs(A2 + c);
        const double2 x0 = __ldg(x2 + c);
        s0 = fma(a0.x, x0.x, s0);
        s1 = fma(a0.y, x0.y, s1);
    }
    if ((n & 1) && lane == 0) s0 = fma(__ldcs(A + n - 1), __ldg(x + n - 1), s0);
    return (s0 + s1) + (s2 + s3);
}

__global__ void k_prologue(RhsArgs a, const double* __restrict__ u, double* __restrict__ du,
                           StateLayout L) {
    if (a.skip && *a.skip) return;
    const int ne = a.ne, N = a.N;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N + ne; t += gridDim.x * blockDim.x) {
        if (t < N) {
            a.xm[t] = u[L.v + t] - a.vpl;
            continue;
        }
        const int i = t - N;
        double d[6];
        viscous_rates(a, u + L.sig, i, d);
        double* deps = du + L.eps;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            deps[i + k * ne] = d[k];
            a.xm[a.npad + i + k * ne] = d[k] - a.deps0[k];
        }
    }
}

__global__ void __launch_bounds__(256) k_rows(RhsArgs a, const double* __restrict__ u,
                                              double* __restrict__ du, StateLayout L) {
    if (a.skip && *a.skip) return;
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    const int N = a.N, nx = a.nx, nxi = a.nxi;
    const long long M = 6LL * a.ne;
    for (long long w = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); w < M + N; w += warps) {
        if (w < M) {  // mantle stress-rate row
            const double r = warp_sum(warp_dot(a.gm + w * a.ldm, a.xm, a.npad + M, lane));
            if (lane == 0) du[L.sig + w] = r;
            continue;
        }
        const int i = (int)(w - M), ii = i % nx, j = i / nx;
        // fault-fault traction rate: symmetric block-Toeplitz sum
        double acc = 0.0;
        const double* v = u + L.v;
        for (int l = 0; l < nxi; ++l) {
            const double* stl = a.st + (size_t)nx * (j + (size_t)nxi * l);
            const double* vl = v + (size_t)nx * l;
            for (int k = lane; k < nx; k += 32) {
                const int d = ii > k ? ii - k : k - ii;
                acc = fma(__ldg(stl + d), vl[k] - a.vpl, acc);
            }
        }
        if (M > 0) acc += warp_dot(a.g21 + (size_t)i * a.ld21, a.xm + a.npad, M, lane);
        const double dtau = warp_sum(acc);
        if (lane == 0 && a.dila) {
            // update_fault_with_dilatancy! (equation.jl:248-276) and d𝓅_dt (:282)
            const double vi = v[i], th = u[L.th + i], pi = u[L.p + i];
            const double Li = a.L[i];
            const double dth = 1.0 - vi * th / Li;
            const double dp = -(pi - a.p0[i]) / a.tp[i] + a.deps_d[i] / a.beta_d[i] / th * dth;
            const double af = a.a[i] / a.f0, bf = a.b[i] / a.f0;
            const double vf = fmax(0.0, vi / a.v0), thf = fmax(0.0, th * a.v0 / Li);
            const double vfa1 = pow(vf, af - 1.0), thfb1 = pow(thf, bf - 1.0);
            const double vfa = pow(vf, af), thfb = pow(thf, bf);
            du[L.th + i] = dth;
            du[L.p + i] = dp;
            du[L.v + i] = (dtau + a.f0 * dp * vfa * thfb - a.f0 * (a.sig[i] - pi) * vfa * thfb1 * bf * a.v0 / Li * dth) /
                          (a.f0 * (a.sig[i] - pi) * vfa1 * thfb * af / a.v0);
            du[L.delta + i] = vi;
        } else if (lane == 0) {
            fault_friction(a, u, du, L, i, dtau);
        }
    }
}

int rhs_kernel_count(const RhsArgs& a) {
    if (uses_mixed(a) && a.mode == GBC_PREC_DF64) return 2;
    if (uses_mixed(a)) return a.ne > 0 ? 3 : 1;
    return a.ne > 0 ? 2 : 1;
}

int launch_rhs(const RhsArgs& a, const double* u, double* du, cudaStream_t s) {
    if (uses_mixed(a)) return launch_rhs_mixed(a, u, du, s);
    const StateLayout L = layout_of(a.N, a.ne, a.dila);
    const int sms = sm_count();
    if (a.ne > 0) {
        const int n = a.N + a.ne;
        int g = (n + 255) / 256;
        if (g > sms * 8) g = sms * 8;
        k_prologue<<<g, 256, 0, s>>>(a, u, du, L);
        GBC_CUDA(cudaGetLastError());
    }
    const long long rows = 6LL * a.ne + a.N;
    long long g = (rows + 7) / 8;
    if (g > (long long)sms * 8) g = (long long)sms * 8;
    k_rows<<<(int)g, 256, 0, s>>>(a, u, du, L);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace gbc
