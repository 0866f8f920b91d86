// Batched ensemble: many independent fault-only cycle models of uneven size integrated in one
// persistent launch per cluster size, one CTA or one 2/4/8-CTA thread-block cluster per model. Each
// model runs its own Tsit5 or VCABM5 steps with its own dt (per-instance step control). The
// traction rate is an rFFT convolution in shared memory accumulating in FP32 (the spectra of the
// circulant embedding of its Toeplitz kernel are precomputed per model); the state, stage sums,
// friction update and error norm are FP64. Cluster ranks own whole 32-patch chunks and exchange
// their slip rates and error-norm sums with st.async pushes into the peers' shared memory, so a
// model's trajectory does not depend on the block or cluster size; as models finish, the host
// moves the rest to larger clusters. A launch runs until its wall-clock budget and returns; the
// host relaunches a captured CUDA graph until every model is done.
//
// Reference: the fault-only ode (src/BEM/equation.jl:156-166) = relative_velocity! (:35-42),
// dτ_dt! (:44-61, the FFT convolution), update_fault! (:233-246) and the ageing law (:279); the
// integrators stand in for OrdinaryDiffEq's solve (src/io.jl:125-130).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <set>
#include <utility>
#include <cstring>
#include <string>
#include <vector>

#include "ensemble.cuh"
#include "gbc_internal.cuh"
#include "tma.cuh"

namespace gbc {

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__constant__ double e_ta[7][6] = {
    {0},
    {0.161},
    {-0.008480655492356989, 0.335480655492357},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
__constant__ double e_te[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                               -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                               0.015151515151515152};

// Shared-memory layout of one model CTA (floats): complex FFT work arrays Z (nq x P), real-input
// spectra X (nxi x H complex), twiddles (P/2 complex).
struct EnsSmem {
    float2* Z;
    float2* W;      // mixed row pairs of the CTA's patches, inverse-transformed in place (padded)
    float2* tw;
    double* pr;     // 2 x (nch + 1): error-norm sums of every 32-patch chunk + rank 0's stop flag
    double* cp;     // 3 x nch: VCABM5 error-norm sums of the CTA's chunks, one per component
    uint64_t* mb;   // mbarriers: received slip rates (buffers 0, 1), received norms (2, 3)
    float* xr;      // 2 x N: v - vpl of every patch (clusters: own slice + the peers' pushes)
    const float* G; // the model's real spectra: a shared-memory copy (EnsArgs::gsm) or global memory
};

// ---- cluster exchange: st.async pushes into the peers' shared memory, completing a transaction
// count on the peer's mbarrier (no cluster-wide release fence over the global stores) -------------
__device__ __forceinline__ unsigned peer_addr(const void* p, int rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ void push_f32(const float* dst, float v, const uint64_t* bar, int rank) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(peer_addr(dst, rank)),
                 "r"(__float_as_uint(v)), "r"(peer_addr(bar, rank))
                 : "memory");
}
__device__ __forceinline__ void push_f64(const double* dst, double v, const uint64_t* bar, int rank) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(peer_addr(dst, rank)),
                 "l"(__double_as_longlong(v)), "r"(peer_addr(bar, rank))
                 : "memory");
}
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, unsigned parity) {
    for (long long i = 0; i < kWaitLimit; ++i) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// 1/x by Newton-Raphson (r <- r + r (1 - x r), the relative error squaring each step) from the
// FP64 reciprocal by Newton-Raphson from the correctly rounded FP32 reciprocal of x rounded to FP32
// (error < 2^-23): two steps leave ~2^-90 plus FP64 rounding, about 1 ulp -- four dependent FMAs
// where an FP64 division is a long chain of dependent FP64 instructions at 64 cycles each on this
// chip. For arguments in FP32's normal range: step sizes, error-norm scales, the state θ (between
// about 1e-3 and 1e12 s over a cycle) and friction denominators (at least the radiation damping
// η). Below that range the seed overflows and the result is not finite (the step control rejects
// the stage); above it the result is zero.
__device__ __forceinline__ double ens_rcp_in_range(double x) {
    double r = (double)__frcp_rn(__double2float_rn(x));
    r = fma(r, fma(-x, r, 1.0), r);
    return fma(r, fma(-x, r, 1.0), r);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

__device__ __forceinline__ float2 bfly_add(float2 a, float2 c) { return make_float2(a.x + c.x, a.y + c.y); }
__device__ __forceinline__ float2 bfly_sub(float2 a, float2 c) { return make_float2(a.x - c.x, a.y - c.y); }
// Shared-memory FFT buffers (work arrays and twiddles) hold element i at i + i / 8: one float2 of
// padding per eight. The strided accesses of the radix-8 passes (stride 8 in the first) and the
// bit-reversed scatters then spread over the 32 banks instead of landing on two.
__device__ __forceinline__ int zp(int i) { return i + (i >> 3); }
__host__ __device__ __forceinline__ size_t zlen(size_t n) { return n + (n >> 3) + 1; }

__device__ __forceinline__ float2 tw_get(const float2* tw, int idx, int inverse) {
    float2 w = tw[zp(idx)];
    if (inverse) w.y = -w.y;
    return w;
}

// in-place radix-2 DIT FFT of arrays q0 .. q0 + nq - 1 (length P = 2^logP, padded as above) of the
// buffer Z, already in bit-reversed order; forward uses twiddles e^{-2πi t/P}, inverse their
// conjugates (no scaling). Up to three
// consecutive radix-2 stages are done per pass with a thread's eight elements in registers (the
// same butterflies in the same order as one stage per pass), so a 512-point transform takes three
// passes and barriers; indices come from shifts (P is a power of two).
// three consecutive radix-2 stages st, st+1, st+2 on a thread's eight elements (stride h, offset
// pos within the group)
__device__ __forceinline__ void radix8(float2 (&x)[8], const float2* tw, int st, int pos, int h, int P, int inverse) {
    const float2 w1 = tw_get(tw, pos * (P >> (st + 1)), inverse);
#pragma unroll
    for (int m = 0; m < 8; m += 2) {  // stage st: pairs (m, m+1)
        const float2 c = cmul(x[m + 1], w1);
        x[m + 1] = bfly_sub(x[m], c);
        x[m] = bfly_add(x[m], c);
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) {     // stage st+1: pairs (m, m+2) in groups of four
        if (m & 2) continue;
        const float2 w = tw_get(tw, (pos + (m & 1) * h) * (P >> (st + 2)), inverse);
        const float2 c = cmul(x[m + 2], w);
        x[m + 2] = bfly_sub(x[m], c);
        x[m] = bfly_add(x[m], c);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {     // stage st+2: pairs (m, m+4)
        const float2 w = tw_get(tw, (pos + m * h) * (P >> (st + 3)), inverse);
        const float2 c = cmul(x[m + 4], w);
        x[m + 4] = bfly_sub(x[m], c);
        x[m] = bfly_add(x[m], c);
    }
}

template <int BS>
__device__ __forceinline__ void fft_many(float2* Z, int q0, int nq, int P, int logP, const float2* tw, int inverse,
                                         int st0 = 0) {
    int st = st0;  // stages before st0 already done
    while (st < logP) {
        const int ns = min(3, logP - st);       // stages in this pass
        const int h = 1 << st;
        const int lgi = logP - ns;              // log2 of the butterfly groups per array
        const int items = nq << lgi;
        for (int t = threadIdx.x; t < items; t += BS) {
            const int q = t >> lgi, r = t & ((1 << lgi) - 1);
            const int g = r >> st, pos = r & (h - 1);
            const int zb = (q0 + q) * P;  // arrays q0.. of the padded buffer
            if (ns == 3) {
                const int b0 = g * 8 * h + pos;
                float2 x[8];
#pragma unroll
                for (int m = 0; m < 8; ++m) x[m] = Z[zp(zb + b0 + m * h)];
                radix8(x, tw, st, pos, h, P, inverse);
#pragma unroll
                for (int m = 0; m < 8; ++m) Z[zp(zb + b0 + m * h)] = x[m];
            } else if (ns == 2) {
                const int b0 = g * 4 * h + pos;
                const float2 w1 = tw_get(tw, pos * (P >> (st + 1)), inverse);
                const float2 w2a = tw_get(tw, pos * (P >> (st + 2)), inverse);
                const float2 w2b = tw_get(tw, (pos + h) * (P >> (st + 2)), inverse);
                const float2 x0 = Z[zp(zb + b0)], x1 = Z[zp(zb + b0 + h)], x2 = Z[zp(zb + b0 + 2 * h)], x3 = Z[zp(zb + b0 + 3 * h)];
                float2 c = cmul(x1, w1);
                const float2 y0 = bfly_add(x0, c), y1 = bfly_sub(x0, c);
                c = cmul(x3, w1);
                const float2 y2 = bfly_add(x2, c), y3 = bfly_sub(x2, c);
                c = cmul(y2, w2a);
                Z[zp(zb + b0)] = bfly_add(y0, c);
                Z[zp(zb + b0 + 2 * h)] = bfly_sub(y0, c);
                c = cmul(y3, w2b);
                Z[zp(zb + b0 + h)] = bfly_add(y1, c);
                Z[zp(zb + b0 + 3 * h)] = bfly_sub(y1, c);
            } else {
                const int i0 = (g << (st + 1)) + pos, i1 = i0 + h;
                const float2 w = tw_get(tw, pos * (P >> (st + 1)), inverse);
                const float2 a = Z[zp(zb + i0)], c = cmul(Z[zp(zb + i1)], w);
                Z[zp(zb + i0)] = bfly_add(a, c);
                Z[zp(zb + i1)] = bfly_sub(a, c);
            }
        }
        st += ns;
        __syncthreads();
    }
}

// The forward transform's first pass (stages 0-2, P >= 8) read straight from the slip rates: element
// p of row pair q holds v - vpl at patch brev(p) of rows 2q (real part) and 2q + 1 (imaginary part),
// zero beyond nx, so packing the rows in bit-reversed order and the pass's loads are one step (the
// same values through the same butterflies). xin: v - vpl of every patch in shared memory, or null
// to read the stage state.
template <int BS>
__device__ __forceinline__ void fft_first_from_rows(float2* Z, int nq, int P, int logP, const float2* tw,
                                                    const float* xin, const double* __restrict__ v, double vpl,
                                                    int nx, int nxi) {
    const int lgi = logP - 3, items = nq << lgi;
    for (int t = threadIdx.x; t < items; t += BS) {
        const int q = t >> lgi, b0 = (t & ((1 << lgi) - 1)) * 8;
        const int r0 = nx * (2 * q), r1 = nx * (2 * q + 1);
        const bool odd = 2 * q + 1 < nxi;
        float2 x[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int i = __brev(b0 + m) >> (32 - logP);
            float re = 0.f, im = 0.f;
            if (i < nx) {
                if (xin) {
                    re = xin[i + r0];
                    if (odd) im = xin[i + r1];
                } else {
                    re = (float)(v[i + r0] - vpl);
                    if (odd) im = (float)(v[i + r1] - vpl);
                }
            }
            x[m] = make_float2(re, im);
        }
        radix8(x, tw, 0, 0, 1, P, 0);
#pragma unroll
        for (int m = 0; m < 8; ++m) Z[zp(q * P + b0 + m)] = x[m];
    }
    __syncthreads();
}

// fault-only RHS of one model: y (v, θ-or-ψ, δ) -> k. The traction rate is the rFFT convolution
// of the reference (equation.jl:44-61) done in shared memory: two real rows per complex FFT,
// a real per-frequency mixing (the symmetric circulant kernel has a real spectrum), two output
// rows per inverse FFT.
// xin: v - vpl of every patch in shared memory (cluster ranks, after the exchange), or null to
// read the stage state y itself (one-CTA models).
template <int BS>
__device__ __forceinline__ void ens_rhs(const EnsModel& m, const EnsArgs& A, const EnsSmem& S,
                                        const double* __restrict__ y, double* __restrict__ k, int lo, int hi,
                                        const float* xin) {
    __syncthreads();
    const int N = m.N, nx = m.nx, nxi = m.nxi, P = m.P, logP = m.logP, H = P / 2 + 1;
    const int nq = (nxi + 1) / 2;
    const double* v = y;
    const double* th = y + N;
    if (logP >= 3) {
        fft_first_from_rows<BS>(S.Z, nq, P, logP, S.tw, xin, v, m.vpl, nx, nxi);
        fft_many<BS>(S.Z, 0, nq, P, logP, S.tw, 0, 3);
    } else {
        // (P < 8) pack rows (2q, 2q+1) as real/imag, zero padded, in bit-reversed order
        for (int t = threadIdx.x; t < nq * P; t += BS) {
            const int q = t >> logP, i = t & (P - 1);
            float re = 0.f, im = 0.f;
            if (i < nx) {
                if (xin) {
                    re = xin[i + nx * (2 * q)];
                    if (2 * q + 1 < nxi) im = xin[i + nx * (2 * q + 1)];
                } else {
                    re = (float)(v[i + nx * (2 * q)] - m.vpl);
                    if (2 * q + 1 < nxi) im = (float)(v[i + nx * (2 * q + 1)] - m.vpl);
                }
            }
            S.Z[zp(q * P + (__brev(i) >> (32 - logP)))] = make_float2(re, im);
        }
        __syncthreads();
        fft_many<BS>(S.Z, 0, nq, P, logP, S.tw, 0);
    }
    // Y_j[f] = sum_l G[j,l,f] X_l[f] (G real), the row spectra X taken straight from the transformed
    // pairs: X_{2q}[f] = (Z_q[f] + conj Z_q[P-f]) / 2, X_{2q+1}[f] = (Z_q[f] - conj Z_q[P-f]) / 2i.
    // Y is repacked (2q, 2q+1) as Y_2q + i Y_2q+1 with Hermitian fill, bit-reversed, into W for the
    // inverse transform (every thread still reads Z). Only the row pairs holding this CTA's patches
    // [lo, hi) are mixed and transformed back (a cluster rank's slice spans one or two depth rows):
    // the forward spectra of every row are needed, the traction rates of the other rows are not.
    const float* G = S.G;
    const int qlo = (hi > lo) ? (lo / nx) >> 1 : 0;
    const int nqr = (hi > lo) ? (((hi - 1) / nx) >> 1) - qlo + 1 : 0;
    for (int t = threadIdx.x; t < nqr * H; t += BS) {
        const int q = qlo + t / H, f = t - (q - qlo) * H, fm = (P - f) & (P - 1);
        const int j0 = 2 * q, j1 = 2 * q + 1;
        float2 y0 = make_float2(0.f, 0.f), y1 = make_float2(0.f, 0.f);
        for (int qi = 0; qi < nq; ++qi) {
            const float2 a = S.Z[zp(qi * P + f)], b = S.Z[zp(qi * P + fm)];
#pragma unroll
            for (int s2 = 0; s2 < 2; ++s2) {
                const int l = 2 * qi + s2;
                if (l >= nxi) break;
                const float2 x = s2 ? make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x))
                                    : make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
                // generic loads: G is global memory or a shared-memory copy (a read-only-path load
                // would accept only global addresses)
                const float g0 = G[((size_t)(j0 * nxi + l)) * H + f];
                y0.x = fmaf(g0, x.x, y0.x);
                y0.y = fmaf(g0, x.y, y0.y);
                if (j1 < nxi) {
                    const float g1 = G[((size_t)(j1 * nxi + l)) * H + f];
                    y1.x = fmaf(g1, x.x, y1.x);
                    y1.y = fmaf(g1, x.y, y1.y);
                }
            }
        }
        // W[f] = Y0[f] + i Y1[f]; W[P-f] = conj(Y0[f]) + i conj(Y1[f])
        const int wb = (q - qlo) * P;
        S.W[zp(wb + (__brev(f) >> (32 - logP)))] = make_float2(y0.x - y1.y, y0.y + y1.x);
        if (f > 0 && f < P - f) S.W[zp(wb + (__brev(P - f) >> (32 - logP)))] = make_float2(y0.x + y1.y, -y0.y + y1.x);
    }
    __syncthreads();
    fft_many<BS>(S.W, 0, nqr, P, logP, S.tw, 1);
    const double invP = 1.0 / P;
    const double* pa = m.a;
    const double* pb = m.b;
    const double* pL = m.L;
    const double* ps = m.sig;
    const double* pc = m.c1;
    for (int i = lo + threadIdx.x; i < hi; i += BS) {
        const int ii = i % nx, j = i / nx;
        const float2 w = S.W[zp(((j >> 1) - qlo) * P + ii)];
        const double dtau = (double)((j & 1) ? w.y : w.x) * invP;
        const double vi = v[i];
        const double ai = pa[i], bi = pb[i], Li = pL[i];
        // ψ1 = exp((f0 + b ln(v0 θ / L)) / a) / (2 v0) = exp(c1 + (b/a) ln θ) and ψ2 = σ ψ1 / hypot(1, v ψ1)
        // = σ / sqrt(v² + ψ1⁻²). ψ1⁻¹ is tiny against the slip rate (ψ1 grows with θ as v falls; along
        // the FP64 oracle trajectory of the most eventful model of the 8-year ensemble, every 50th of
        // 315,835 steps, all patches: ψ1⁻¹ <= 8.2e-15 m/s, ψ1⁻¹ / |v| <= 5.5e-10), so it enters ψ2 only
        // as a correction of relative size ψ1⁻² / v²; computed with FP32 exp and log it moves ψ2 by far
        // less than FP64 rounding, and its ~40 FP64 instructions (a warp issues one per 64 cycles)
        // become FP32 ones. The rest of the friction is FP64; the per-patch constants replace three
        // serial divisions.
        if (m.log_theta) {
            // ψ = ln θ: 1/θ = exp(-ψ) (FP64: the ageing law's 1/θ - v/L cancels near steady state);
            // dψ = 1/θ - v/L; dμ/dθ dθ = b v ψ2 dψ
            const double psi = th[i];
            const double ei = (double)expf(-fmaf(__double2float_rn(m.boa[i]), __double2float_rn(psi), __double2float_rn(pc[i])));
            const double psi2 = ps[i] * rsqrt(fma(vi, vi, ei * ei));
            const double dpsi = fma(-vi, m.iL[i], exp(-psi));
            k[i] = fma(-bi * vi * psi2, dpsi, dtau) / fma(ai, psi2, m.eta);
            k[N + i] = dpsi;
        } else {
            const double tht = th[i];
            (void)Li;
            const float lt = logf(fmaxf(0.f, __double2float_rn(tht)));  // θ <= 0: ψ1 = 0, ψ2 = 0
            const double ei = (double)expf(-fmaf(__double2float_rn(m.boa[i]), lt, __double2float_rn(pc[i])));
            const double psi2 = ps[i] * rsqrt(fma(vi, vi, ei * ei));
            const double dth = fma(-vi * tht, m.iL[i], 1.0);
            k[i] = fma(-bi * vi * psi2, dth * ens_rcp_in_range(tht), dtau) * ens_rcp_in_range(fma(ai, psi2, m.eta));
            k[N + i] = dth;
        }
        k[2 * N + i] = vi;
    }
    __syncthreads();
}

namespace cg = cooperative_groups;

// per-CTA copy of the model's step control; every CTA of a cluster computes it identically and
// cluster rank 0 writes it back to the descriptor
struct EnsCtl {
    double t, dt, t1, qold;
    long long naccept, nreject, iters, maxiters;
    int done, status, go, stop;
    // VCABM5: order, order of the step in flight, consecutive rejections, psi of the last accepted
    // step, and this step's psi, beta and Adams weights (the oracle's orc_abm_coefficients)
    int k, kq, fails;
    double psi_prev[5], psi[6], beta[6], g[7];
    double rat[9];  // h / psi_j (j = 0..4) and psi_{i-1} / psi_prev_{i-1} (i = 1..4), one warp each
};

// this step's ψ, β and Adams weights (the oracle's orc_abm_coefficients, same operations), in two
// parts. A warp issues about one FP64 instruction per 64 cycles however few lanes are active, so
// the nine independent ratios (h / ψ_j and ψ_{i-1} / ψ_prev_{i-1}, a Newton reciprocal and a
// product each) go to nine warps (lane 0 of warp w computes ratio w); one thread then forms the
// β products and the weights from them.
__device__ __forceinline__ double ens_abm_psi(const EnsCtl& c, double h, int j) {
    return (j == 0) ? h : (j < c.k ? h + c.psi_prev[j - 1] : 1.0);
}

__device__ __forceinline__ void ens_abm_ratio(EnsCtl& c, double h, int w) {
    if (w < 5) {
        c.rat[w] = h * ens_rcp_in_range(ens_abm_psi(c, h, w));
    } else {
        const int i = w - 4;  // 1..4
        c.rat[w] = (i < c.k) ? ens_abm_psi(c, h, i - 1) * ens_rcp_in_range(c.psi_prev[i - 1]) : 0.0;
    }
}

__device__ __forceinline__ void ens_abm_coef(EnsCtl& c, double h) {
    const int k = c.k;
    c.kq = k;
    double psi[5], beta[5], r[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        psi[i] = ens_abm_psi(c, h, i);
        r[i] = c.rat[i];
    }
    beta[0] = 1.0;
#pragma unroll
    for (int i = 1; i < 5; ++i) beta[i] = (i < k) ? beta[i - 1] * c.rat[4 + i] : 0.0;
    double cq[8] = {0.0, 1.0, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 0.0};
#pragma unroll
    for (int q = 1; q <= 6; ++q)
        if (q > k + 1) cq[q] = 0.0;
    double g[6];
    g[0] = cq[1];
#pragma unroll
    for (int j = 1; j <= 5; ++j) {
        if (j <= k) {
#pragma unroll
            for (int q = 1; q <= 5; ++q)
                if (q <= k + 1 - j) cq[q] = cq[q] - cq[q + 1] * r[j - 1];
        }
        g[j] = cq[1];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        c.psi[i] = psi[i];
        c.beta[i] = beta[i];
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) c.g[j] = g[j];
}

// ALG 0: Tsit5 (6 RHS per step); ALG 1: VCABM5 (PECE: 1 RHS per step + 1 per accepted step;
// the modified divided differences Phi_0..Phi_5 live in the stage buffers k[0..5], k[6] holds f at
// the predicted and then at the corrected point)
template <int BS, int ALG>
__global__ void __launch_bounds__(BS, 512 / BS) k_ensemble(EnsArgs A) {  // 128 registers a thread at any block size
    extern __shared__ __align__(16) float sm[];
    __shared__ double red[BS / 32];
    __shared__ EnsCtl c;
    cg::cluster_group cl = cg::this_cluster();
    const int csize = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const unsigned long long t_launch = global_ns();
    const int slot = A.first + (int)(blockIdx.x / csize);
    const int mi = A.order ? A.order[slot] : slot;
    EnsModel& M = A.models[mi];
    const EnsModel m = M;  // sizes, constants and the step control state at launch
    if (m.done) return;    // the same descriptor for every rank: cluster-uniform
    const int N = m.N;
    // each rank owns whole 32-patch chunks, so the error norm below sums the same chunks in the
    // same order whatever the cluster and block sizes: a model's trajectory does not depend on them
    const int nch = (N + 31) / 32;
    const double inv3n = 1.0 / (double)(3 * N);  // the RMS error norm's 1/n, once per launch
    const int lo = 32 * (int)((long long)nch * rank / csize);
    const int hi = min(N, 32 * (int)((long long)nch * (rank + 1) / csize));
    const int nq = (m.nxi + 1) / 2;
    const int c0 = (int)((long long)nch * rank / csize), c1 = (int)((long long)nch * (rank + 1) / csize);
    const bool clus = csize > 1;
    EnsSmem S;
    S.Z = reinterpret_cast<float2*>(sm);
    S.W = S.Z + zlen((size_t)nq * m.P);
    S.tw = S.W + zlen((size_t)nq * m.P);
    S.pr = reinterpret_cast<double*>(S.tw + zlen((size_t)m.P / 2));
    S.cp = S.pr + 2 * (nch + 1);
    S.mb = reinterpret_cast<uint64_t*>(S.cp + 3 * nch);
    S.xr = reinterpret_cast<float*>(S.mb + 4);
    S.G = m.ghat;
    if (A.gsm) {  // the spectra read every RHS: one copy per launch into shared memory
        const size_t off = (reinterpret_cast<uintptr_t>(S.xr + 2 * (size_t)N) + 15) & ~(uintptr_t)15;
        float* gs = reinterpret_cast<float*>(off);
        const int ng = m.nxi * m.nxi * (m.P / 2 + 1);
        for (int t = threadIdx.x; t < ng; t += BS) gs[t] = m.ghat[t];
        S.G = gs;  // visible to every thread after the barrier below
    }
    for (int t = threadIdx.x; t < m.P / 2; t += BS) {
        double sn, cs;
        sincospi(2.0 * t / m.P, &sn, &cs);
        S.tw[zp(t)] = make_float2((float)cs, (float)-sn);
    }
    __shared__ int xfail;  // a bounded exchange wait gave up
    if (threadIdx.x == 0) {
        c.t = m.t; c.dt = m.dt; c.t1 = m.t1; c.qold = m.qold;
        c.naccept = m.naccept; c.nreject = m.nreject; c.iters = m.iters; c.maxiters = m.maxiters;
        c.done = m.done; c.status = m.status; c.go = 0; c.stop = 0;
        c.k = m.abm_k > 0 ? m.abm_k : 1;
        c.kq = c.k;
        c.fails = m.abm_fails;
        for (int i = 0; i < 5; ++i) c.psi_prev[i] = m.psi_prev[i];
        xfail = 0;
        if (clus) {
            for (int b = 0; b < 4; ++b) mbar_init(&S.mb[b], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    if (clus) cl.sync();  // every peer's barriers exist before the first push
    else __syncthreads();
    double* u = m.u;
    double* kk[7];
    for (int s = 0; s < 7; ++s) kk[s] = m.k[s];
    double* y = m.y;
    double* un = m.un;
    const bool writer = (rank == 0 && threadIdx.x == 0);
    // thread 0's parity of the current phase of each exchange barrier (bit b; a phase per use)
    unsigned phase = 0;
    auto collect = [&](int b, unsigned bytes) {
        if (threadIdx.x == 0) {
            mbar_expect_tx(&S.mb[b], bytes);  // the peers' bytes of this phase (some may be in already)
            if (!mbar_wait_cluster(&S.mb[b], (phase >> b) & 1u)) xfail = 1;
            phase ^= 1u << b;
        }
        __syncthreads();
    };
    const unsigned xbytes = 4u * (unsigned)(N - (hi - lo));
    int rx = 0;  // RHS evaluations in this launch: slip-rate buffer rx & 1
    if (!m.started) {  // FSAL seed
        const float* xin = nullptr;
        if (clus) {
            float* xb = S.xr + (size_t)(rx & 1) * N;
            for (int i = lo + threadIdx.x; i < hi; i += BS) {
                const float x = (float)(u[i] - m.vpl);
                xb[i] = x;
                for (int d = 1; d < csize; ++d) push_f32(xb + i, x, &S.mb[rx & 1], (rank + d) % csize);
            }
            collect(rx & 1, xbytes);
            xin = xb;
        }
        if (!xfail) ens_rhs<BS>(m, A, S, u, kk[0], lo, hi, xin);
        ++rx;
        if (writer) M.started = 1;
    }
    for (int step = 0; step < A.budget && !xfail; ++step) {
        if (c.stop) break;  // decided by the last step's controller, identically in every rank
        const double dt = c.dt;
        const int e = step & 1;
        double* prb = S.pr + (size_t)e * (nch + 1);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (ALG == 0) {
            for (int s = 1; s < 7; ++s) {
                double* dst = (s == 6) ? un : y;
                float* xb = S.xr + (size_t)(rx & 1) * N;
                // the three components' FMA chains interleaved (FP64 latency, not throughput, binds here);
                // cluster ranks publish v - vpl of their slice to every peer as they go
                for (int i = lo + threadIdx.x; i < hi; i += BS) {
                    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
                    for (int r = 0; r < s; ++r) {
                        const double a = e_ta[s][r];
                        acc0 = fma(a, kk[r][i], acc0);
                        acc1 = fma(a, kk[r][N + i], acc1);
                        acc2 = fma(a, kk[r][2 * N + i], acc2);
                    }
                    const double vnew = u[i] + dt * acc0;
                    dst[i] = vnew;
                    dst[N + i] = u[N + i] + dt * acc1;
                    dst[2 * N + i] = u[2 * N + i] + dt * acc2;
                    if (clus) {
                        const float x = (float)(vnew - m.vpl);
                        xb[i] = x;
                        for (int d = 1; d < csize; ++d) push_f32(xb + i, x, &S.mb[rx & 1], (rank + d) % csize);
                    }
                }
                if (clus) {
                    collect(rx & 1, xbytes);
                    if (xfail) break;
                }
                ens_rhs<BS>(m, A, S, dst, kk[s], lo, hi, clus ? xb : nullptr);
                ++rx;
            }
            if (xfail) break;
            // error norm: per 32-patch chunk, lane i sums r^2 over the three components, then a fixed
            // shuffle tree; the chunk sums (pushed to every rank) are added in chunk order, identically
            // in every rank, together with rank 0's wall-clock stop flag
            for (int ch = c0 + warp; ch < c1; ch += BS / 32) {
                const int i = 32 * ch + lane;
                double ss = 0.0;
                int bad = 0;
                if (i < N) {
                    double ev[3], r[3];
    #pragma unroll
                    for (int comp = 0; comp < 3; ++comp) ev[comp] = 0.0;
    #pragma unroll
                    for (int s = 0; s < 7; ++s)
    #pragma unroll
                        for (int comp = 0; comp < 3; ++comp) ev[comp] = fma(e_te[s], kk[s][comp * N + i], ev[comp]);
    #pragma unroll
                    for (int comp = 0; comp < 3; ++comp) {
                        const int g = comp * N + i;
                        const double unv = un[g];
                        // ψ = ln θ: an absolute ψ error is a relative θ error, scaled by reltol
                        const double sc = (comp == 1 && m.log_theta) ? A.abstol + A.reltol
                                                                     : A.abstol + A.reltol * fmax(fabs(u[g]), fabs(unv));
                        r[comp] = (ev[comp] * dt) / sc;
                        bad |= !isfinite(unv);
                    }
                    ss = fma(r[0], r[0], ss);  // components summed in order 0, 1, 2
                    ss = fma(r[1], r[1], ss);
                    ss = fma(r[2], r[2], ss);
                }
                for (int o = 16; o > 0; o >>= 1) {
                    ss += __shfl_xor_sync(0xffffffffu, ss, o);
                    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
                }
                if (lane == 0) {
                    const double val = bad ? INFINITY : ss;
                    prb[ch] = val;
                    for (int d = 1; d < csize; ++d) push_f64(prb + ch, val, &S.mb[2 + e], (rank + d) % csize);
                }
            }
        } else {
            // VCABM5 step: coefficients, predictor (publishing v), f at the predicted point, corrector
            // with the error chunks; f at the corrected point and the Phi update after acceptance
            // every thread is done with the last step's beta (its Phi update) before thread 0 rewrites it
            __syncthreads();
            if (lane == 0)
                for (int w = warp; w < 9; w += BS / 32) ens_abm_ratio(c, dt, w);
            __syncthreads();
            if (threadIdx.x == 0) ens_abm_coef(c, dt);
            __syncthreads();
            const int kq = c.kq;
            {
                float* xb = S.xr + (size_t)(rx & 1) * N;
                // one (component, patch) per thread: a CTA's slice of a split model is a few hundred
                // elements, so its threads take the three components side by side instead of in turn
                const int nl = hi - lo;
                for (int t = threadIdx.x; t < 3 * nl; t += BS) {
                    const int comp = (t >= nl) + (t >= 2 * nl);
                    const int i = lo + t - comp * nl, g = comp * N + i;
                    double acc = 0.0;
                    // compile-time bounds: the stage pointers stay in registers and every load of
                    // the differences issues before the first FMA needs one (same sums, same order)
#pragma unroll
                    for (int j = 0; j < 5; ++j)
                        if (j < kq) acc = fma(c.g[j], c.beta[j] * kk[j][g], acc);
                    const double yv = u[g] + dt * acc;
                    y[g] = yv;
                    if (clus && comp == 0) {
                        const float x = (float)(yv - m.vpl);
                        xb[i] = x;
                        for (int d = 1; d < csize; ++d) push_f32(xb + i, x, &S.mb[rx & 1], (rank + d) % csize);
                    }
                }
                if (clus) {
                    collect(rx & 1, xbytes);
                    if (xfail) break;
                }
                ens_rhs<BS>(m, A, S, y, kk[6], lo, hi, clus ? xb : nullptr);
                ++rx;
            }
            // corrector and error estimate, one warp per (chunk, component): each warp sums its 32
            // patches' r^2 in a fixed shuffle order, and a chunk's norm is (s_v + s_θ) + s_δ, so a
            // model's trajectory still does not depend on the block or cluster size
            const double gk = c.g[kq], ce = dt * (c.g[kq] - c.g[kq - 1]);
            const int ncp = 3 * (c1 - c0);
            for (int wi = warp; wi < ncp; wi += BS / 32) {
                const int q = wi / 3, comp = wi - 3 * q;
                const int i = 32 * (c0 + q) + lane;
                double ss = 0.0;
                int bad = 0;
                if (i < N) {
                    const int g = comp * N + i;
                    double sacc = 0.0;
#pragma unroll
                    for (int j = 0; j < 5; ++j)
                        if (j < kq) sacc += c.beta[j] * kk[j][g];
                    const double pk = kk[6][g] - sacc;
                    const double yn = y[g] + dt * gk * pk;
                    un[g] = yn;
                    const double sc = (comp == 1 && m.log_theta) ? A.abstol + A.reltol
                                                                 : A.abstol + A.reltol * fmax(fabs(u[g]), fabs(yn));
                    const double r = (ce * pk) * ens_rcp_in_range(sc);
                    bad = !isfinite(yn);
                    ss = r * r;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    ss += __shfl_xor_sync(0xffffffffu, ss, o);
                    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
                }
                if (lane == 0) S.cp[wi] = bad ? INFINITY : ss;
            }
            __syncthreads();
            for (int q = threadIdx.x; q < c1 - c0; q += BS) {
                const int ch = c0 + q;
                const double val = (S.cp[3 * q] + S.cp[3 * q + 1]) + S.cp[3 * q + 2];
                prb[ch] = val;
                for (int d = 1; d < csize; ++d) push_f64(prb + ch, val, &S.mb[2 + e], (rank + d) % csize);
            }
        }
        if (writer) {
            const double f = (global_ns() - t_launch > A.budget_ns) ? 1.0 : 0.0;
            prb[nch] = f;
            for (int d = 1; d < csize; ++d) push_f64(prb + nch, f, &S.mb[2 + e], d);
        }
        if (clus) {
            collect(2 + e, 8u * (unsigned)(nch - (c1 - c0)) + (rank != 0 ? 8u : 0u));
            if (xfail) break;
        } else {
            __syncthreads();
        }
        if (warp == 0) {
            double tot = 0.0;
            for (int ch = lane; ch < nch; ch += 32) tot += prb[ch];
            for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
            red[0] = tot;  // lane 0 below
        }
        if (threadIdx.x == 0 && ALG == 1) {
            const double tot = red[0];
            // the squared RMS norm decides acceptance (sqrt is monotonic and sqrt(1) = 1, so
            // EEst <= 1 exactly when EEst^2 <= 1); the step factor needs only FP32
            double EEst = tot * inv3n;
            if (!isfinite(EEst)) EEst = INFINITY;
            const int kq = c.kq;
            // step factor 0.8 EEst^(-1/(k+1)) within [0.2, 2] (at most 0.8 after a rejection), in FP32
            // like the PI gains; acceptance compares the FP64 norm
            const double fac = 0.8 * (double)exp2f(-0.5f * log2f((float)EEst) / (float)(kq + 1));
            c.iters += 1;
            double dtn;
            int acc = 0;
            if (EEst <= 1.0) {
                const double tn = c.t + dt;
                c.t = (tn >= c.t1) ? c.t1 : tn;
                c.naccept += 1;
                acc = 1;
                for (int i = 0; i < kq; ++i) c.psi_prev[i] = c.psi[i];
                if (c.k < 5) c.k += 1;
                c.fails = 0;
                dtn = dt * fmin(2.0, fmax(0.2, fac));
            } else {
                c.nreject += 1;
                if (++c.fails >= 3) c.k = 1;
                dtn = dt * fmax(0.2, fmin(0.8, isfinite(fac) ? fac : 0.2));
            }
            if (c.t >= c.t1) { c.done = 1; c.status = 0; }
            else if (dtn < A.dtmin || !isfinite(dtn) || c.iters >= c.maxiters) { c.done = 1; c.status = -5; }
            if (dtn > A.dtmax) dtn = A.dtmax;
            const double rem = c.t1 - c.t;
            if (dtn >= rem) dtn = rem;
            c.dt = dtn;
            c.go = acc;
            c.stop = c.done || (prb[nch] != 0.0);
            if (rank == 0) {
                M.t = c.t; M.dt = c.dt; M.qold = c.qold;
                M.naccept = c.naccept; M.nreject = c.nreject; M.iters = c.iters;
                M.done = c.done; M.status = c.status;
                M.abm_k = c.k; M.abm_fails = c.fails;
                for (int i = 0; i < 5; ++i) M.psi_prev[i] = c.psi_prev[i];
            }
        }
        if (threadIdx.x == 0 && ALG == 0) {
            const double tot = red[0];
            double EEst = sqrt(tot * inv3n);
            if (!isfinite(EEst)) EEst = INFINITY;
            const double beta1 = 0.14, beta2 = 0.08, gam = 0.9, qmin = 0.2, qmax = 10.0;
            // the PI gain factors EEst^β1 and qold^β2 only shape the next dt: FP32 (a serial FP64
            // pow costs ~3 µs per step on this chip); acceptance uses the FP64 norm EEst itself
            auto powf_ = [](double x, float ex) { return (double)exp2f(ex * log2f((float)x)); };
            const double q11 = powf_(EEst, (float)beta1);
            c.iters += 1;
            double dtn;
            int acc = 0;
            if (EEst <= 1.0) {
                double q = q11 / powf_(c.qold, (float)beta2);
                q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gam));
                const double tn = c.t + dt;
                c.t = (tn >= c.t1) ? c.t1 : tn;
                c.qold = fmax(EEst, 1e-4);
                c.naccept += 1;
                acc = 1;
                dtn = dt / q;
            } else {
                const double q = isfinite(q11) ? fmin(1.0 / qmin, q11 / gam) : 1.0 / qmin;
                c.nreject += 1;
                dtn = dt / q;
            }
            if (c.t >= c.t1) { c.done = 1; c.status = 0; }
            else if (dtn < A.dtmin || !isfinite(dtn) || c.iters >= c.maxiters) { c.done = 1; c.status = -5; }
            if (dtn > A.dtmax) dtn = A.dtmax;
            const double rem = c.t1 - c.t;
            if (dtn >= rem) dtn = rem;
            c.dt = dtn;
            c.go = acc;
            c.stop = c.done || (prb[nch] != 0.0);
            if (rank == 0) {
                M.t = c.t; M.dt = c.dt; M.qold = c.qold;
                M.naccept = c.naccept; M.nreject = c.nreject; M.iters = c.iters;
                M.done = c.done; M.status = c.status;
            }
        }
        __syncthreads();
        if (c.go && ALG == 0) {
            for (int comp = 0; comp < 3; ++comp)
                for (int i = lo + threadIdx.x; i < hi; i += BS) {
                    const int g = comp * N + i;
                    u[g] = un[g];
                    kk[0][g] = kk[6][g];
                }
        } else if (c.go) {
            // f at the corrected point, then Phi_0 = f_{n+1}, Phi_{j+1} = Phi_j(new) - beta_j Phi_j(old)
            float* xb = S.xr + (size_t)(rx & 1) * N;
            if (clus) {
                for (int i = lo + threadIdx.x; i < hi; i += BS) {
                    const float x = (float)(un[i] - m.vpl);
                    xb[i] = x;
                    for (int d = 1; d < csize; ++d) push_f32(xb + i, x, &S.mb[rx & 1], (rank + d) % csize);
                }
                collect(rx & 1, xbytes);
                if (xfail) break;
            }
            ens_rhs<BS>(m, A, S, un, kk[6], lo, hi, clus ? xb : nullptr);
            ++rx;
            const int kq = c.kq;
            // the old differences are loaded before any is overwritten (the stage buffers are
            // distinct arrays): one round trip instead of one per order, same arithmetic
            const int nl = hi - lo;
            for (int t = threadIdx.x; t < 3 * nl; t += BS) {  // one (component, patch) per thread
                    const int comp = (t >= nl) + (t >= 2 * nl);
                    const int g = comp * N + lo + t - comp * nl;
                    double old[5];
#pragma unroll
                    for (int j = 0; j < 5; ++j) old[j] = (j < kq) ? kk[j][g] : 0.0;
                    double nw = kk[6][g];
                    const double un_g = un[g];
#pragma unroll
                    for (int j = 0; j < 5; ++j) {
                        if (j < kq) {
                            kk[j][g] = nw;
                            nw = nw - c.beta[j] * old[j];
                        }
                    }
#pragma unroll
                    for (int j = 1; j <= 5; ++j)
                        if (j == kq) kk[j][g] = nw;
                    u[g] = un_g;
                }
        }
    }
    if (xfail && writer) {  // an exchange timed out: the model stops with an error status
        M.done = 1;
        M.status = -6;
    }
    // every rank leaves the loop at the same step (or on a timed-out exchange); none may exit
    // while a peer can still push into its shared memory
    if (clus) cl.sync();
}

__global__ void k_ens_theta(EnsArgs A, int to_log);

// FFT work arrays Z and W (nq x P each, padded), twiddles (P/2, padded), all float2; two buffers of
// chunk norms + stop flag and the per-component chunk sums (doubles); four mbarriers; two
// slip-rate buffers of N floats
size_t ens_smem_bytes(int nx, int nxi, int P) {
    const size_t N = (size_t)nx * nxi, nch = (N + 31) / 32;
    return sizeof(float2) * (2 * zlen((size_t)((nxi + 1) / 2) * P) + zlen((size_t)P / 2)) +
           sizeof(double) * (2 * (nch + 1) + 3 * nch) + sizeof(uint64_t) * 4 + sizeof(float) * 2 * N;
}

int ens_prepare_model(EnsModel& m, int nx, int nxi, size_t* smem_bytes) {
    if (nx <= 0 || nxi <= 0 || nx > 4096 || nxi > 64)
        return fail(GBC_EINVAL, "ensemble model sizes must satisfy 0 < nx <= 4096, 0 < nxi <= 64");
    memset(&m, 0, sizeof(m));
    m.nx = nx; m.nxi = nxi; m.N = nx * nxi;
    m.P = 2; m.logP = 1;
    while (m.P < 2 * nx - 1) { m.P <<= 1; ++m.logP; }
    *smem_bytes = ens_smem_bytes(nx, nxi, m.P);
    if (*smem_bytes > 200 * 1024) return fail(GBC_EINVAL, "model exceeds the 200 KB shared-memory budget of its FFT buffers");
    return 0;
}

size_t ens_ghat_floats(const EnsModel& m) { return (size_t)m.nxi * m.nxi * (m.P / 2 + 1); }

__global__ void k_ghat(const double* __restrict__ st, int nx, int nxi, int P, float* __restrict__ g);

int ens_ghat(const double* st_dev, const EnsModel& m, float* ghat_dev, cudaStream_t s) {
    k_ghat<<<64, 256, 0, s>>>(st_dev, m.nx, m.nxi, m.P, ghat_dev);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int ens_csize(int N, int maxc, int boost) {
    int c = N <= 600 ? 1 : N <= 1200 ? 2 : N <= 2400 ? 4 : 8;
    if (c < boost) c = boost;
    return c < maxc ? c : maxc;
}

// Predicted microseconds per VCABM5 step of an N-patch model on a cluster of c CTAs of 512 threads:
// a fixed part (step control and barriers), the model's patches spread over the cluster (FFT
// convolution, friction, error norm) and the cluster's exchanges. A fit to single-model timings on
// a GB300 (N = 400 to 1960, c = 1 to 16, within 10 %) of an earlier version of the kernel, whose
// steps were ~1.5x longer throughout; it only ranks the models and the gains of larger clusters
// when they are planned, which the uniform speed-up leaves in the same order.
double ens_step_us(int N, int c) {
    int lg = 0;
    while ((1 << lg) < c) ++lg;
    return 16.0 + (double)N / (11.7 * c) + 2.0 * lg;
}

// Cluster sizes for the n models (done[i] != 0: finished, size 1): every model starts on one
// CTA; then, repeatedly, the model with the largest predicted step latency (ties: more steps left,
// then the lower index) moves to the next size, if that saves at least 3 % and the grouping stays
// within the GPU: the sum over models of 1 / cap[log2 size] at most one, cap[g] the clusters of
// 1 << g CTAs it holds at once (0: size not available).
void ens_plan(int n, const int* N, const int* done, const double* left, const double cap[kEnsGroups], int* w) {
    double used = 0.0;
    for (int i = 0; i < n; ++i) {
        w[i] = 1;
        if (!done[i]) used += cap[0] > 0 ? 1.0 / cap[0] : 1.0;
    }
    for (;;) {
        int best = -1, bg = 0;
        double bl = -1.0, bkey = 0.0;
        for (int i = 0; i < n; ++i) {
            if (done[i]) continue;
            int g = 0;
            while ((1 << g) < w[i]) ++g;
            if (g + 1 >= kEnsGroups || cap[g + 1] <= 0 || cap[g] <= 0) continue;
            const double l = ens_step_us(N[i], w[i]);
            if (ens_step_us(N[i], 2 * w[i]) > 0.97 * l) continue;
            if (used + 1.0 / cap[g + 1] - 1.0 / cap[g] > 1.0 + 1e-9) continue;
            if (l > bl || (l == bl && left[i] > bkey)) { best = i; bg = g; bl = l; bkey = left[i]; }
        }
        if (best < 0) break;
        used += 1.0 / cap[bg + 1] - 1.0 / cap[bg];
        w[best] *= 2;
    }
}

int ens_boost(int nactive, int maxb) {
    int b = 1;
    while (b < maxb && (long long)nactive * b * 2 <= sm_count()) b *= 2;
    return b;
}

// the models still running, grouped by cluster size
void ens_groups(const EnsModel* models, int n, int maxc, int boost, std::vector<int>& order, int first[kEnsGroups],
                int count[kEnsGroups], const int* want) {
    order.clear();
    for (int g = 0; g < kEnsGroups; ++g) {
        first[g] = (int)order.size();
        for (int i = 0; i < n; ++i) {
            const int cs = want ? want[i] : ens_csize(models[i].N, maxc, boost);
            if (!models[i].done && cs == (1 << g)) order.push_back(i);
        }
        count[g] = (int)order.size() - first[g];
    }
}

static int allow_cluster16(const void* kern) {
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(std::make_pair(kern, dev))) return 0;
    GBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    done.insert(std::make_pair(kern, dev));
    return 0;
}

// how many clusters of csize CTAs (block threads each, smem bytes of dynamic shared memory) the
// GPU holds at once; clusters live inside one GPC, so this is less than SMs / csize for large sizes
int ens_max_clusters(int csize, int block, size_t smem, int alg) {
    void (*kern)(EnsArgs) = (block == 128) ? ((alg == 1) ? k_ensemble<128, 1> : k_ensemble<128, 0>)
                          : (block == 256) ? ((alg == 1) ? k_ensemble<256, 1> : k_ensemble<256, 0>)
                                           : ((alg == 1) ? k_ensemble<512, 1> : k_ensemble<512, 0>);
    if ((csize > 8 && allow_cluster16((const void*)kern)) || set_smem_limit((const void*)kern, (int)smem)) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)csize);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (const void*)kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

bool ens_cluster16_ok(size_t smem, int alg) { return ens_max_clusters(16, 512, smem, alg) >= 1; }

template <int BS>
static int launch_cluster(const EnsArgs& A, int nmod, int csize, size_t smem, cudaStream_t s, int prioritize) {
    void (*kern)(EnsArgs) = (A.alg == 1) ? k_ensemble<BS, 1> : k_ensemble<BS, 0>;
    if (int rc = set_smem_limit((const void*)kern, (int)smem)) return rc;
    if (csize > 8)
        if (int rc = allow_cluster16((const void*)kern)) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nmod * csize));
    cfg.blockDim = dim3(BS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    // prioritize 1: larger clusters hold the stiffest models, their CTAs are dispatched first;
    // 2: every group at the greatest priority (a server's batch beside its mantle requests)
    int least = 0, greatest = 0;
    GBC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    int lg = 0;
    while ((1 << lg) < csize) ++lg;
    at[1].id = cudaLaunchAttributePriority;
    at[1].val.priority = (prioritize == 2) ? greatest : std::max(greatest, least - lg);
    cfg.attrs = at;
    cfg.numAttrs = prioritize ? 2 : 1;
    GBC_CUDA(cudaLaunchKernelEx(&cfg, kern, A));
    return 0;
}

int ens_run_groups(const EnsLaunch& L, double reltol, double abstol, double dtmax, double dtmin,
                   unsigned long long budget_ns, int block, size_t smem, cudaStream_t main, int alg,
                   size_t gbytes, int prioritize) {
    EnsArgs A{};
    A.alg = alg;
    // Room for each CTA's copy of its model's spectra (the mixing then reads shared memory instead
    // of L2; same values, same sums): always in the 512-thread cluster groups, which hold a whole
    // SM's registers anyway; in the one-CTA group once every active CTA has an SM to itself.
    long long ctas = 0;
    for (int g = 0; g < kEnsGroups; ++g) ctas += (long long)L.count[g] << g;
    const bool gfit = gbytes > 0 && smem + gbytes + 16 <= 200 * 1024;
    A.models = L.models; A.nmodels = L.n; A.order = L.order;
    A.reltol = reltol; A.abstol = abstol; A.dtmax = dtmax; A.dtmin = dtmin;
    A.budget = 1 << 20;
    A.budget_ns = budget_ns;
    GBC_CUDA(cudaEventRecord(L.fork, main));
    int launched = 0;
    for (int g = kEnsGroups - 1; g >= 0; --g) {  // the largest clusters first
        if (L.count[g] == 0) continue;
        cudaStream_t s = L.aux[g];
        GBC_CUDA(cudaStreamWaitEvent(s, L.fork, 0));
        A.first = L.first[g];
        // models split over clusters are the large ones: 512 threads per CTA measured best for them;
        // the one-CTA group uses the (autotuned) block size
        const int b = (g > 0) ? 512 : block;
        A.gsm = gfit && (g > 0 || ctas <= sm_count()) ? 1 : 0;
        const size_t sg = A.gsm ? smem + gbytes + 16 : smem;
        int rc;
        if (b == 128) rc = launch_cluster<128>(A, L.count[g], 1 << g, sg, s, prioritize);
        else if (b == 512) rc = launch_cluster<512>(A, L.count[g], 1 << g, sg, s, prioritize);
        else rc = launch_cluster<256>(A, L.count[g], 1 << g, sg, s, prioritize);
        if (rc) return rc;
        GBC_CUDA(cudaEventRecord(L.join[g], s));
        GBC_CUDA(cudaStreamWaitEvent(main, L.join[g], 0));
        ++launched;
    }
    count_launches(launched);
    return 0;
}

int ens_launch_create(EnsLaunch& L, int capacity) {
    L = EnsLaunch();
    L.cap = capacity;
    GBC_CUDA(cudaMalloc(&L.order, sizeof(int) * capacity));
    GBC_CUDA(cudaEventCreateWithFlags(&L.fork, cudaEventDisableTiming));
    for (int g = 0; g < kEnsGroups; ++g) {
        GBC_CUDA(cudaStreamCreateWithFlags(&L.aux[g], cudaStreamNonBlocking));
        GBC_CUDA(cudaEventCreateWithFlags(&L.join[g], cudaEventDisableTiming));
    }
    return 0;
}

void ens_launch_destroy(EnsLaunch& L) {
    if (L.order) cudaFree((void*)L.order);
    if (L.fork) cudaEventDestroy(L.fork);
    for (int g = 0; g < kEnsGroups; ++g) {
        if (L.aux[g]) cudaStreamDestroy(L.aux[g]);
        if (L.join[g]) cudaEventDestroy(L.join[g]);
    }
    L = EnsLaunch();
}

// uploads the grouped order of the models (host descriptors) and fills the group table
int ens_launch_prepare(EnsLaunch& L, EnsModel* d_models, const EnsModel* host, int n, int maxc, int boost,
                       cudaStream_t s, const int* want) {
    if (n > L.cap) return fail(GBC_EINVAL, "ensemble launch capacity exceeded");
    std::vector<int> order;
    ens_groups(host, n, maxc, boost, order, L.first, L.count, want);
    L.models = d_models;
    L.n = n;
    if (!order.empty())
        GBC_CUDA(cudaMemcpyAsync((void*)L.order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int ens_theta(EnsModel* d_models, int n, int to_log, cudaStream_t s) {
    EnsArgs A{};
    A.models = d_models; A.nmodels = n;
    k_ens_theta<<<n, 256, 0, s>>>(A, to_log);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

__global__ void k_ens_theta(EnsArgs A, int to_log) {
    const EnsModel& m = A.models[blockIdx.x];
    if (!m.logged) return;  // models with nothing to integrate keep θ untouched
    double* th = m.u + m.N;
    for (int i = threadIdx.x; i < m.N; i += blockDim.x) th[i] = to_log ? log(th[i]) : exp(th[i]);
}

}  // namespace gbc

using namespace gbc;

struct gbc_ensemble {
    int n = 0;
    std::vector<EnsModel> host;
    std::vector<int> has_gf, has_props;
    long long total_n = 0, total_st = 0;
    size_t smem = 0;
    size_t gbytes = 0;  // spectra of the largest model, bytes
    cudaStream_t stream = nullptr;
    EnsModel* d_models = nullptr;
    float* ghat = nullptr;
    double *a = nullptr, *b = nullptr, *L = nullptr, *sig = nullptr, *c1 = nullptr, *boa = nullptr, *iL = nullptr,
           *u = nullptr, *y = nullptr, *un = nullptr;
    double* k[7] = {};
    int block = 256;
    int max_cluster = 16;
    int c16 = -1;  // whether 16-CTA clusters can launch (-1: not yet checked)
    int regroup = 1;
    int log_theta = 1;
    cudaGraphExec_t exec = nullptr;
    int exec_block = 0, exec_budget = 0;
    EnsLaunch lp;
};

namespace gbc {
int launch_gf_ff(const FaultDev& f, double lambda, double mu, int ftype, int nrept, double buffer_ratio, double* st,
                 cudaStream_t s);
}

static int ens_free(gbc_ensemble* e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    ens_launch_destroy(e->lp);
    void* ptrs[] = {e->d_models, e->ghat, e->a, e->b, e->L, e->sig, e->c1, e->boa, e->iL, e->u, e->y, e->un};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int s = 0; s < 7; ++s)
        if (e->k[s]) cudaFree(e->k[s]);
    if (e->stream) cudaStreamDestroy(e->stream);
    return 0;
}

namespace gbc {
// Real spectrum of the symmetric circulant embedding of each Toeplitz column block (length P):
// G[j,l,f] = st[0,j,l] + 2 sum_{m=1}^{nx-1} st[m,j,l] cos(2 pi f m / P), computed in FP64.
__global__ void k_ghat(const double* __restrict__ st, int nx, int nxi, int P, float* __restrict__ g) {
    const int H = P / 2 + 1;
    const long long total = (long long)nxi * nxi * H;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(t % H);
        const long long jl = t / H;  // j * nxi + l
        const int j = (int)(jl / nxi), l = (int)(jl % nxi);
        const double* col = st + (size_t)nx * (j + (size_t)nxi * l);
        double acc = col[0];
        for (int m = 1; m < nx; ++m) acc += 2.0 * col[m] * cospi(2.0 * (double)(((long long)f * m) % P) / P);
        g[t] = (float)acc;
    }
}

}  // namespace gbc

namespace gbc {
int launch_gf_ff_idft(int nx, int nxi, const double* st_dft, double* st, cudaStream_t s);
}


extern "C" {

int gbc_ensemble_create(int nmodels, const int* nx, const int* nxi, gbc_ensemble** out) {
    if (!out) return fail(GBC_EINVAL, "null output handle");
    *out = nullptr;
    if (nmodels <= 0 || !nx || !nxi) return fail(GBC_EINVAL, "ensemble needs at least one model");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(GBC_ENODEV, "no CUDA device available (libgbcycle has no CPU fallback)");
    gbc_ensemble* e = new gbc_ensemble();
    e->n = nmodels;
    e->host.resize(nmodels);
    e->has_gf.assign(nmodels, 0);
    e->has_props.assign(nmodels, 0);
    long long on = 0, os = 0;
    for (int i = 0; i < nmodels; ++i) {
        if (nx[i] <= 0 || nxi[i] <= 0 || nx[i] > 4096 || nxi[i] > 64) {
            delete e;
            return fail(GBC_EINVAL, "ensemble model sizes must satisfy 0 < nx <= 4096, 0 < nxi <= 64");
        }
        EnsModel& m = e->host[i];
        size_t sm = 0;
        if (int rc = ens_prepare_model(m, nx[i], nxi[i], &sm)) {  // sizes and FFT length, as the server's
            delete e;
            return rc;
        }
        m.off_n = on; m.off_st = os;
        on += m.N;
        os += (long long)nxi[i] * nxi[i] * (m.P / 2 + 1);
        e->smem = std::max(e->smem, sm);
        e->gbytes = std::max(e->gbytes, sizeof(float) * ens_ghat_floats(m));
    }
    e->total_n = on;
    e->total_st = os;
    if (e->smem > 200 * 1024) { delete e; return fail(GBC_EINVAL, "largest ensemble model exceeds the 200 KB shared-memory budget of its FFT buffers"); }
    int rc = 0;
    cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaStreamCreate");
    auto A = [&](void** p, size_t bytes) {
        if (rc) return;
        cudaError_t c2 = cudaMalloc(p, bytes);
        if (c2 != cudaSuccess) rc = cuda_fail(c2, "cudaMalloc");
    };
    A((void**)&e->d_models, sizeof(EnsModel) * nmodels);
    A((void**)&e->ghat, sizeof(float) * os);
    for (double** p : {&e->a, &e->b, &e->L, &e->sig, &e->c1, &e->boa, &e->iL}) A((void**)p, sizeof(double) * on);
    for (double** p : {&e->u, &e->y, &e->un}) A((void**)p, sizeof(double) * 3 * on);
    for (int s = 0; s < 7; ++s) A((void**)&e->k[s], sizeof(double) * 3 * on);
    if (!rc) rc = ens_launch_create(e->lp, nmodels);
    if (rc) { ens_free(e); delete e; return rc; }
    for (EnsModel& m : e->host) {
        m.ghat = e->ghat + m.off_st;
        m.a = e->a + m.off_n; m.b = e->b + m.off_n; m.L = e->L + m.off_n; m.sig = e->sig + m.off_n; m.c1 = e->c1 + m.off_n;
        m.boa = e->boa + m.off_n; m.iL = e->iL + m.off_n;
        m.u = e->u + 3 * m.off_n; m.y = e->y + 3 * m.off_n; m.un = e->un + 3 * m.off_n;
        for (int s = 0; s < 7; ++s) m.k[s] = e->k[s] + 3 * m.off_n;
    }
    *out = e;
    return 0;
}

void gbc_ensemble_destroy(gbc_ensemble* e) {
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    ens_free(e);
    delete e;
}

long long gbc_ensemble_state_offset(const gbc_ensemble* e, int model) {
    if (!e || model < 0 || model >= e->n) return -1;
    return 3 * e->host[model].off_n;
}

long long gbc_ensemble_state_len(const gbc_ensemble* e) { return e ? 3 * e->total_n : 0; }

int gbc_ensemble_set_gf(gbc_ensemble* e, int model, int which, const double* host) {
    if (!e || !host || model < 0 || model >= e->n) return fail(GBC_EINVAL, "bad ensemble model or buffer");
    const EnsModel& m = e->host[model];
    const size_t nst = (size_t)m.nx * m.nxi * m.nxi;
    double *d1 = nullptr, *d2 = nullptr;
    GBC_CUDA(cudaMalloc(&d1, sizeof(double) * nst * (which == GBC_GF11_DFT ? 3 : 1)));
    int rc = 0;
    if (which == GBC_GF11_DFT) {
        d2 = d1 + 2 * nst;
        cudaError_t c = cudaMemcpyAsync(d1, host, sizeof(double) * 2 * nst, cudaMemcpyHostToDevice, e->stream);
        if (c != cudaSuccess) rc = cuda_fail(c, "cudaMemcpyAsync");
        if (!rc) rc = launch_gf_ff_idft(m.nx, m.nxi, d1, d2, e->stream);
        count_launches(1);
    } else if (which == GBC_GF11_REAL) {
        d2 = d1;
        cudaError_t c = cudaMemcpyAsync(d1, host, sizeof(double) * nst, cudaMemcpyHostToDevice, e->stream);
        if (c != cudaSuccess) rc = cuda_fail(c, "cudaMemcpyAsync");
    } else {
        rc = fail(GBC_EINVAL, "ensembles hold fault-only models (GBC_GF11_REAL or GBC_GF11_DFT)");
    }
    if (!rc) {
        k_ghat<<<64, 256, 0, e->stream>>>(d2, m.nx, m.nxi, m.P, e->ghat + m.off_st);
        count_launches(1);
        cudaError_t c = cudaStreamSynchronize(e->stream);
        if (c != cudaSuccess) rc = cuda_fail(c, "cudaStreamSynchronize");
    }
    cudaFree(d1);
    if (!rc) e->has_gf[model] = 1;
    return rc;
}

int gbc_ensemble_assemble(gbc_ensemble* e, int model, const gbc_fault_mesh* mf, double lambda, double mu, int ftype,
                          int nrept, double buffer_ratio) {
    if (!e || model < 0 || model >= e->n || !mf) return fail(GBC_EINVAL, "bad ensemble model or mesh");
    const EnsModel& m = e->host[model];
    if (mf->nx != m.nx || mf->nxi != m.nxi) return fail(GBC_EINVAL, "fault mesh does not match the model");
    if (!(buffer_ratio >= 0)) return fail(GBC_EINVAL, "Argument `buffer_ratio` must be ≥ 0.");
    std::vector<double> ax(mf->ax, mf->ax + 2 * mf->nx), axi(mf->axi, mf->axi + 2 * mf->nxi);
    const size_t nst = (size_t)m.nx * m.nxi * m.nxi;
    double* d = nullptr;
    size_t need = nst + 3 * (size_t)mf->nxi + mf->nx + 2 * (size_t)mf->nx + 2 * (size_t)mf->nxi;
    GBC_CUDA(cudaMalloc(&d, sizeof(double) * need));
    double* st = d;
    double* dx = st + nst;
    double* dy = dx + mf->nx;
    double* dz = dy + mf->nxi;
    double* dax = dz + mf->nxi;
    double* daxi = dax + 2 * mf->nx;
    int rc = 0;
    auto up = [&](double* dst, const double* src, size_t n) {
        if (rc) return;
        cudaError_t c = cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream);
        if (c != cudaSuccess) rc = cuda_fail(c, "cudaMemcpyAsync");
    };
    up(dx, mf->x, mf->nx);
    up(dy, mf->y, mf->nxi);
    up(dz, mf->z, mf->nxi);
    up(dax, mf->ax, 2 * mf->nx);
    up(daxi, mf->axi, 2 * mf->nxi);
    if (!rc) {
        FaultDev f{mf->nx, mf->nxi, dx, dy, dz, dax, daxi, mf->dx, mf->dep, mf->dip};
        rc = launch_gf_ff(f, lambda, mu, ftype, nrept, buffer_ratio, st, e->stream);
    }
    if (!rc) {
        k_ghat<<<64, 256, 0, e->stream>>>(st, m.nx, m.nxi, m.P, e->ghat + m.off_st);
        count_launches(2);
        cudaError_t c = cudaStreamSynchronize(e->stream);
        if (c != cudaSuccess) rc = cuda_fail(c, "cudaStreamSynchronize");
    }
    cudaFree(d);
    if (!rc) e->has_gf[model] = 1;
    return rc;
}

int gbc_ensemble_set_fault_props(gbc_ensemble* e, int model, const double* a, const double* b, const double* L,
                                 const double* sigma, double eta, double vpl, double f0, double v0) {
    if (!e || model < 0 || model >= e->n || !a || !b || !L || !sigma) return fail(GBC_EINVAL, "bad argument");
    if (!(f0 > 0) || !(v0 > 0) || !(eta > 0) || !(vpl > 0)) return fail(GBC_EINVAL, "AssertionError: f₀, v₀, η, vpl must be > 0");
    EnsModel& m = e->host[model];
    const size_t N = m.N;
    GBC_CUDA(cudaMemcpyAsync(e->a + m.off_n, a, sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    GBC_CUDA(cudaMemcpyAsync(e->b + m.off_n, b, sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    GBC_CUDA(cudaMemcpyAsync(e->L + m.off_n, L, sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    GBC_CUDA(cudaMemcpyAsync(e->sig + m.off_n, sigma, sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    std::vector<double> c1(N), boa(N), iL(N);
    for (size_t i = 0; i < N; ++i) {
        c1[i] = f0 / a[i] + (b[i] / a[i]) * std::log(v0 / L[i]) - std::log(2.0 * v0);
        boa[i] = b[i] / a[i];
        iL[i] = 1.0 / L[i];
    }
    GBC_CUDA(cudaMemcpyAsync(e->c1 + m.off_n, c1.data(), sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    GBC_CUDA(cudaMemcpyAsync(e->boa + m.off_n, boa.data(), sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    GBC_CUDA(cudaMemcpyAsync(e->iL + m.off_n, iL.data(), sizeof(double) * N, cudaMemcpyHostToDevice, e->stream));
    GBC_CUDA(cudaStreamSynchronize(e->stream));
    m.eta = eta; m.vpl = vpl; m.f0 = f0; m.v0 = v0;
    e->has_props[model] = 1;
    return 0;
}

int gbc_ensemble_set_block(gbc_ensemble* e, int threads) {
    if (!e || (threads != 128 && threads != 256 && threads != 512)) return fail(GBC_EINVAL, "block must be 128, 256 or 512");
    e->block = threads;
    return 0;
}

int gbc_ensemble_set_max_cluster(gbc_ensemble* e, int ctas) {
    if (!e || (ctas != 1 && ctas != 2 && ctas != 4 && ctas != 8 && ctas != 16))
        return fail(GBC_EINVAL, "cluster size must be 1, 2, 4, 8 or 16");
    e->max_cluster = ctas;
    return 0;
}

int gbc_ensemble_set_regroup(gbc_ensemble* e, int on) {
    if (!e) return fail(GBC_EINVAL, "null ensemble");
    e->regroup = on != 0;
    return 0;
}

int gbc_ensemble_plan_clusters(int n, const int* npatch, const int* done, const double* steps_left,
                               const int* capacity, int* sizes) {
    if (n < 0 || !capacity || (n > 0 && (!npatch || !done || !steps_left || !sizes)))
        return fail(GBC_EINVAL, "null argument");
    if (n == 0) return 0;
    double cap[kEnsGroups];
    for (int g = 0; g < kEnsGroups; ++g) {
        if (capacity[g] < 0) return fail(GBC_EINVAL, "negative cluster capacity");
        cap[g] = capacity[g];
    }
    ens_plan(n, npatch, done, steps_left, cap, sizes);
    return 0;
}

int gbc_ensemble_set_log_theta(gbc_ensemble* e, int on) {
    if (!e) return fail(GBC_EINVAL, "null ensemble");
    e->log_theta = on ? 1 : 0;
    return 0;
}


// Integrates every model (or only those with active != 0 when given) from its current state to its
// own t1; state u is the concatenation of the models' (v, θ, δ) on the device.
int gbc_ensemble_integrate_dev(gbc_ensemble* e, double* u_dev, const double* t0, const double* t1,
                               const gbc_solver_opts* o, gbc_solver_stats* stats) {
    if (!e || !u_dev || !t0 || !t1 || !o) return fail(GBC_EINVAL, "null argument");
    if (!(o->reltol > 0) || !(o->abstol >= 0) || !(o->dt0 > 0) || !(o->dtmax > 0) || o->maxiters <= 0)
        return fail(GBC_EINVAL, "invalid solver options");
    if (o->alg != GBC_ALG_TSIT5 && o->alg != GBC_ALG_VCABM5) return fail(GBC_EINVAL, "unknown integrator");
    for (int i = 0; i < e->n; ++i)
        if (!e->has_gf[i] || !e->has_props[i]) return fail(GBC_ESTATE, "ensemble model " + std::to_string(i) + " is missing its Green's function or properties");
    for (int i = 0; i < e->n; ++i) {
        EnsModel& m = e->host[i];
        m.t = t0[i]; m.t1 = t1[i];
        m.dt = std::min(o->dt0, o->dtmax);
        if (m.dt > t1[i] - t0[i]) m.dt = t1[i] - t0[i];
        m.qold = 1e-4;
        m.naccept = m.nreject = m.iters = 0;
        m.maxiters = o->maxiters;
        m.status = 0;
        m.done = (t1[i] <= t0[i]) ? 1 : 0;
        m.started = 0;
        m.abm_k = 1;
        m.abm_fails = 0;
        for (int j = 0; j < 5; ++j) m.psi_prev[j] = 0.0;
        m.log_theta = e->log_theta && !m.done;
        m.logged = m.log_theta;
    }
    cudaStream_t s = e->stream;
    GBC_CUDA(cudaMemcpyAsync(e->d_models, e->host.data(), sizeof(EnsModel) * e->n, cudaMemcpyHostToDevice, s));
    if (u_dev != e->u) GBC_CUDA(cudaMemcpyAsync(e->u, u_dev, sizeof(double) * 3 * e->total_n, cudaMemcpyDeviceToDevice, s));
    if (e->log_theta) {
        if (int rc = ens_theta(e->d_models, e->n, 1, s)) return rc;
        count_launches(1);
    }
    // Persistent launches (one per cluster size, on forked streams, 100 ms of wall clock each),
    // relaunched until every model reports done. With regrouping, the models still running are
    // planned onto cluster sizes again after every launch (their FP64 friction, stage and
    // error-norm work spreads over more SMs; the trajectory does not depend on the cluster size).
    std::vector<int> want;  // per-model cluster sizes (regrouping), empty: the size rule
    // one-CTA models that outnumber the SMs the clusters leave free run at 256 threads, two per
    // SM (128 registers a thread), so that all of them stay resident; a model's steps do not
    // depend on it
    auto block0 = [&]() {
        long long hot_sms = 0;
        for (int g = 1; g < kEnsGroups; ++g) hot_sms += (long long)e->lp.count[g] << g;
        return (e->lp.count[0] > sm_count() - hot_sms) ? 256 : e->block;
    };
    // the fixed size rule: a captured pair of launches, relaunched
    auto capture = [&](int boost) -> int {
        if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
        if (int rc = ens_launch_prepare(e->lp, e->d_models, e->host.data(), e->n, e->max_cluster, boost, s, nullptr))
            return rc;
        const int b0 = block0();
        cudaGraph_t g;
        GBC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int rc = 0;
        for (int k = 0; k < 2 && !rc; ++k)
            rc = ens_run_groups(e->lp, o->reltol, o->abstol, o->dtmax, o->dtmin, 100000000ull, b0, e->smem, s,
                                o->alg, e->gbytes, 1);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (rc) return rc;
        GBC_CUDA(ce);
        GBC_CUDA(cudaGraphInstantiate(&e->exec, g, 0));
        cudaGraphDestroy(g);
        e->exec_block = e->block;
        return 0;
    };
    auto active = [&]() {
        int a = 0;
        for (int i = 0; i < e->n; ++i) a += (e->host[i].done == 0);
        return a;
    };
    // the largest cluster the regrouped tail may use: 16 CTAs where that non-portable size can be
    // resident with the tail's shared memory (FFT buffers + spectra), else 8
    if (e->c16 < 0) e->c16 = ens_cluster16_ok(e->smem + e->gbytes + 16, o->alg) ? 1 : 0;
    const int maxb = std::min(e->max_cluster, e->c16 ? 16 : 8);
    // Regrouping: the models still running are planned onto cluster sizes so that all their CTAs are
    // resident at once (a CTA that waits for a free SM waits a whole launch). Clusters live inside
    // one GPC, so the GPU holds fewer large clusters than SMs / size: a grouping is admitted while
    // the sum over models of 1 / (clusters of its size the GPU holds, from the occupancy query) stays
    // at most one. Every model starts on one CTA; then, repeatedly, the model with the largest
    // predicted per-step latency moves to the next cluster size, if that saves at least 3 % and
    // still fits. A model's trajectory does not depend on its cluster.
    const bool gfit = e->gbytes > 0 && e->smem + e->gbytes + 16 <= 200 * 1024;
    double cap[kEnsGroups];  // clusters of 1 << g CTAs the GPU holds, as launched
    cap[0] = ens_max_clusters(1, 256, e->smem, o->alg);
    for (int g = 1; g < kEnsGroups; ++g)
        cap[g] = ((1 << g) <= maxb) ? ens_max_clusters(1 << g, 512, gfit ? e->smem + e->gbytes + 16 : e->smem, o->alg) : 0;
    auto sizes = [&]() {
        std::vector<int> N(e->n), done(e->n), w(e->n);
        std::vector<double> left(e->n);
        for (int i = 0; i < e->n; ++i) {
            const EnsModel& m = e->host[i];
            N[i] = m.N; done[i] = m.done;
            left[i] = (m.t1 - m.t) / std::max(m.dt, 1e-300);
        }
        ens_plan(e->n, N.data(), done.data(), left.data(), cap, w.data());
        return w;
    };
    if (e->regroup) {
        // One launch per cluster size per host round trip, issued to an idle GPU with the largest
        // clusters first (and at a higher priority): a captured graph, or launches queued behind
        // the previous ones, would leave the order in which the grids reach the GPU open, and a
        // smaller-cluster grid placed first can split the GPCs so that a large cluster waits a
        // whole launch for room (measured: 5 x 16 + 4 x 8 CTAs all start together largest-first,
        // not smallest-first). The host synchronisation costs microseconds per 100 ms launch.
        want = sizes();
        if (int rc = ens_launch_prepare(e->lp, e->d_models, e->host.data(), e->n, e->max_cluster, 1, s, want.data()))
            return rc;
        for (;;) {
            if (int rc = ens_run_groups(e->lp, o->reltol, o->abstol, o->dtmax, o->dtmin, 100000000ull, block0(),
                                        e->smem, s, o->alg, e->gbytes, 1))
                return rc;
            GBC_CUDA(cudaMemcpyAsync(e->host.data(), e->d_models, sizeof(EnsModel) * e->n, cudaMemcpyDeviceToHost, s));
            GBC_CUDA(cudaStreamSynchronize(s));
            if (active() == 0) break;
            std::vector<int> w = sizes();
            bool changed = false;
            for (int i = 0; i < e->n && !changed; ++i) changed = !e->host[i].done && w[i] != want[i];
            if (changed) {
                want = w;
                if (int rc = ens_launch_prepare(e->lp, e->d_models, e->host.data(), e->n, e->max_cluster, 1, s,
                                                want.data()))
                    return rc;
            }
        }
    } else {
        if (int rc = capture(1)) return rc;
        for (;;) {
            GBC_CUDA(cudaGraphLaunch(e->exec, s));
            GBC_CUDA(cudaMemcpyAsync(e->host.data(), e->d_models, sizeof(EnsModel) * e->n, cudaMemcpyDeviceToHost, s));
            GBC_CUDA(cudaStreamSynchronize(s));
            if (active() == 0) break;
        }
    }
    if (e->log_theta) {
        if (int rc = ens_theta(e->d_models, e->n, 0, s)) return rc;
        count_launches(1);
    }
    if (u_dev != e->u) GBC_CUDA(cudaMemcpyAsync(u_dev, e->u, sizeof(double) * 3 * e->total_n, cudaMemcpyDeviceToDevice, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    int status = 0;
    for (int i = 0; i < e->n; ++i) {
        const EnsModel& m = e->host[i];
        if (stats) {
            stats[i].naccept = m.naccept; stats[i].nreject = m.nreject;
            stats[i].nrhs = (o->alg == GBC_ALG_VCABM5) ? m.iters + m.naccept + 1 : 6 * m.iters + 1;
            stats[i].t = m.t; stats[i].dt = m.dt; stats[i].status = m.status;
        }
        if (m.status != 0) status = GBC_ESOLVER;
    }
    if (status) return fail(GBC_ESOLVER, "at least one ensemble model stopped early");
    return 0;
}

int gbc_ensemble_integrate(gbc_ensemble* e, double* u_host, const double* t0, const double* t1,
                           const gbc_solver_opts* o, gbc_solver_stats* stats) {
    if (!e || !u_host) return fail(GBC_EINVAL, "null argument");
    GBC_CUDA(cudaMemcpyAsync(e->u, u_host, sizeof(double) * 3 * e->total_n, cudaMemcpyHostToDevice, e->stream));
    int rc = gbc_ensemble_integrate_dev(e, e->u, t0, t1, o, stats);
    if (rc != 0 && rc != GBC_ESOLVER) return rc;
    GBC_CUDA(cudaMemcpyAsync(u_host, e->u, sizeof(double) * 3 * e->total_n, cudaMemcpyDeviceToHost, e->stream));
    GBC_CUDA(cudaStreamSynchronize(e->stream));
    return rc;
}

void* gbc_ensemble_stream(gbc_ensemble* e) { return e ? (void*)e->stream : nullptr; }

}  // extern "C"
