// Parameter sweeps on one geometry: K variants of a viscoelastic model (equation.jl:185-205) that
// share its Green's functions and differ in their friction and viscosity properties and their
// initial states (the reference's scripts rerun one assembled model with other properties,
// examples/otf-with-mantle.jl:44-56, 140-162). One right-hand side applies the block-scaled BF16
// interaction rows [G12 | 0 | G22 ; 0 | G21] to all K states at once: a product with K columns
// instead of K matrix-vector products, so the matrix streams from HBM once per evaluation for the
// whole sweep. Two engines compute it:
//  * SIMT: one 32-row tile and a group of 8 variants per CTA on the FP32 pipe, every variant's sum
//    in the order of the single-model GEMV (k_gemv_tma), so a variant's right-hand side equals the
//    single model's bit for bit. The matrix is read once per group of 8 variants.
//  * UMMA: tcgen05 MMAs (BF16 x BF16 -> FP32 in TMEM) on 128-row tiles that TMA stages with
//    128-byte swizzle. Each FP32 state column enters as three BF16 columns hi + mid + lo whose
//    sum is the FP32 value exactly (8 + 8 + 8 significand bits); the products are exact in FP32.
//    A 128 x 128 k-block is one scale block of the matrix, so each k-block's MMAs start a fresh
//    accumulator and the epilogue warps apply the block's FP32 scale as they drain it from TMEM
//    (two accumulators alternate so the drain overlaps the next k-block's MMAs).
// UMMA is the default engine. The fault rows (FP32 Toeplitz sum + the G21 part, FP64 friction) run
// per variant with the single model's kernel body; optionally (gbc_sweep_set_fault_product) the
// dense fault-fault block joins the tensor-core product as a second segment of exact hi/mid/lo BF16
// planes and only the friction stays per variant. Integration: each variant has its own step size, error norm and
// accept/reject (the single model's Tsit5 or VCABM5 controllers); the variants go through the
// stages together so one product serves all of them, and a variant that reached t1 stops changing.
//
// Every mbarrier wait of the UMMA kernel is bounded and also gives up when another role of the CTA
// has given up; on a timeout the CTA records an error word, waits (bounded) for its own TMA copies
// and MMAs in flight, frees its TMEM and returns. Its shared memory (> 114 KB) keeps one CTA per SM,
// so the TMEM allocation never waits for another CTA.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "control.cuh"
#include "gbc_internal.cuh"
#include "mixed.cuh"
#include "model.cuh"
#include "rhs.cuh"
#include "tma.cuh"
#include "umma.cuh"

namespace gbc {

constexpr int kSwMaxVariants = 64;

struct SweepArgs {
    int K, Kp, N, ne, nx, nxi, npad, nlaws;
    long long n, ldq, rowsq, Mpad;   // n: state length of one variant
    StateLayout lay;                 // offsets of v, θ, ϵ, σ, δ in one variant's state
    const uint16_t* q;               // the base model's block-scaled BF16 rows (rowsq x ldq)
    const float* qscale;             // one FP32 scale per 128 x 128 block
    const float* st32;               // FP32 Toeplitz kernel
    const double *a, *b, *L, *sig;   // K x N
    const double* fp;                // K x 4: eta, vpl, f0, v0
    const double *gamma, *nexp;      // K x (nlaws x ne)
    const double* deps0;             // K x 6
    float* x32;                      // Kp x ldq state columns in FP32 (SIMT)
    uint16_t* xb;                    // 3 Kp x ldq BF16: rows [0,Kp) hi, [Kp,2Kp) mid, [2Kp,3Kp) lo (UMMA)
    float* y32;                      // K x N: the G21 part of every variant's fault rows
    const Ctrl* ctrl;                // K; nullptr: evaluate every variant
    int skip;                        // 1: skip variants done; 2: also the ones whose step was rejected
    const int* ndone;                // variants done; the product returns once all are
    int* err;                        // device error word
};

// the single-model argument view of variant k (the fields friction, viscosity and fault rows read)
__device__ __forceinline__ RhsArgs variant_view(const SweepArgs& s, int k) {
    RhsArgs a{};
    a.nx = s.nx;
    a.nxi = s.nxi;
    a.ne = s.ne;
    a.N = s.N;
    a.npad = s.npad;
    a.a = s.a + (size_t)k * s.N;
    a.b = s.b + (size_t)k * s.N;
    a.L = s.L + (size_t)k * s.N;
    a.sig = s.sig + (size_t)k * s.N;
    a.eta = s.fp[4 * k];
    a.vpl = s.fp[4 * k + 1];
    a.f0 = s.fp[4 * k + 2];
    a.v0 = s.fp[4 * k + 3];
    a.gamma = s.gamma + (size_t)k * s.nlaws * s.ne;
    a.nexp = s.nexp + (size_t)k * s.nlaws * s.ne;
    a.nlaws = s.nlaws;
#pragma unroll
    for (int j = 0; j < 6; ++j) a.deps0[j] = s.deps0[6 * k + j];
    a.st32 = s.st32;
    a.y32 = s.y32 + (size_t)k * s.N;
    a.mode = GBC_PREC_BF16;
    a.log_theta = 0;
    return a;
}

__device__ __forceinline__ bool sw_skip(const SweepArgs& s, int k) {
    if (!s.ctrl || s.skip == 0) return false;
    const Ctrl& c = s.ctrl[k];
    return s.skip == 1 ? c.done != 0 : (c.done != 0 || c.skip2 != 0);
}

// x = hi + mid + lo exactly for 2^-102 <= |x| < 2^128 (1 - 2^-9): each residual is exact in FP32
// and holds at most 16, then 8 significant bits (below the range the last part rounds to a BF16
// subnormal, off by at most 2^-134; above it bf16(x) overflows)
__device__ __forceinline__ void bf16_split3(float x, uint16_t& h, uint16_t& m, uint16_t& l) {
    const __nv_bfloat16 bh = __float2bfloat16_rn(x);
    const float r1 = __fsub_rn(x, __bfloat162float(bh));
    const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
    const float r2 = __fsub_rn(r1, __bfloat162float(bm));
    const __nv_bfloat16 bl = __float2bfloat16_rn(r2);
    h = __bfloat16_as_ushort(bh);
    m = __bfloat16_as_ushort(bm);
    l = __bfloat16_as_ushort(bl);
}

template <bool SPLIT>
__device__ __forceinline__ void sw_put(const SweepArgs& s, int k, long long col, float x) {
    if (SPLIT) {
        uint16_t h, m, l;
        bf16_split3(x, h, m, l);
        s.xb[(size_t)k * s.ldq + col] = h;
        s.xb[(size_t)(s.Kp + k) * s.ldq + col] = m;
        s.xb[(size_t)(2 * s.Kp + k) * s.ldq + col] = l;
    } else {
        s.x32[(size_t)k * s.ldq + col] = x;
    }
}

// per variant (blockIdx.y): x = [v - vpl; 0; dϵ - dϵ₀; 0] and dϵ, as k_prologue_mixed does
template <bool SPLIT>
__global__ void k_sw_prologue(SweepArgs s, const double* __restrict__ U, double* __restrict__ DU) {
    const int k = blockIdx.y;
    if (sw_skip(s, k)) return;
    const StateLayout L = s.lay;
    const double* u = U + (size_t)k * s.n;
    double* du = DU + (size_t)k * s.n;
    const RhsArgs a = variant_view(s, k);
    const int ne = s.ne, N = s.N;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N + ne; t += gridDim.x * blockDim.x) {
        if (t < N) {
            sw_put<SPLIT>(s, k, t, (float)(u[L.v + t] - a.vpl));
            continue;
        }
        const int i = t - N;
        double d[6];
        viscous_rates(a, u + L.sig, i, d);
        double* deps = du + L.eps;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            deps[i + j * ne] = d[j];
            sw_put<SPLIT>(s, k, s.npad + i + (long long)j * ne, (float)(d[j] - a.deps0[j]));
        }
    }
}

// the product's row `row` for variant k: mantle rows to dσ (FP64), fault rows to y32
__device__ __forceinline__ void sw_store(const SweepArgs& s, const StateLayout& L, double* __restrict__ DU, int k,
                                         long long row, float v) {
    if (row < 6LL * s.ne) DU[(size_t)k * s.n + L.sig + row] = (double)v;
    else if (row >= s.Mpad && row < s.Mpad + s.N) s.y32[(size_t)k * s.N + (row - s.Mpad)] = v;
}

// ---- SIMT engine ------------------------------------------------------------------------------
constexpr int kSwRows = 32, kSwGroup = 8;

__global__ void __launch_bounds__(256) k_sw_gemm_simt(SweepArgs s, double* __restrict__ DU) {
    if (s.ndone && *s.ndone >= s.K) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long row0 = (long long)blockIdx.x * kSwRows;
    const int k0 = blockIdx.y * kSwGroup;
    const int nch = (int)(s.ldq / 256);
    const long long ncb = s.ldq / 128, rb = row0 / 128;
    float acc[4][kSwGroup];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int v = 0; v < kSwGroup; ++v) acc[r][v] = 0.f;
    for (int c = 0; c < nch; ++c) {
        float4 x0[kSwGroup], x1[kSwGroup];
#pragma unroll
        for (int v = 0; v < kSwGroup; ++v) {
            const float4* xv = reinterpret_cast<const float4*>(s.x32 + (size_t)(k0 + v) * s.ldq + (size_t)c * 256) + 2 * lane;
            x0[v] = __ldg(xv);
            x1[v] = __ldg(xv + 1);
        }
        const float sc = __ldg(s.qscale + rb * ncb + 2LL * c + (lane >> 4));
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint4 qv =
                __ldg(reinterpret_cast<const uint4*>(s.q + (size_t)(row0 + 4 * warp + r) * s.ldq + (size_t)c * 256) + lane);
            float f[8];
            unpack8<GBC_PREC_BF16>(qv, f);
#pragma unroll
            for (int v = 0; v < kSwGroup; ++v) {
                float p = f[0] * x0[v].x;
                p = fmaf(f[1], x0[v].y, p);
                p = fmaf(f[2], x0[v].z, p);
                p = fmaf(f[3], x0[v].w, p);
                p = fmaf(f[4], x1[v].x, p);
                p = fmaf(f[5], x1[v].y, p);
                p = fmaf(f[6], x1[v].z, p);
                p = fmaf(f[7], x1[v].w, p);
                acc[r][v] = fmaf(sc, p, acc[r][v]);
            }
        }
    }
    const StateLayout L = s.lay;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const long long row = row0 + 4 * warp + r;
#pragma unroll
        for (int v = 0; v < kSwGroup; ++v) {
            float val = acc[r][v];
            for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
            if (lane == 0 && k0 + v < s.K) sw_store(s, L, DU, k0 + v, row, val);
        }
    }
}

// ---- UMMA engine ------------------------------------------------------------------------------
// Per stage (one 128-column k-block = one scale block): A as two 128-row x 64-column halves and B
// (the 3 Kp split state columns) as two N-row x 64-column halves, each half rows of 128 bytes.
template <int KP>
struct UmmaCfg {
    static constexpr int N = 3 * KP;              // MMA N: hi, mid, lo columns of every variant
    static constexpr int A_HALF = 128 * 128;      // bytes
    static constexpr int B_HALF = N * 128;
    static constexpr int STAGE = 2 * A_HALF + 2 * B_HALF;
    static constexpr int STAGES = KP == 16 ? 4 : KP == 32 ? 3 : 2;
    static constexpr int TCOLS = 2 * N <= 128 ? 128 : 2 * N <= 256 ? 256 : 512;  // two accumulators
    static constexpr int SMEM = 1024 + STAGES * STAGE + 128;  // alignment slack, stages, barriers
    static_assert(N % 16 == 0 && N <= 256, "M = 128 MMAs need N a multiple of 16 up to 256");
    static_assert(B_HALF % 1024 == 0, "swizzled tiles must stay 1024-byte aligned");
    static_assert(SMEM > 116 * 1024 && SMEM <= 227 * 1024, "one CTA per SM, inside the 227 KB limit");
};

__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, unsigned parity, volatile int* abort_flag) {
    for (long long i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255) == 0 && *abort_flag) return false;
    }
    return false;
}

// One product launch: the 128-row tiles of a BF16 matrix (tmA) times the split state columns.
// Mantle segment: the base model's unified rows, an FP32 scale per 128 x 128 block, results to dσ
// and y32 (sw_store). Fault segment: the hi, mid and lo BF16 planes of the dense fault-fault block
// (no scale), results to y[k * ldy + row].
struct UmmaSeg {
    long long ntiles;    // 128-row tiles
    int nkb;             // 128-column k-blocks per tile
    const float* scale;  // (ntiles x nkb) block scales, or nullptr
    float* y;            // fault segment output (nullptr: mantle stores)
    long long ldy;
};

// Warp 0 lane 0: TMA producer. Warp 1 lane 0: MMA issuer. Warps 2-5: epilogue, warp w draining
// TMEM lanes 32 (w % 4) .. +31 (= tile rows). Persistent over 128-row tiles t = blockIdx.x + i grid.
template <int KP>
__global__ void __launch_bounds__(192, 1) k_sw_gemm_umma(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB, SweepArgs s,
                                                         UmmaSeg g, double* __restrict__ DU) {
    using C = UmmaCfg<KP>;
    if (s.ndone && *s.ndone >= s.K) return;
    extern __shared__ unsigned char sm_raw[];
    const unsigned raw = smem_u32(sm_raw);
    unsigned char* sm = sm_raw + (((raw + 1023u) & ~1023u) - raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + C::STAGES * C::STAGE);
    uint64_t* empty = full + C::STAGES;
    uint64_t* tfull = empty + C::STAGES;  // 2: accumulator b ready
    uint64_t* tempty = tfull + 2;         // 2: accumulator b drained (4 epilogue warps)
    uint64_t* mdone = tempty + 2;         // every MMA of this CTA completed
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mdone + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < C::STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 4);
        }
        mbar_init(mdone, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) umma::tmem_alloc(tslot, C::TCOLS);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = *tslot;
    const long long ntiles = g.ntiles;
    const int nkb = g.nkb;

    if (warp == 0 && lane == 0) {  // ---- producer
        long long it = 0;
        bool ok = true;
        for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x)
            for (int cb = 0; cb < nkb; ++cb, ++it) {
                const int st = (int)(it % C::STAGES);
                const unsigned ph = (unsigned)((it / C::STAGES) & 1);
                if (!wait_or_abort(&empty[st], ph ^ 1u, abort_flag)) { ok = false; break; }
                unsigned char* a0 = sm + st * C::STAGE;
                unsigned char* b0 = a0 + 2 * C::A_HALF;
                mbar_expect_tx(&full[st], C::STAGE);
                tma_tile(a0, &tmA, cb * 128, (int)(t * 128), &full[st]);
                tma_tile(a0 + C::A_HALF, &tmA, cb * 128 + 64, (int)(t * 128), &full[st]);
                tma_tile(b0, &tmB, cb * 128, 0, &full[st]);
                tma_tile(b0 + C::B_HALF, &tmB, cb * 128 + 64, 0, &full[st]);
            }
        if (!ok) {
            *abort_flag = 1;
            atomicExch(s.err, 3);
        }
        // the copies of the last STAGES fills have landed before the shared memory goes away
        for (long long j = (it > C::STAGES ? it - C::STAGES : 0); j < it; ++j)
            mbar_wait(&full[j % C::STAGES], (unsigned)((j / C::STAGES) & 1));
    } else if (warp == 1 && lane == 0) {  // ---- MMA issuer
        const uint32_t idesc = umma::idesc_bf16_f32(128, C::N);
        long long it = 0;
        bool ok = true;
        for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x)
            for (int cb = 0; cb < nkb; ++cb, ++it) {
                const int st = (int)(it % C::STAGES);
                const unsigned ph = (unsigned)((it / C::STAGES) & 1);
                const int b = (int)(it & 1);
                const unsigned bph = (unsigned)((it >> 1) & 1);
                if (!wait_or_abort(&full[st], ph, abort_flag) || !wait_or_abort(&tempty[b], bph ^ 1u, abort_flag)) {
                    ok = false;
                    break;
                }
                umma::fence_after();
                const uint32_t sa = smem_u32(sm + st * C::STAGE);
                const uint32_t sb = sa + 2 * C::A_HALF;
                const uint32_t d = tmem + (uint32_t)(b * C::N);
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        umma::mma_bf16(d, umma::sdesc_sw128(sa + h * C::A_HALF + 32 * kk),
                                       umma::sdesc_sw128(sb + h * C::B_HALF + 32 * kk), idesc, (h | kk) ? 1u : 0u);
                umma::commit(&empty[st]);
                umma::commit(&tfull[b]);
            }
        if (!ok) {
            *abort_flag = 1;
            atomicExch(s.err, 3);
        }
        umma::commit(mdone);  // every MMA issued above has completed once this arrives
        mbar_wait(mdone, 0);
    } else if (warp >= 2) {  // ---- epilogue
        const int quad = warp & 3;
        const long long ncb = nkb;
        const StateLayout L = s.lay;
        long long it = 0;
        bool ok = true;
        for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            float acc[KP];
#pragma unroll
            for (int j = 0; j < KP; ++j) acc[j] = 0.f;
            for (int cb = 0; cb < nkb; ++cb, ++it) {
                const int b = (int)(it & 1);
                const unsigned bph = (unsigned)((it >> 1) & 1);
                if (!wait_or_abort(&tfull[b], bph, abort_flag)) { ok = false; break; }
                umma::fence_after();
                const float sc = g.scale ? __ldg(g.scale + t * ncb + cb) : 1.0f;
                const uint32_t tb = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(b * C::N);
#pragma unroll
                for (int ch = 0; ch < KP / 16; ++ch) {
                    uint32_t r[48];
                    umma::ld3x16(tb + ch * 16, tb + KP + ch * 16, tb + 2 * KP + ch * 16, r);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        acc[ch * 16 + j] = fmaf(sc, (__uint_as_float(r[j]) + __uint_as_float(r[16 + j])) +
                                                        __uint_as_float(r[32 + j]),
                                                acc[ch * 16 + j]);
                }
                umma::fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[b]);
            }
            if (!ok) break;
            const long long row = t * 128 + 32 * quad + lane;
            if (g.y) {
#pragma unroll
                for (int k = 0; k < KP; ++k)
                    if (k < s.K) g.y[(size_t)k * g.ldy + row] = acc[k];
            } else {
#pragma unroll
                for (int k = 0; k < KP; ++k)
                    if (k < s.K) sw_store(s, L, DU, k, row, acc[k]);
            }
        }
        if (!ok) {
            *abort_flag = 1;
            atomicExch(s.err, 3);
        }
    }
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        umma::fence_after();
        umma::tmem_dealloc(tmem, C::TCOLS);
    }
}

// ---- fault rows ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(kFR_II * kFR_L) k_sw_fault_rows(SweepArgs s, const double* __restrict__ U,
                                                                double* __restrict__ DU) {
    const int k = blockIdx.y;
    if (sw_skip(s, k)) return;
    extern __shared__ float fsm[];
    const RhsArgs a = variant_view(s, k);
    fault_rows_cta(a, U + (size_t)k * s.n, DU + (size_t)k * s.n, s.lay, (int)blockIdx.x, fsm);
}

// ---- fault rows on the tensor cores ----------------------------------------------------------
// The dense fault-fault block G11[i][k] = st32[|ii - kk| + nx (j + nxi l)] (i = ii + nx j, k = kk + nx l)
// as three BF16 planes hi + mid + lo whose sum is the FP32 entry exactly; planes are (Nf x Nf),
// Nf = N rounded up to 128, stacked as rows [p Nf, (p + 1) Nf), zero outside the N x N block.
__global__ void k_sw_fault_planes(int nx, int nxi, int N, long long Nf, const float* __restrict__ st32,
                                  uint16_t* __restrict__ qf) {
    const long long total = Nf * Nf;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long i = e / Nf, k = e % Nf;
        float g = 0.f;
        if (i < N && k < N) {
            const int ii = (int)(i % nx), j = (int)(i / nx), kk = (int)(k % nx), l = (int)(k / nx);
            g = st32[(ii > kk ? ii - kk : kk - ii) + (size_t)nx * (j + (size_t)nxi * l)];
        }
        uint16_t h, m, lo;
        bf16_split3(g, h, m, lo);
        qf[e] = h;
        qf[total + e] = m;
        qf[2 * total + e] = lo;
    }
}

// per variant (blockIdx.y): dτ = (G11 x from the three planes) + (G21 part), then the FP64 friction
__global__ void k_sw_friction(SweepArgs s, const float* __restrict__ yf, long long Nf, const double* __restrict__ U,
                              double* __restrict__ DU) {
    const int k = blockIdx.y;
    if (sw_skip(s, k)) return;
    const RhsArgs a = variant_view(s, k);
    const float* y = yf + (size_t)k * 3 * Nf;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.N; i += gridDim.x * blockDim.x) {
        const float ff = (y[i] + y[Nf + i]) + y[2 * Nf + i];
        fault_friction(a, U + (size_t)k * s.n, DU + (size_t)k * s.n, s.lay, i, (double)ff + (double)a.y32[i]);
    }
}

// ---- integration kernels: blockIdx.y (or the thread, for the one-block kernels) = variant --------
struct SwK {
    const double* k[7];
};
struct SwPhi {
    double* p[kAbmMax + 1];
};

__global__ void k_sw_stage(int st, long long n, const double* __restrict__ U, SwK K, double* __restrict__ Y,
                           const Ctrl* __restrict__ ctrl) {
    const Ctrl* c = ctrl + blockIdx.y;
    if (c->done) return;
    const double dt = c->dt;
    const size_t off = (size_t)blockIdx.y * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int r = 0; r < st; ++r) acc = fma(c_ta[st][r], K.k[r][off + i], acc);
        Y[off + i] = U[off + i] + dt * acc;
    }
}

// block sum of per-thread error squares into partial[variant * gridDim.x + block]
__device__ __forceinline__ void sw_partial(double ss, int bad, double* partial) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) {
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = bad ? INFINITY : ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += red[w];
        partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = b;
    }
}

__global__ void k_sw_error(long long n, const double* __restrict__ U, const double* __restrict__ UN, SwK K,
                           double* __restrict__ partial, const Ctrl* __restrict__ ctrl) {
    const Ctrl* c = ctrl + blockIdx.y;
    if (c->done) return;
    const double dt = c->dt, rtol = c->reltol, atol = c->abstol;
    const size_t off = (size_t)blockIdx.y * n;
    double ss = 0.0;
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double e = 0.0;
#pragma unroll
        for (int st = 0; st < 7; ++st) e = fma(c_te[st], K.k[st][off + i], e);
        e *= dt;
        const double unv = UN[off + i];
        const double r = e / (atol + rtol * fmax(fabs(U[off + i]), fabs(unv)));
        ss = fma(r, r, ss);
        bad |= !isfinite(unv);
    }
    sw_partial(ss, bad, partial);
}

// one thread per variant: the error norm from its block partials (summed in block order) and the
// step controller; alg 0 Tsit5, 1 VCABM5
__global__ void k_sw_control(int K, long long n, int eb, const double* __restrict__ partial, Ctrl* ctrl, int alg) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= K) return;
    Ctrl* c = ctrl + v;
    if (c->done) return;
    double tot = 0.0;
    for (int b = 0; b < eb; ++b) tot += partial[(size_t)v * eb + b];
    if (alg == 1) abm_control(c, sqrt(tot / (double)n));
    else tsit5_control(c, sqrt(tot / (double)n));
}

__global__ void k_sw_commit(long long n, double* __restrict__ U, const double* __restrict__ UN, double* __restrict__ K0,
                            const double* __restrict__ K6, const Ctrl* __restrict__ ctrl) {
    if (!ctrl[blockIdx.y].accept) return;
    const size_t off = (size_t)blockIdx.y * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        U[off + i] = UN[off + i];
        K0[off + i] = K6[off + i];
    }
}

// one block of >= K threads: clear the accept flags and count the variants done
__global__ void k_sw_clear(int K, Ctrl* ctrl, int* ndone) {
    const int v = threadIdx.x;
    int done = 0;
    if (v < K) {
        ctrl[v].accept = 0;
        ctrl[v].record = 0;
        done = ctrl[v].done;
    }
    const int cnt = __syncthreads_count(done);
    if (threadIdx.x == 0) *ndone = cnt;
}

__global__ void k_sw_abm_coef(int K, Ctrl* ctrl) {
    const int v = threadIdx.x;
    if (v < K && !ctrl[v].done) abm_coef(ctrl + v);
}

__global__ void k_sw_abm_predict(long long n, const double* __restrict__ U, SwPhi P, double* __restrict__ YP,
                                 double* __restrict__ SV, const Ctrl* __restrict__ ctrl) {
    const Ctrl* c = ctrl + blockIdx.y;
    if (c->done) return;
    const int k = c->kq;
    const double h = c->dt;
    double beta[kAbmMax], g[kAbmMax];
#pragma unroll
    for (int j = 0; j < kAbmMax; ++j) {
        beta[j] = c->beta[j];
        g[j] = c->g[j];
    }
    const size_t off = (size_t)blockIdx.y * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double sacc = 0.0, acc = 0.0;
#pragma unroll
        for (int j = 0; j < kAbmMax; ++j) {
            if (j < k) {
                const double pj = beta[j] * P.p[j][off + i];
                sacc += pj;
                acc = fma(g[j], pj, acc);
            }
        }
        SV[off + i] = sacc;
        YP[off + i] = U[off + i] + h * acc;
    }
}

__global__ void k_sw_abm_correct(long long n, const double* __restrict__ U, const double* __restrict__ YP,
                                 const double* __restrict__ FP, const double* __restrict__ SV, double* __restrict__ UN,
                                 double* __restrict__ partial, const Ctrl* __restrict__ ctrl) {
    const Ctrl* c = ctrl + blockIdx.y;
    if (c->done) return;
    const int k = c->kq;
    const double h = c->dt, rtol = c->reltol, atol = c->abstol;
    const double gk = c->g[k], ce = h * (c->g[k] - c->g[k - 1]);
    const size_t off = (size_t)blockIdx.y * n;
    double ss = 0.0;
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double pk = FP[off + i] - SV[off + i];
        const double yn = YP[off + i] + h * gk * pk;
        UN[off + i] = yn;
        const double r = ce * pk / (atol + rtol * fmax(fabs(U[off + i]), fabs(yn)));
        ss = fma(r, r, ss);
        bad |= !isfinite(yn);
    }
    sw_partial(ss, bad, partial);
}

__global__ void k_sw_abm_commit(long long n, double* __restrict__ U, const double* __restrict__ UN,
                                const double* __restrict__ FN, SwPhi P, const Ctrl* __restrict__ ctrl) {
    const Ctrl* c = ctrl + blockIdx.y;
    if (!c->accept) return;
    const int k = c->kq;
    double beta[kAbmMax];
#pragma unroll
    for (int j = 0; j < kAbmMax; ++j) beta[j] = c->beta[j];
    const size_t off = (size_t)blockIdx.y * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        // every old difference is loaded before any is overwritten: the arrays are distinct, but
        // pointers held in a struct carry no no-alias promise, so loads interleaved with the stores
        // would each wait for the store before them
        double old[kAbmMax];
#pragma unroll
        for (int j = 0; j < kAbmMax; ++j) old[j] = (j < k) ? P.p[j][off + i] : 0.0;
        const double un = UN[off + i];
        double nw = FN[off + i];
        U[off + i] = un;
#pragma unroll
        for (int j = 0; j < kAbmMax; ++j) {
            if (j < k) {
                P.p[j][off + i] = nw;
                nw = nw - beta[j] * old[j];
            }
        }
        P.p[k][off + i] = nw;
    }
}

}  // namespace gbc

using namespace gbc;

struct gbc_sweep {
    gbc_model* base = nullptr;
    int K = 0, Kp = 0, engine = GBC_SWEEP_UMMA, nlaws = 1;
    int N = 0, ne = 0, nx = 0, nxi = 0, npad = 0;
    long long n = 0, ldq = 0, rowsq = 0, Mpad = 0;
    cudaStream_t stream = nullptr;
    DevBuf a, b, L, sig, fp, gamma, nexp, deps0;
    RawBuf x32, xb, y32, err, ndone;
    alignas(128) unsigned char tmA[128];
    alignas(128) unsigned char tmB[128];
    // fault rows on the tensor cores (optional): the hi/mid/lo planes of the dense fault-fault block
    int fault_tc = 0;
    long long Nf = 0;
    RawBuf qf, yf;
    alignas(128) unsigned char tmF[128];
    // integration
    DevBuf U, DU, k[7], y, un, phi[kAbmMax + 1], partial;
    RawBuf ctrl;
    Ctrl* ctrl_host = nullptr;
    int* ndone_host = nullptr;
    int eb = 0;
    cudaGraphExec_t exec = nullptr;
    long long graph_launches = 0, steps_per_launch = 0;

    SweepArgs args(const Ctrl* c, int skip) const {
        SweepArgs s{};
        s.K = K; s.Kp = Kp; s.N = N; s.ne = ne; s.nx = nx; s.nxi = nxi; s.npad = npad; s.nlaws = nlaws;
        s.n = n; s.ldq = ldq; s.rowsq = rowsq; s.Mpad = Mpad;
        s.lay = layout_of(N, ne);
        s.q = static_cast<const uint16_t*>(base->q.p);
        s.qscale = static_cast<const float*>(base->qscale.p);
        s.st32 = static_cast<const float*>(base->st32.p);
        s.a = a.p; s.b = b.p; s.L = L.p; s.sig = sig.p; s.fp = fp.p;
        s.gamma = gamma.p; s.nexp = nexp.p; s.deps0 = deps0.p;
        s.x32 = static_cast<float*>(x32.p);
        s.xb = static_cast<uint16_t*>(xb.p);
        s.y32 = static_cast<float*>(y32.p);
        s.ctrl = c;
        s.skip = skip;
        s.ndone = c ? static_cast<const int*>(ndone.p) : nullptr;
        s.err = static_cast<int*>(err.p);
        return s;
    }
    // the base model still holds the BF16 rows the sweep was built on
    int check_base() const {
        if (base->precision != GBC_PREC_BF16 || base->mixed_dirty)
            return fail(GBC_ESTATE, "the base model's Green's functions or precision changed: create the sweep again");
        return 0;
    }
};

namespace gbc {

template <int KP>
static int launch_umma(const unsigned char* tmap_a, const gbc_sweep* w, const SweepArgs& s, const UmmaSeg& g,
                       double* DU, cudaStream_t st) {
    using C = UmmaCfg<KP>;
    if (int rc = set_smem_limit((const void*)k_sw_gemm_umma<KP>, C::SMEM)) return rc;
    const int grid = (int)std::min<long long>(g.ntiles, sm_count());
    CUtensorMap ta, tb;
    memcpy(&ta, tmap_a, sizeof(ta));
    memcpy(&tb, w->tmB, sizeof(tb));
    k_sw_gemm_umma<KP><<<grid, 192, C::SMEM, st>>>(ta, tb, s, g, DU);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

static int launch_umma_kp(const unsigned char* tmap_a, const gbc_sweep* w, const SweepArgs& s, const UmmaSeg& g,
                          double* DU, cudaStream_t st) {
    return s.Kp == 16 ? launch_umma<16>(tmap_a, w, s, g, DU, st)
         : s.Kp == 32 ? launch_umma<32>(tmap_a, w, s, g, DU, st)
                      : launch_umma<64>(tmap_a, w, s, g, DU, st);
}

// prologue, product, fault rows: three kernels for all variants
static int sweep_rhs(const gbc_sweep* w, const SweepArgs& s, const double* U, double* DU, cudaStream_t st) {
    const int sms = sm_count();
    int g = (s.N + s.ne + 255) / 256;
    if (g > sms * 8) g = sms * 8;
    const dim3 gp((unsigned)g, (unsigned)s.K);
    const bool umma = (w->engine == GBC_SWEEP_UMMA);
    if (umma) k_sw_prologue<true><<<gp, 256, 0, st>>>(s, U, DU);
    else k_sw_prologue<false><<<gp, 256, 0, st>>>(s, U, DU);
    GBC_CUDA(cudaGetLastError());
    if (umma) {
        const UmmaSeg gm{s.rowsq / 128, (int)(s.ldq / 128), s.qscale, nullptr, 0};
        if (int rc = launch_umma_kp(w->tmA, w, s, gm, DU, st)) return rc;
        if (w->fault_tc) {  // fault-fault block on the tensor cores, then friction alone
            float* yf = static_cast<float*>(w->yf.p);
            const UmmaSeg gf{3 * w->Nf / 128, (int)(w->Nf / 128), nullptr, yf, 3 * w->Nf};
            if (int rc = launch_umma_kp(w->tmF, w, s, gf, DU, st)) return rc;
            int gx = (s.N + 255) / 256;
            k_sw_friction<<<dim3((unsigned)gx, (unsigned)s.K), 256, 0, st>>>(s, yf, w->Nf, U, DU);
            GBC_CUDA(cudaGetLastError());
            return 0;
        }
    } else {
        const dim3 gg((unsigned)(s.rowsq / kSwRows), (unsigned)((s.K + kSwGroup - 1) / kSwGroup));
        k_sw_gemm_simt<<<gg, 256, 0, st>>>(s, DU);
        GBC_CUDA(cudaGetLastError());
    }
    if (int rc = set_smem_limit((const void*)k_sw_fault_rows, 160 * 1024)) return rc;
    const int nb = (s.nx + kFR_II - 1) / kFR_II;
    const dim3 gf((unsigned)(nb * s.nxi), (unsigned)s.K);
    k_sw_fault_rows<<<gf, kFR_II * kFR_L, fault_rows_smem_bytes(s.N, s.nx, s.nxi), st>>>(s, U, DU);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

// kernels one sweep_rhs launches: prologue, product(s), fault rows or friction
static int sweep_rhs_kernels(const gbc_sweep* w) { return (w->engine == GBC_SWEEP_UMMA && w->fault_tc) ? 4 : 3; }

static int sweep_tsit5_step(gbc_sweep* w, cudaStream_t st) {
    const long long n = w->n;
    const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 4);
    const dim3 gk((unsigned)g, (unsigned)w->K);
    Ctrl* ctrl = static_cast<Ctrl*>(w->ctrl.p);
    const SweepArgs s = w->args(ctrl, 1);
    SwK K;
    for (int r = 0; r < 7; ++r) K.k[r] = w->k[r].p;
    for (int stg = 1; stg < 7; ++stg) {
        double* dst = (stg == 6) ? w->un.p : w->y.p;
        k_sw_stage<<<gk, 256, 0, st>>>(stg, n, w->U.p, K, dst, ctrl);
        GBC_CUDA(cudaGetLastError());
        if (int rc = sweep_rhs(w, s, dst, w->k[stg].p, st)) return rc;
    }
    k_sw_error<<<dim3((unsigned)w->eb, (unsigned)w->K), 256, 0, st>>>(n, w->U.p, w->un.p, K, w->partial.p, ctrl);
    GBC_CUDA(cudaGetLastError());
    k_sw_control<<<1, kSwMaxVariants, 0, st>>>(w->K, n, w->eb, w->partial.p, ctrl, 0);
    GBC_CUDA(cudaGetLastError());
    k_sw_commit<<<gk, 256, 0, st>>>(n, w->U.p, w->un.p, w->k[0].p, w->k[6].p, ctrl);
    GBC_CUDA(cudaGetLastError());
    k_sw_clear<<<1, kSwMaxVariants, 0, st>>>(w->K, ctrl, static_cast<int*>(w->ndone.p));
    GBC_CUDA(cudaGetLastError());
    return 0;
}

static int sweep_abm_step(gbc_sweep* w, cudaStream_t st) {
    const long long n = w->n;
    const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 4);
    const dim3 gk((unsigned)g, (unsigned)w->K);
    Ctrl* ctrl = static_cast<Ctrl*>(w->ctrl.p);
    SwPhi P;
    for (int j = 0; j <= kAbmMax; ++j) P.p[j] = w->phi[j].p;
    double* yp = w->y.p;
    double* fp = w->k[1].p;
    double* sv = w->k[2].p;
    double* fn = w->k[3].p;
    k_sw_abm_coef<<<1, kSwMaxVariants, 0, st>>>(w->K, ctrl);
    GBC_CUDA(cudaGetLastError());
    k_sw_abm_predict<<<gk, 256, 0, st>>>(n, w->U.p, P, yp, sv, ctrl);
    GBC_CUDA(cudaGetLastError());
    if (int rc = sweep_rhs(w, w->args(ctrl, 1), yp, fp, st)) return rc;
    k_sw_abm_correct<<<dim3((unsigned)w->eb, (unsigned)w->K), 256, 0, st>>>(n, w->U.p, yp, fp, sv, w->un.p,
                                                                             w->partial.p, ctrl);
    GBC_CUDA(cudaGetLastError());
    k_sw_control<<<1, kSwMaxVariants, 0, st>>>(w->K, n, w->eb, w->partial.p, ctrl, 1);
    GBC_CUDA(cudaGetLastError());
    // the corrected point is evaluated only for the variants whose step was accepted
    if (int rc = sweep_rhs(w, w->args(ctrl, 2), w->un.p, fn, st)) return rc;
    k_sw_abm_commit<<<gk, 256, 0, st>>>(n, w->U.p, w->un.p, fn, P, ctrl);
    GBC_CUDA(cudaGetLastError());
    k_sw_clear<<<1, kSwMaxVariants, 0, st>>>(w->K, ctrl, static_cast<int*>(w->ndone.p));
    GBC_CUDA(cudaGetLastError());
    return 0;
}

static int sweep_alloc_integration(gbc_sweep* w, int alg) {
    const size_t kn = (size_t)w->K * w->n;
    if (int rc = w->U.alloc(kn)) return rc;
    for (int r = 0; r < 7; ++r)
        if (int rc = w->k[r].alloc(kn)) return rc;
    if (int rc = w->y.alloc(kn)) return rc;
    if (int rc = w->un.alloc(kn)) return rc;
    if (alg == GBC_ALG_VCABM5)
        for (int j = 0; j <= kAbmMax; ++j) {
            if (int rc = w->phi[j].alloc(kn)) return rc;
            GBC_CUDA(cudaMemsetAsync(w->phi[j].p, 0, sizeof(double) * kn, w->stream));
        }
    // the single model's error-norm grid: the same per-block partial sums
    w->eb = (int)std::min<long long>((w->n + 255) / 256, (long long)sm_count() * 2);
    if (w->eb < 1) w->eb = 1;
    if (int rc = w->partial.alloc((size_t)w->K * w->eb)) return rc;
    if (int rc = w->ctrl.alloc(sizeof(Ctrl) * (size_t)w->K)) return rc;
    if (!w->ctrl_host) GBC_CUDA(cudaMallocHost(&w->ctrl_host, sizeof(Ctrl) * kSwMaxVariants));
    if (!w->ndone_host) GBC_CUDA(cudaMallocHost(&w->ndone_host, sizeof(int)));
    return 0;
}

}  // namespace gbc

extern "C" {

int gbc_sweep_create(gbc_model* m, int nvariants, gbc_sweep** out) {
    if (!out) return fail(GBC_EINVAL, "null output handle");
    *out = nullptr;
    if (!m) return fail(GBC_EINVAL, "null base model");
    if (nvariants < 1 || nvariants > kSwMaxVariants)
        return fail(GBC_EINVAL, "a sweep has 1 to " + std::to_string(kSwMaxVariants) + " variants");
    if (m->ne == 0 || m->dila) return fail(GBC_EINVAL, "a sweep shares the mantle rows of a viscoelastic model");
    if (m->precision != GBC_PREC_BF16)
        return fail(GBC_EINVAL, "a sweep shares block-scaled BF16 Green's functions: set GBC_PREC_BF16 on the base model");
    if (fault_rows_smem_bytes(m->N, m->nx, m->nxi) > 160 * 1024)
        return fail(GBC_EINVAL, "fault too large for the sweep's shared-memory fault rows (N + nx*nxi floats <= 160 KB)");
    if (int rc = m->ready()) return rc;
    if (int rc = m->prepare()) return rc;
    gbc_sweep* w = new gbc_sweep();
    w->base = m;
    w->K = nvariants;
    w->Kp = nvariants <= 16 ? 16 : nvariants <= 32 ? 32 : 64;
    w->N = m->N; w->ne = m->ne; w->nx = m->nx; w->nxi = m->nxi; w->npad = m->npad; w->nlaws = m->nlaws;
    w->n = m->state_len(); w->ldq = m->ldq; w->rowsq = m->rowsq; w->Mpad = m->Mpad;
    int rc = 0;
    cudaError_t e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
    const size_t K = (size_t)w->K, N = (size_t)w->N, lne = (size_t)w->nlaws * w->ne;
    if (!rc) rc = w->a.alloc(K * N);
    if (!rc) rc = w->b.alloc(K * N);
    if (!rc) rc = w->L.alloc(K * N);
    if (!rc) rc = w->sig.alloc(K * N);
    if (!rc) rc = w->gamma.alloc(K * lne);
    if (!rc) rc = w->nexp.alloc(K * lne);
    if (!rc) rc = w->x32.alloc(sizeof(float) * (size_t)w->Kp * w->ldq);
    if (!rc) rc = w->xb.alloc(2 * 3 * (size_t)w->Kp * w->ldq);
    if (!rc) rc = w->y32.alloc(sizeof(float) * K * N);
    if (!rc) rc = w->err.alloc(sizeof(int));
    if (!rc) rc = w->ndone.alloc(sizeof(int));
    // every variant starts with the base model's properties
    std::vector<double> fp(4 * K), d0(6 * K);
    for (size_t k = 0; k < K; ++k) {
        fp[4 * k] = m->eta; fp[4 * k + 1] = m->vpl; fp[4 * k + 2] = m->f0; fp[4 * k + 3] = m->v0;
        for (int j = 0; j < 6; ++j) d0[6 * k + j] = m->deps0[j];
    }
    if (!rc) rc = upload(w->fp, fp.data(), fp.size(), w->stream);
    if (!rc) rc = upload(w->deps0, d0.data(), d0.size(), w->stream);
    for (size_t k = 0; k < K && !rc; ++k) {
        const cudaMemcpyKind dd = cudaMemcpyDeviceToDevice;
        e = cudaMemcpyAsync(w->a.p + k * N, m->a.p, sizeof(double) * N, dd, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->b.p + k * N, m->b.p, sizeof(double) * N, dd, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->L.p + k * N, m->L.p, sizeof(double) * N, dd, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->sig.p + k * N, m->sig.p, sizeof(double) * N, dd, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->gamma.p + k * lne, m->gamma.p, sizeof(double) * lne, dd, w->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w->nexp.p + k * lne, m->nexp.p, sizeof(double) * lne, dd, w->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync");
    }
    // padding columns and padded variants stay zero
    if (!rc) {
        e = cudaMemsetAsync(w->x32.p, 0, w->x32.bytes, w->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(w->xb.p, 0, w->xb.bytes, w->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(w->y32.p, 0, w->y32.bytes, w->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(w->err.p, 0, sizeof(int), w->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(w->ndone.p, 0, sizeof(int), w->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemsetAsync");
    }
    // TMA views with 128-byte swizzle: the matrix in 128-row x 64-column boxes, the split state
    // columns in 3 Kp-row x 64-column boxes (every box starts at a multiple of 64 columns = 128 B)
    if (!rc) rc = encode_tmap_2d(m->q.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, w->rowsq, w->ldq, 64, 128, true, w->tmA);
    if (!rc) rc = encode_tmap_2d(w->xb.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, 3LL * w->Kp, w->ldq, 64, 3 * w->Kp, true,
                                 w->tmB);
    if (!rc) {
        e = cudaStreamSynchronize(w->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
    }
    if (rc) {
        gbc_sweep_destroy(w);
        return rc;
    }
    *out = w;
    return 0;
}

void gbc_sweep_destroy(gbc_sweep* w) {
    if (!w) return;
    if (w->stream) cudaStreamSynchronize(w->stream);
    if (w->exec) cudaGraphExecDestroy(w->exec);
    if (w->ctrl_host) cudaFreeHost(w->ctrl_host);
    if (w->ndone_host) cudaFreeHost(w->ndone_host);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
}

long long gbc_sweep_state_len(const gbc_sweep* w) { return w ? w->n : 0; }

void* gbc_sweep_stream(gbc_sweep* w) { return w ? (void*)w->stream : nullptr; }

int gbc_sweep_set_engine(gbc_sweep* w, int engine) {
    if (!w) return fail(GBC_EINVAL, "null sweep");
    if (engine != GBC_SWEEP_SIMT && engine != GBC_SWEEP_UMMA) return fail(GBC_EINVAL, "unknown sweep engine");
    w->engine = engine;
    return 0;
}

int gbc_sweep_set_fault_product(gbc_sweep* w, int on) {
    if (!w) return fail(GBC_EINVAL, "null sweep");
    if (!on) {
        w->fault_tc = 0;
        return 0;
    }
    if (int rc = w->check_base()) return rc;
    w->Nf = ((long long)w->N + 127) / 128 * 128;
    const long long planes = w->Nf * w->Nf;
    if (int rc = w->qf.alloc(2 * 3 * (size_t)planes)) return rc;
    if (int rc = w->yf.alloc(sizeof(float) * 3 * (size_t)w->Nf * w->K)) return rc;
    cudaStream_t s = w->stream;
    GBC_CUDA(cudaMemsetAsync(w->yf.p, 0, w->yf.bytes, s));
    k_sw_fault_planes<<<sm_count() * 8, 256, 0, s>>>(w->nx, w->nxi, w->N, w->Nf,
                                                     static_cast<const float*>(w->base->st32.p),
                                                     static_cast<uint16_t*>(w->qf.p));
    GBC_CUDA(cudaGetLastError());
    count_launches(1);
    if (int rc = encode_tmap_2d(w->qf.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, 3 * w->Nf, w->Nf, 64, 128, true, w->tmF))
        return rc;
    GBC_CUDA(cudaStreamSynchronize(s));
    w->fault_tc = 1;
    return 0;
}

int gbc_sweep_set_fault_props(gbc_sweep* w, int k, const double* a, const double* b, const double* L,
                              const double* sigma, double eta, double vpl, double f0, double v0) {
    if (!w || !a || !b || !L || !sigma) return fail(GBC_EINVAL, "null argument");
    if (k < 0 || k >= w->K) return fail(GBC_EINVAL, "variant index out of range");
    if (!(f0 > 0)) return fail(GBC_EINVAL, "AssertionError: f₀ > 0");
    if (!(v0 > 0)) return fail(GBC_EINVAL, "AssertionError: v₀ > 0");
    if (!(eta > 0)) return fail(GBC_EINVAL, "AssertionError: η > 0");
    if (!(vpl > 0)) return fail(GBC_EINVAL, "AssertionError: vpl > 0");
    const size_t N = (size_t)w->N, o = (size_t)k * N;
    const double fp[4] = {eta, vpl, f0, v0};
    cudaStream_t s = w->stream;
    GBC_CUDA(cudaMemcpyAsync(w->a.p + o, a, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->b.p + o, b, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->L.p + o, L, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->sig.p + o, sigma, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->fp.p + 4 * (size_t)k, fp, sizeof(fp), cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_sweep_set_mantle_props(gbc_sweep* w, int k, const double* gamma, const double* n, const double* deps0) {
    if (!w || !gamma || !n || !deps0) return fail(GBC_EINVAL, "null argument");
    if (k < 0 || k >= w->K) return fail(GBC_EINVAL, "variant index out of range");
    const size_t lne = (size_t)w->nlaws * w->ne, o = (size_t)k * lne;
    cudaStream_t s = w->stream;
    GBC_CUDA(cudaMemcpyAsync(w->gamma.p + o, gamma, sizeof(double) * lne, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->nexp.p + o, n, sizeof(double) * lne, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->deps0.p + 6 * (size_t)k, deps0, sizeof(double) * 6, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_sweep_rhs_dev(gbc_sweep* w, const double* u, double* du) {
    if (!w || !u || !du) return fail(GBC_EINVAL, "null argument");
    if (int rc = w->check_base()) return rc;
    if (int rc = sweep_rhs(w, w->args(nullptr, 0), u, du, w->stream)) return rc;
    count_launches(sweep_rhs_kernels(w));
    return 0;
}

int gbc_sweep_rhs(gbc_sweep* w, const double* u, double* du) {
    if (!w || !u || !du) return fail(GBC_EINVAL, "null argument");
    const size_t kn = (size_t)w->K * w->n;
    if (int rc = w->U.alloc(kn)) return rc;
    if (int rc = w->DU.alloc(kn)) return rc;
    GBC_CUDA(cudaMemcpyAsync(w->U.p, u, sizeof(double) * kn, cudaMemcpyHostToDevice, w->stream));
    if (int rc = gbc_sweep_rhs_dev(w, w->U.p, w->DU.p)) return rc;
    GBC_CUDA(cudaMemcpyAsync(du, w->DU.p, sizeof(double) * kn, cudaMemcpyDeviceToHost, w->stream));
    GBC_CUDA(cudaStreamSynchronize(w->stream));
    return gbc_sweep_error_word(w) ? fail(GBC_ECUDA, "a tensor-core pipeline wait timed out") : 0;
}

int gbc_sweep_error_word(gbc_sweep* w) {
    if (!w || !w->err.p) return 0;
    int h = 0;
    if (cudaMemcpy(&h, w->err.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h;
}

int gbc_sweep_integrate_dev(gbc_sweep* w, double* u_dev, double t0, double t1, const gbc_solver_opts* o,
                            gbc_solver_stats* stats) {
    if (!w || !u_dev || !o) return fail(GBC_EINVAL, "null argument");
    if (!(o->reltol > 0) || !(o->abstol >= 0) || !(o->dt0 > 0) || !(o->dtmax > 0) || o->maxiters <= 0)
        return fail(GBC_EINVAL, "invalid solver options");
    if (o->alg != GBC_ALG_TSIT5 && o->alg != GBC_ALG_VCABM5)
        return fail(GBC_EINVAL, "unknown integrator (GBC_ALG_TSIT5 or GBC_ALG_VCABM5)");
    if (int rc = w->check_base()) return rc;
    if (int rc = sweep_alloc_integration(w, o->alg)) return rc;
    cudaStream_t s = w->stream;
    const size_t kn = (size_t)w->K * w->n;
    if (u_dev != w->U.p) GBC_CUDA(cudaMemcpyAsync(w->U.p, u_dev, sizeof(double) * kn, cudaMemcpyDeviceToDevice, s));
    const Ctrl h0 = ctrl_start(o->alg, t0, t1, o->reltol, o->abstol, o->dt0, o->dtmax, o->dtmin, o->maxiters);
    for (int k = 0; k < w->K; ++k) {
        w->ctrl_host[k] = h0;
        w->ctrl_host[k].th_lo = w->N;
        w->ctrl_host[k].th_hi = 2LL * w->N;
    }
    *w->ndone_host = h0.done ? w->K : 0;
    GBC_CUDA(cudaMemcpyAsync(w->ctrl.p, w->ctrl_host, sizeof(Ctrl) * w->K, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(w->ndone.p, w->ndone_host, sizeof(int), cudaMemcpyHostToDevice, s));
    // FSAL seed k0 = f(u0) (Tsit5) or Phi_0 = f(u0) (VCABM5) for every variant
    double* seed = (o->alg == GBC_ALG_VCABM5) ? w->phi[0].p : w->k[0].p;
    if (int rc = sweep_rhs(w, w->args(nullptr, 0), w->U.p, seed, s)) return rc;
    const int group = (o->alg == GBC_ALG_VCABM5) ? 16 : 8;
    if (w->exec) {
        cudaGraphExecDestroy(w->exec);
        w->exec = nullptr;
    }
    cudaGraph_t graph;
    GBC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int i = 0; i < group && rc == 0; ++i) rc = (o->alg == GBC_ALG_VCABM5) ? sweep_abm_step(w, s) : sweep_tsit5_step(w, s);
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (rc) return rc;
    GBC_CUDA(ce);
    GBC_CUDA(cudaGraphInstantiate(&w->exec, graph, 0));
    cudaGraphDestroy(graph);
    w->steps_per_launch = group;
    w->graph_launches = 0;
    while (*w->ndone_host < w->K) {
        GBC_CUDA(cudaGraphLaunch(w->exec, s));
        ++w->graph_launches;
        GBC_CUDA(cudaMemcpyAsync(w->ndone_host, w->ndone.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        if (gbc_sweep_error_word(w)) return fail(GBC_ECUDA, "a tensor-core pipeline wait timed out");
    }
    GBC_CUDA(cudaMemcpyAsync(w->ctrl_host, w->ctrl.p, sizeof(Ctrl) * w->K, cudaMemcpyDeviceToHost, s));
    if (u_dev != w->U.p) GBC_CUDA(cudaMemcpyAsync(u_dev, w->U.p, sizeof(double) * kn, cudaMemcpyDeviceToDevice, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    const long long rk = sweep_rhs_kernels(w);
    const long long per_step = (o->alg == GBC_ALG_VCABM5) ? 6 + 2 * rk : 10 + 6 * rk;
    count_launches(rk + w->graph_launches * w->steps_per_launch * per_step);
    int status = 0;
    for (int k = 0; k < w->K; ++k) {
        const Ctrl& c = w->ctrl_host[k];
        if (stats) {
            stats[k].naccept = c.naccept;
            stats[k].nreject = c.nreject;
            stats[k].nrhs = c.nrhs + 1;
            stats[k].t = c.t;
            stats[k].dt = c.dt;
            stats[k].status = c.status;
        }
        if (c.status != 0) status = GBC_ESOLVER;
    }
    if (status) return fail(GBC_ESOLVER, "a variant stopped early (dt < dtmin, maxiters or non-finite state)");
    return 0;
}

int gbc_sweep_integrate(gbc_sweep* w, double* u, double t0, double t1, const gbc_solver_opts* o,
                        gbc_solver_stats* stats) {
    if (!w || !u) return fail(GBC_EINVAL, "null argument");
    const size_t kn = (size_t)w->K * w->n;
    if (int rc = w->U.alloc(kn)) return rc;
    GBC_CUDA(cudaMemcpyAsync(w->U.p, u, sizeof(double) * kn, cudaMemcpyHostToDevice, w->stream));
    int rc = gbc_sweep_integrate_dev(w, w->U.p, t0, t1, o, stats);
    if (rc != 0 && rc != GBC_ESOLVER) return rc;
    GBC_CUDA(cudaMemcpyAsync(u, w->U.p, sizeof(double) * kn, cudaMemcpyDeviceToHost, w->stream));
    GBC_CUDA(cudaStreamSynchronize(w->stream));
    return rc;
}

}  // extern "C"
